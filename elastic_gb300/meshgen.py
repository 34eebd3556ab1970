"""Structured meshes in the reference's input layout.

Every generator returns a :class:`Mesh` whose arrays follow the reference's
Fortran conventions (lmn-labest/Elastic, mef/src/Rdata.f): 1-based node and
material numbers, ``ix(nen+1, numel)`` with the material number in the last
row, ``x(ndm, nnode)``, ``id(ndf, nnode)`` with 1 = constrained, ``e(prop,
numat)`` with E in e(1), nu in e(2), thickness in e(3), ``ie(numat)`` the element
type per material (Elmlib.f:43-144: 2/3 TRIA3 plane strain/stress, 4/5 QUAD4
plane strain/stress, 6 TETRA4, 7 HEXA8) and ``f(ndf, nnode)`` nodal forces.
The numpy arrays are C-ordered with the Fortran leading dimension last, so
``mesh.ix[el, :]`` is column ``el`` of the Fortran array and the raw buffer is
byte-identical to the Fortran one.

Node numbering is x-fastest, as in the reference's example decks
(input/quad/exemplo1_apostila_el.dat: node n at (i, j) = n-1 = j*(nx+1)+i,
element (n, n+1, n+nx+2, n+nx+1)).  HEXA8 local node order follows
sfhexa8_m (Elmlib.f:1177-1184): (+,+,+), (-,+,+), (-,-,+), (+,-,+) and then the
same four at t = -1.  TETRA4 meshes split each hexahedron into six tetrahedra
with the positively oriented split of Pdata.f:503-513.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

PROP = 15  # include/termprop.fi: prop = 15

# reference element types (Elmlib.f:43-144)
TRIA3_STRAIN, TRIA3_STRESS, QUAD4_STRAIN, QUAD4_STRESS, TETRA4, HEXA8 = 2, 3, 4, 5, 6, 7

NEN_OF_TYPE = {2: 3, 3: 3, 4: 4, 5: 4, 6: 4, 7: 8}
NDM_OF_TYPE = {2: 2, 3: 2, 4: 2, 5: 2, 6: 3, 7: 3}


@dataclass
class Mesh:
    """One finite-element model in the reference's array layout."""

    ndm: int
    ndf: int
    nen: int
    x: np.ndarray          # (nnode, ndm) float64
    ix: np.ndarray         # (numel, nen+1) int32, 1-based, last = material
    ie: np.ndarray         # (numat,) int32 element type per material
    e: np.ndarray          # (numat, PROP) float64
    id: np.ndarray         # (nnode, ndf) int32, 1 = constrained
    f: np.ndarray          # (nnode, ndf) float64 nodal forces
    eload: np.ndarray | None = None    # (numel, 7) int32 side loads (2-D)
    loadvec: np.ndarray | None = None  # (numload, 2) float64 type-40 vectors
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def nnode(self) -> int:
        return int(self.x.shape[0])

    @property
    def numel(self) -> int:
        return int(self.ix.shape[0])

    @property
    def numat(self) -> int:
        return int(self.ie.shape[0])

    @property
    def nenv(self) -> int:
        return self.nen

    def free_dofs(self) -> int:
        return int((self.id == 0).sum())


def _materials(types, E, nu, thick=None):
    types = np.atleast_1d(np.asarray(types, np.int32))
    numat = types.shape[0]
    e = np.zeros((numat, PROP), np.float64)
    e[:, 0] = E
    e[:, 1] = nu
    if thick is not None:
        e[:, 2] = thick
    return types, e


def box2d(nx, ny, lx=1.0, ly=1.0, etype=QUAD4_STRESS, E=1.0, nu=0.3,
          thick=1.0, clamp="left", traction=None, traction_side="right",
          nodal_force=None, name=""):
    """nx x ny QUAD4 (or TRIA3, two per cell) mesh of [0,lx] x [0,ly].

    ``clamp`` names the edge whose nodes are fixed in both dofs.
    ``traction`` = (tx, ty) applies a uniform type-40 edge load on
    ``traction_side`` through ``eload``/``loadvec`` (the elmtloads path,
    Elmlib02.f:856-910).  ``nodal_force`` = (fx, fy) puts a nodal force on
    every node of ``traction_side`` instead.
    """
    X = nx + 1
    ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    x = np.stack([(ii.ravel() * lx) / nx, (jj.ravel() * ly) / ny], axis=1)
    nid = lambda i, j: j * X + i + 1
    ci, cj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    ci, cj = ci.ravel(), cj.ravel()
    n1 = nid(ci, cj)
    n2 = nid(ci + 1, cj)
    n3 = nid(ci + 1, cj + 1)
    n4 = nid(ci, cj + 1)
    tri = etype in (TRIA3_STRAIN, TRIA3_STRESS)
    if not tri:
        conn = np.stack([n1, n2, n3, n4], axis=1)
        nen = 4
    else:
        # two triangles per cell, both counter-clockwise
        t1 = np.stack([n1, n2, n3], axis=1)
        t2 = np.stack([n1, n3, n4], axis=1)
        conn = np.empty((2 * t1.shape[0], 3), np.int64)
        conn[0::2] = t1
        conn[1::2] = t2
        nen = 3
    numel = conn.shape[0]
    ix = np.empty((numel, nen + 1), np.int32)
    ix[:, :nen] = conn
    ix[:, nen] = 1
    ie, e = _materials([etype], E, nu, thick)
    nnode = x.shape[0]
    idm = np.zeros((nnode, 2), np.int32)
    edge = {
        "left": nid(np.zeros(ny + 1, int), np.arange(ny + 1)),
        "right": nid(np.full(ny + 1, nx), np.arange(ny + 1)),
        "bottom": nid(np.arange(nx + 1), np.zeros(nx + 1, int)),
        "top": nid(np.arange(nx + 1), np.full(nx + 1, ny)),
    }
    idm[edge[clamp] - 1, :] = 1
    f = np.zeros((nnode, 2), np.float64)
    eload = loadvec = None
    if traction is not None:
        eload = np.zeros((numel, 7), np.int32)
        loadvec = np.asarray([traction], np.float64)
        if not tri:
            # quad sides (Elmlib02.f quad_side_node4): 1:(1,2) 2:(2,3) 3:(3,4) 4:(4,1)
            side = {"right": 2, "top": 3, "bottom": 1, "left": 4}[traction_side]
            sel = {"right": ci == nx - 1, "top": cj == ny - 1,
                   "bottom": cj == 0, "left": ci == 0}[traction_side]
            eload[np.nonzero(sel)[0], side - 1] = 1
        else:
            # t1=(n1,n2,n3): side 1 bottom, side 2 right; t2=(n1,n3,n4): side 2 top, side 3 left
            sel_c = {"right": ci == nx - 1, "top": cj == ny - 1,
                     "bottom": cj == 0, "left": ci == 0}[traction_side]
            cells = np.nonzero(sel_c)[0]
            if traction_side == "right":
                eload[2 * cells, 1] = 1
            elif traction_side == "bottom":
                eload[2 * cells, 0] = 1
            elif traction_side == "top":
                eload[2 * cells + 1, 1] = 1
            else:
                eload[2 * cells + 1, 2] = 1
    if nodal_force is not None:
        f[edge[traction_side] - 1, :] = nodal_force
    return Mesh(ndm=2, ndf=2, nen=nen, x=x, ix=ix, ie=ie, e=e, id=idm, f=f,
                eload=eload, loadvec=loadvec, name=name or f"box2d_{nx}x{ny}")


def cantilever_quad4_64x16():
    """Plane-stress QUAD4 cantilever, 64x16 on [0,4]x[0,1], E=210e3, nu=0.3,
    thickness 1, left edge clamped, uniform traction (0,-1) on the right edge."""
    return box2d(64, 16, 4.0, 1.0, QUAD4_STRESS, 210e3, 0.3, 1.0, "left",
                 traction=(0.0, -1.0), traction_side="right",
                 name="quad4_cantilever_64x16")


def square_quad4_100(plane_stress=False):
    """100x100 QUAD4 on [0,1]^2, E=1, nu=0.3, left edge clamped, traction
    (0,-1) on the top edge: the model of input/quad/exemplo1_apostila_el.dat."""
    t = QUAD4_STRESS if plane_stress else QUAD4_STRAIN
    return box2d(100, 100, 1.0, 1.0, t, 1.0, 0.3, 0.0, "left",
                 traction=(0.0, -1.0), traction_side="top",
                 name="quad4_square_100")


# HEXA8 local node offsets (i, j, k) in sfhexa8_m order (Elmlib.f:1177-1184)
HEX_LOCAL = np.array([(1, 1, 1), (0, 1, 1), (0, 0, 1), (1, 0, 1),
                      (1, 1, 0), (0, 1, 0), (0, 0, 0), (1, 0, 0)], np.int64)
# positively oriented 6-tet split of a hexahedron (Pdata.f:503-513), local 1-based
TET_SPLIT = np.array([(2, 5, 6, 7), (2, 5, 7, 3), (2, 5, 3, 1),
                      (3, 5, 7, 8), (3, 1, 8, 4), (3, 1, 5, 8)], np.int64)


def _box3d_nodes(nx, ny, nz, lx, ly, lz):
    ii, jj, kk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1),
                             np.arange(nz + 1), indexing="ij")
    # x-fastest numbering: n-1 = (k*(ny+1) + j)*(nx+1) + i
    order = np.lexsort((ii.ravel(), jj.ravel(), kk.ravel()))
    i, j, k = ii.ravel()[order], jj.ravel()[order], kk.ravel()[order]
    x = np.stack([(i * lx) / nx, (j * ly) / ny, (k * lz) / nz], axis=1)
    return x, (i, j, k)


def _hex_conn(nx, ny, nz):
    X, Y = nx + 1, ny + 1
    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                             indexing="ij")
    order = np.lexsort((ci.ravel(), cj.ravel(), ck.ravel()))
    ci, cj, ck = ci.ravel()[order], cj.ravel()[order], ck.ravel()[order]
    conn = np.empty((ci.shape[0], 8), np.int64)
    for a, (di, dj, dk) in enumerate(HEX_LOCAL):
        conn[:, a] = ((ck + dk) * Y + (cj + dj)) * X + (ci + di) + 1
    return conn, (ci, cj, ck)


def _top_pressure_forces(nx, ny, nz, lx, ly, p, ijk):
    """Consistent nodal forces of a uniform pressure p on the z = lz face:
    -p * hx * hy * {1/4 corner, 1/2 edge, 1 interior} in z."""
    i, j, k = ijk
    nnode = i.shape[0]
    f = np.zeros((nnode, 3), np.float64)
    top = k == nz
    wx = np.where((i == 0) | (i == nx), 0.5, 1.0)
    wy = np.where((j == 0) | (j == ny), 0.5, 1.0)
    f[top, 2] = -p * (lx / nx) * (ly / ny) * (wx * wy)[top]
    return f


def _jitter_interior(x, ijk, nx, ny, nz, lx, ly, lz, jitter, rng):
    i, j, k = ijk
    inner = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
    h = np.array([lx / nx, ly / ny, lz / nz])
    x[inner] += rng.uniform(-jitter, jitter, size=(int(inner.sum()), 3)) * h


def box_hexa8(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, E=1.0, nu=0.3,
              pressure=1.0, jitter=0.0, seed=20261203, name=""):
    """HEXA8 box, z = 0 face fixed, uniform pressure on z = lz as nodal forces.
    ``jitter`` moves interior nodes by U[-jitter*h, jitter*h] per axis."""
    x, ijk = _box3d_nodes(nx, ny, nz, lx, ly, lz)
    if jitter > 0.0:
        _jitter_interior(x, ijk, nx, ny, nz, lx, ly, lz, jitter, np.random.default_rng(seed))
    conn, _ = _hex_conn(nx, ny, nz)
    numel = conn.shape[0]
    ix = np.empty((numel, 9), np.int32)
    ix[:, :8] = conn
    ix[:, 8] = 1
    ie, e = _materials([HEXA8], E, nu)
    idm = np.zeros((x.shape[0], 3), np.int32)
    idm[ijk[2] == 0, :] = 1
    f = _top_pressure_forces(nx, ny, nz, lx, ly, pressure, ijk)
    return Mesh(ndm=3, ndf=3, nen=8, x=x, ix=ix, ie=ie, e=e, id=idm, f=f,
                name=name or f"hexa8_{nx}x{ny}x{nz}")


def cube_hexa8_64():
    """HEXA8 cube 64^3 on [0,1]^3, E=1, nu=0.3, z=0 fixed, pressure 1 on z=1."""
    return box_hexa8(64, 64, 64, name="hexa8_cube_64")


def box_tetra4(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, E=1.0, nu=0.3,
               pressure=1.0, jitter=0.0, seed=20261203, lognormal_E=False,
               nu_range=None, name=""):
    """TETRA4 box: each hexahedron split into six tetrahedra (Pdata.f:503-513).

    ``jitter`` moves interior nodes by U[-jitter*h, jitter*h] per axis from
    ``seed``; ``lognormal_E`` gives one material per element with
    E = exp(N(0,1)) and nu = U[nu_range] (both from the same seed).
    """
    rng = np.random.default_rng(seed)
    x, ijk = _box3d_nodes(nx, ny, nz, lx, ly, lz)
    i, j, k = ijk
    if jitter > 0.0:
        _jitter_interior(x, ijk, nx, ny, nz, lx, ly, lz, jitter, rng)
    hconn, _ = _hex_conn(nx, ny, nz)
    nh = hconn.shape[0]
    conn = hconn[:, TET_SPLIT - 1].reshape(nh * 6, 4)
    numel = conn.shape[0]
    if jitter > 0.0:
        # A few tetrahedra of the 6-tet split invert under +-0.2h jitter; the
        # interior nodes of any element with det < 1% of an undistorted one
        # get a fresh U[-jitter*h, jitter*h] draw until every element is valid
        # (the element routine stops on det <= 1e-14, Elmlib.f:2664-2667).
        h = np.array([lx / nx, ly / ny, lz / nz])
        x0, _ = _box3d_nodes(nx, ny, nz, lx, ly, lz)
        inner = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
        for _round in range(200):
            xs = x[conn - 1]
            det = np.einsum("ij,ij->i", xs[:, 0] - xs[:, 3],
                            np.cross(xs[:, 1] - xs[:, 3], xs[:, 2] - xs[:, 3]))
            bad = det < 0.01 * h.prod()
            if not bad.any():
                break
            nodes = np.unique(conn[bad] - 1)
            nodes = nodes[inner[nodes]]
            x[nodes] = x0[nodes] + rng.uniform(-jitter, jitter, size=(nodes.shape[0], 3)) * h
        else:
            raise RuntimeError("could not draw a valid jittered tetra mesh")
    ix = np.empty((numel, 5), np.int32)
    ix[:, :4] = conn
    if lognormal_E:
        lo, hi = nu_range if nu_range is not None else (0.25, 0.45)
        Ev = np.exp(rng.standard_normal(numel))
        nuv = rng.uniform(lo, hi, numel)
        ie, e = _materials(np.full(numel, TETRA4), Ev, nuv)
        ix[:, 4] = np.arange(1, numel + 1)
    else:
        ie, e = _materials([TETRA4], E, nu)
        ix[:, 4] = 1
    idm = np.zeros((x.shape[0], 3), np.int32)
    idm[k == 0, :] = 1
    f = _top_pressure_forces(nx, ny, nz, lx, ly, pressure, ijk)
    return Mesh(ndm=3, ndf=3, nen=4, x=x, ix=ix, ie=ie, e=e, id=idm, f=f,
                name=name or f"tetra4_{nx}x{ny}x{nz}")


def cube_tetra4_48_mixed():
    """TETRA4 from a 48^3 cube (6 tets per hex), interior nodes jittered by
    U[-0.2h, 0.2h], per-element E = lognormal(0,1), nu = U[0.25, 0.45]."""
    return box_tetra4(48, 48, 48, jitter=0.2, lognormal_E=True,
                      nu_range=(0.25, 0.45), name="tetra4_cube_48_mixed")


def plate_hexa8_96(nrhs=16, seed=20261203):
    """HEXA8 plate 96x96x48 elements (unit spacing), bottom fixed, and nrhs
    load cases of N(0,1) nodal forces on the top-face nodes (seed per case).
    Returns (mesh, F) with F of shape (nrhs, nnode, 3)."""
    m = box_hexa8(96, 96, 48, 96.0, 96.0, 48.0, pressure=0.0,
                  name="hexa8_plate_96x96x48")
    top = np.nonzero(m.x[:, 2] == 48.0)[0]
    F = np.zeros((nrhs, m.nnode, 3))
    for c in range(nrhs):
        r = np.random.default_rng(seed + c)
        F[c, top, :] = r.standard_normal((top.shape[0], 3))
    return m, F


def element_dets(mesh: Mesh) -> np.ndarray:
    """Volume-like determinant per element for TETRA4 (jtetra4 convention,
    Elmlib.f:2636-2713): det of rows (x1-x4, x2-x4, x3-x4)."""
    assert mesh.nen == 4 and mesh.ndm == 3
    xs = mesh.x[mesh.ix[:, :4] - 1]
    a = xs[:, 0] - xs[:, 3]
    b = xs[:, 1] - xs[:, 3]
    c = xs[:, 2] - xs[:, 3]
    return np.einsum("ij,ij->i", a, np.cross(b, c))


def serving_request(rng, dof_min=2e3, dof_max=2e6, max_rhs=8):
    """One request of the served stream: a structured box mesh with element
    type uniform over {TRIA3, QUAD4, TETRA4, HEXA8} (plane stress in 2-D),
    about log-uniform [dof_min, dof_max] dofs, E ~ U[0.5, 2], nu ~ U[0.2, 0.45],
    one face fixed (whole nodes) and 1..max_rhs load cases of N(0,1) nodal
    forces on the opposite face.  Returns (mesh, F) with F (nrhs, nnode, ndf)."""
    etype = int(rng.choice([TRIA3_STRESS, QUAD4_STRESS, TETRA4, HEXA8]))
    dof = float(np.exp(rng.uniform(np.log(dof_min), np.log(dof_max))))
    E = float(rng.uniform(0.5, 2.0))
    nu = float(rng.uniform(0.2, 0.45))
    nrhs = int(rng.integers(1, max_rhs + 1))
    if NDM_OF_TYPE[etype] == 2:
        # (nx+1)(ny+1) nodes, 2 dofs each, nx = 2 ny
        ny = max(2, int(round(np.sqrt(dof / 4.0))))
        nx = 2 * ny
        m = box2d(nx, ny, 2.0, 1.0, etype=etype, E=E, nu=nu, clamp="left")
        far = np.isclose(m.x[:, 0], 2.0)
    else:
        n = max(2, int(round((dof / 3.0) ** (1.0 / 3.0))) - 1)
        if etype == HEXA8:
            m = box_hexa8(n, n, n, E=E, nu=nu, pressure=0.0)
        else:
            m = box_tetra4(n, n, n, E=E, nu=nu, pressure=0.0)
        far = np.isclose(m.x[:, 2], 1.0)
    F = np.zeros((nrhs, m.nnode, m.ndf))
    for k in range(nrhs):
        F[k][far] = rng.standard_normal((int(far.sum()), m.ndf))
    m.f = F[0].copy()
    return m, F
