"""The device path against known answers that do not come from the oracle.

  * One-element meshes assembled on the GPU against the exact element
    matrices of tests/golden/pins.json (constant-strain closed forms of
    TRIA3 / TETRA4, exact integrals over a rectangular QUAD4 and a box HEXA8;
    see tests/golden/make_pins.py): the CSRC matrix, expanded to the
    element's dof order, within 1e-14 of the largest entry.
  * Patch test of the assembled and solved system: on distorted meshes of
    every element type, one homogeneous material (a linear field is the
    solution only when the stress it gives is the same in every element),
    every boundary node prescribed to a linear
    displacement field u(x) = a + G x and no load, the load step, assembly,
    PCG solve and update on the device reproduce the linear field at the
    interior nodes -- the finite-element solution of a linear field is that
    field -- within 1e-12 of its largest component.
"""
import json
import os

import numpy as np
import pytest

import elastic_gb300 as E
from elastic_gb300 import meshgen as M
from helpers import full_matrix

pytestmark = pytest.mark.gpu

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "pins.json")))


def one_element(p):
    xl = np.array(p["xl"], dtype=np.float64)
    n, ndm = xl.shape
    e = np.zeros((1, M.PROP))
    e[0, :3] = (p["E"], p["nu"], p["thick"])
    ix = np.array([list(range(1, n + 1)) + [1]], dtype=np.int32)
    return M.Mesh(ndm=ndm, ndf=ndm, nen=n, x=xl.copy(), ix=ix,
                  ie=np.array([p["iel"]], np.int32), e=e, id=np.zeros((n, ndm), np.int32),
                  f=np.zeros((n, ndm)), name="one")


@pytest.mark.parametrize("name", sorted(PINS["elements"]))
def test_one_element_assembly_closed_form(gpu_ctx, name):
    p = PINS["elements"][name]
    m = one_element(p)
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    st = gpu_ctx.structure()
    _, ad, al = gpu_ctx.assemble(None, None, want_matrix=True)
    K = full_matrix(st.ia, st.ja, ad, al).toarray()
    eq = st.id.reshape(-1) - 1  # equation of each (node, dof), node-major
    Kn = K[np.ix_(eq, eq)]
    want = np.array(p["K"])
    assert np.abs(Kn - want).max() <= 1e-14 * np.abs(want).max()


def _jitter2d(m, nx, ny, lx, ly, amount, seed):
    """Moves the interior nodes of a structured 2-D mesh by U[-a h, a h]."""
    rng = np.random.default_rng(seed)
    h = np.array([lx / nx, ly / ny])
    inner = ((m.x[:, 0] > 1e-12) & (m.x[:, 0] < lx - 1e-12) &
             (m.x[:, 1] > 1e-12) & (m.x[:, 1] < ly - 1e-12))
    m.x[inner] += rng.uniform(-amount, amount, (int(inner.sum()), 2)) * h
    return m


PATCH_MESHES = {
    "tria3_strain": lambda: _jitter2d(M.box2d(6, 5, 1.5, 1.0, etype=M.TRIA3_STRAIN, E=3.0,
                                              nu=0.25), 6, 5, 1.5, 1.0, 0.2, 1),
    "tria3_stress": lambda: _jitter2d(M.box2d(6, 5, 1.5, 1.0, etype=M.TRIA3_STRESS, E=3.0,
                                              nu=0.35, thick=2.0), 6, 5, 1.5, 1.0, 0.2, 2),
    "quad4_strain": lambda: _jitter2d(M.box2d(6, 5, 1.5, 1.0, etype=M.QUAD4_STRAIN),
                                      6, 5, 1.5, 1.0, 0.2, 3),
    "quad4_stress": lambda: _jitter2d(M.box2d(6, 5, 1.5, 1.0, etype=M.QUAD4_STRESS,
                                              thick=0.5), 6, 5, 1.5, 1.0, 0.2, 4),
    "tetra4": lambda: M.box_tetra4(4, 4, 3, jitter=0.2, seed=5),
    "hexa8": lambda: M.box_hexa8(4, 4, 3, jitter=0.2, seed=6),
}


@pytest.mark.parametrize("name", sorted(PATCH_MESHES))
def test_patch_linear_field_solved_exactly(gpu_ctx, name):
    m = PATCH_MESHES[name]()
    d = m.ndm
    rng = np.random.default_rng(17)
    a, G = rng.standard_normal(d), rng.standard_normal((d, d))
    u_lin = a + m.x @ G.T
    lo, hi = m.x.min(axis=0), m.x.max(axis=0)
    boundary = np.any(np.isclose(m.x, lo) | np.isclose(m.x, hi), axis=1)
    m.id[:] = 0
    m.id[boundary, :] = 1
    f = np.where(boundary[:, None], u_lin, 0.0)  # prescribed u; no load inside
    m.f = f
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    gpu_ctx.set_loads(f)
    gpu_ctx.assemble_resident()
    info = gpu_ctx.solve_resident(tol=1e-14, maxit=20000)
    assert info["status"] == 0
    gpu_ctx.update_resident()
    u, _ = gpu_ctx.state()
    assert np.abs(u - u_lin).max() <= 1e-12 * np.abs(u_lin).max()
