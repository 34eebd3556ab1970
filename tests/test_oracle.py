"""The CPU oracle pinned against the reference: its known answer, its own
decks (golden.json, made by tests/golden/make_golden.py from the reference's
input files) and the mathematical self-checks of the element and solver
routines.  CPU only."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle as O
from elastic_gb300 import meshgen as M

GOLD = os.path.join(os.path.dirname(__file__), "golden")
with open(os.path.join(GOLD, "golden.json")) as fh:
    GOLDEN = json.load(fh)["decks"]


def full_matrix(s, ad, al):
    """K = D + L + L^T as a scipy CSR matrix from CSRC arrays (1-based)."""
    n = s.neq
    rows = np.repeat(np.arange(n), np.diff(s.ia))
    cols = s.ja - 1
    L = sp.csr_matrix((al, (rows, cols)), shape=(n, n))
    return (L + L.T + sp.diags(ad)).tocsr()


# --------------------------------------------------------------- known answer
def test_quad_energy_norm_known_answer():
    """input/quad/exemplo1_apostila_el.dat:3 states sqrt(uKu) = 1.379745 for
    the exact solution; the 100x100 QUAD4 discretisation must approach it."""
    m = M.square_quad4_100()
    u, info, s, ad, al = O.solvm(m, tol=1e-11)
    e = np.sqrt(info["xkx"])
    assert abs(e - 1.379745) / 1.379745 < 1e-3
    assert e < 1.379745  # displacement FE is stiffer than the exact solution
    g = GOLDEN["quad_el"]
    assert s.neq == g["neq"] and s.nad == g["nad"] and info["iters"] == g["iters"]
    assert abs(e - g["sqrt_xkx"]) <= 1e-12 * e


def test_generator_reproduces_the_quad_deck():
    for k in ("quad_el", "quad_el_ept", "quad_nf", "quad_nl"):
        assert GOLDEN[k]["generator_matches_deck_geometry"], k


@pytest.mark.parametrize("key", ["quad_el", "quad_el_ept"])
def test_quad_decks_golden(key):
    m = M.square_quad4_100(plane_stress=(key == "quad_el_ept"))
    u, info, s, ad, al = O.solvm(m, tol=1e-11)
    g = GOLDEN[key]
    assert info["iters"] == g["iters"]
    np.testing.assert_allclose(info["xkx"], g["xkx"], rtol=1e-12)
    np.testing.assert_allclose(ad.sum(), g["ad_sum"], rtol=1e-13)


@pytest.mark.parametrize("key", ["hexa_nf", "tetra_nf"])
def test_3d_decks_golden(key):
    import sys
    sys.path.insert(0, GOLD)
    from make_golden import load_deck_mesh, sha
    m = load_deck_mesh(key)
    u, info, s, ad, al = O.solvm(m, tol=1e-11)
    g = GOLDEN[key]
    assert (s.neq, s.nad) == (g["neq"], g["nad"])
    assert sha(s.perm) == g["perm_sha"] and sha(s.ia) == g["ia_sha"] and sha(s.ja) == g["ja_sha"]
    assert info["iters"] == g["iters"]
    np.testing.assert_allclose(info["xkx"], g["xkx"], rtol=1e-12)


def test_hexa_and_tetra_decks_agree_on_a_uniform_stress_state():
    """caso_a is a column under uniform load with roller sides: the exact
    solution is linear, so HEXA8 and TETRA4 give the same energy."""
    a, b = GOLDEN["hexa_nf"]["xkx"], GOLDEN["tetra_nf"]["xkx"]
    assert abs(a - b) <= 1e-11 * a


# --------------------------------------------------------------- elements
def _rand_element(iel, rng):
    if iel in (2, 3):
        xl = np.array([[0.0, 0.0], [1.0, 0.1], [0.2, 0.9]]) + rng.uniform(-0.05, 0.05, (3, 2))
    elif iel in (4, 5):
        xl = np.array([[1.0, 1.0], [0.0, 1.0], [0.0, 0.0], [1.0, 0.0]]) + rng.uniform(-0.1, 0.1, (4, 2))
    elif iel == 6:
        # positively oriented for jtetra4: det(x1-x4, x2-x4, x3-x4) > 0
        xl = np.array([[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0], [0, 0, 0]]) + rng.uniform(-0.05, 0.05, (4, 3))
    else:
        xl = M.HEX_LOCAL.astype(float) + rng.uniform(-0.1, 0.1, (8, 3))
    return xl


def _rigid_modes(xl):
    n, d = xl.shape
    if d == 2:
        modes = [np.tile([1.0, 0.0], n), np.tile([0.0, 1.0], n),
                 np.stack([-xl[:, 1], xl[:, 0]], 1).ravel()]
    else:
        modes = [np.tile(e, n) for e in np.eye(3)]
        for a, b in ((0, 1), (1, 2), (2, 0)):
            r = np.zeros_like(xl)
            r[:, a] = -xl[:, b]
            r[:, b] = xl[:, a]
            modes.append(r.ravel())
    return np.array(modes)


@pytest.mark.parametrize("iel", [2, 3, 4, 5, 6, 7])
def test_element_stiffness_symmetric_psd_with_rigid_null_space(iel):
    rng = np.random.default_rng(iel)
    xl = _rand_element(iel, rng)
    s = O.element_stiffness(iel, [2.5, 0.3, 1.0], xl)
    scale = np.abs(s).max()
    assert np.abs(s - s.T).max() <= 1e-13 * scale
    R = _rigid_modes(xl)
    assert np.abs(s @ R.T).max() <= 1e-12 * scale
    w = np.linalg.eigvalsh(0.5 * (s + s.T))
    nz = 3 if iel <= 5 else 6
    assert np.all(np.abs(w[:nz]) <= 1e-11 * w[-1])
    assert np.all(w[nz:] > 1e-8 * w[-1])


def test_element_bad_determinant_is_reported():
    xl = np.array([[0, 0, 0], [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]])  # negative orientation
    with pytest.raises(O.OracleError):
        O.element_stiffness(6, [1.0, 0.3], xl)


def _patch_mesh(kind):
    if kind == "hexa8":
        return M.box_hexa8(3, 3, 3, jitter=0.25, seed=7)
    if kind == "tetra4":
        return M.box_tetra4(3, 3, 3, jitter=0.2, seed=7)
    return None


@pytest.mark.parametrize("kind", ["hexa8", "tetra4"])
def test_constant_strain_patch_test(kind):
    """Prescribe u = A x + c on every boundary node of a distorted mesh: the
    interior nodes must reproduce the linear field."""
    m = _patch_mesh(kind)
    A = np.array([[1e-3, 2e-4, -3e-4], [5e-4, -2e-3, 1e-4], [0.0, 3e-4, 1.5e-3]])
    c = np.array([1e-3, -2e-3, 5e-4])
    ulin = m.x @ A.T + c
    bnd = np.any((m.x <= 1e-12) | (m.x >= 1 - 1e-12), axis=1)
    m.id[:] = 0
    m.id[bnd] = 1
    m.f[:] = 0.0
    m.f[bnd] = ulin[bnd]
    u, info, s, ad, al = O.solvm(m, tol=1e-14, maxit=5000)
    np.testing.assert_allclose(u, ulin, atol=1e-12)


# --------------------------------------------------------------- assembly and solvers
def test_assembled_csrc_equals_dense_element_sum():
    m = M.box_hexa8(2, 2, 2, jitter=0.2)
    s = O.structure(m)
    ad, al, _ = O.assemble(m, s)
    K = full_matrix(s, ad, al).toarray()
    D = np.zeros_like(K)
    for el in range(m.numel):
        nodes = m.ix[el, :8] - 1
        ke = O.element_stiffness(7, m.e[0, :3], m.x[nodes])
        eqs = s.id[nodes].ravel() - 1
        for a, ea in enumerate(eqs):
            for b, eb in enumerate(eqs):
                if ea >= 0 and eb >= 0:
                    D[ea, eb] += ke[a, b] if ea >= eb else 0.0
    D = np.tril(D) + np.tril(D, -1).T
    assert np.abs(K - D).max() <= 1e-13 * np.abs(D).max()


def relabel_nodes(m, seed):
    """The same mesh with its nodes numbered in a random order."""
    rng = np.random.default_rng(seed)
    newnum = rng.permutation(m.nnode)          # old node i -> new node newnum[i]
    inv = np.argsort(newnum)
    m2 = M.Mesh(ndm=m.ndm, ndf=m.ndf, nen=m.nen, x=m.x[inv].copy(), ix=m.ix.copy(), ie=m.ie,
                e=m.e, id=m.id[inv].copy(), f=m.f[inv].copy(), name=m.name + "_relabelled")
    m2.ix[:, :m.nen] = newnum[m.ix[:, :m.nen] - 1] + 1
    return m2


def test_rcm_reduces_bandwidth_of_a_scrambled_numbering():
    m = relabel_nodes(M.box_hexa8(6, 5, 4), 11)
    bw = []
    for reorder in (False, True):
        s = O.structure(m, reorder)
        rows = np.repeat(np.arange(s.neq), np.diff(s.ia))
        bw.append(int((rows - (s.ja - 1)).max()))
    assert bw[1] * 3 < bw[0]


@pytest.mark.parametrize("solver", ["pcg", "bicgstab", "bicgstab_noprec", "gmres"])
def test_solvers_match_direct_solve(solver):
    m = M.box_tetra4(4, 3, 3, jitter=0.2, lognormal_E=True, seed=3)
    s = O.structure(m)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    K = full_matrix(s, ad, al)
    xd = spla.spsolve(K.tocsc(), b)
    fn = {"pcg": O.pcg, "bicgstab": O.pbicgstab, "bicgstab_noprec": O.bicgstab,
          "gmres": O.gmres}[solver]
    x, info = fn(s, ad, al, b, tol=1e-12)
    assert info["status"] == 0
    assert np.abs(x - xd).max() <= 1e-8 * np.abs(xd).max()


def test_plain_bicgstab_is_pbicgstab_with_unit_diagonal():
    """bicgstab (Iters.f:812-1075) is pbicgstab (Iters.f:1079-1349) with
    M = I, its beta from (r, b) the same as (r, r0) since x0 = 0 gives r0 = b
    exactly: on a matrix scaled to a unit diagonal (Jacobi M = I) the two
    restatements agree bitwise, iterate for iterate."""
    m = M.box_hexa8(5, 4, 4, jitter=0.2, seed=2)
    m.f = np.random.default_rng(4).standard_normal(m.f.shape) * (m.id == 0)
    s = O.structure(m)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    # D^-1/2 K D^-1/2 (D = diag(ad)): its diagonal is one, set exactly
    rows = np.repeat(np.arange(s.neq), np.diff(s.ia))
    al1 = al / np.sqrt(ad[rows] * ad[s.ja - 1])
    ad1 = np.ones(s.neq)
    for maxit in (1, 5, 40):
        x1, i1 = O.bicgstab(s, ad1, al1, b, tol=1e-14, maxit=maxit)
        x2, i2 = O.pbicgstab(s, ad1, al1, b, tol=1e-14, maxit=maxit)
        assert np.array_equal(x1, x2) and i1["iters"] == i2["iters"] == maxit
    x1, i1 = O.bicgstab(s, ad, al, b, tol=1e-12)
    assert i1["status"] == 0 and i1["norm_m_r"] == i1["norm_r"]
    assert i1["norm_r"] <= 3.16 * i1["conv"]


def test_flop_cg_count():
    """flop_cg (Matvec.f:1499-1531): per iteration one CSRC product
    (neq + 4 nad, flop_csrc), two dots (2 neq each), 7 neq of vector updates
    and 2 scalar operations; the PCG's Mflops are that count over its time."""
    assert O.flop_cg(10, 20, 3) == (10 + 80 + 40 + 70 + 2) * 3
    m = M.box_hexa8(5, 4, 3)
    s = O.structure(m)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    _, info = O.pcg(s, ad, al, b, tol=1e-10)
    np.testing.assert_allclose(info["mflops"] * info["seconds"] * 1e6,
                               O.flop_cg(s.neq, s.nad, info["iters"]), rtol=1e-9)


def test_openmp_pcg_matches_sequential_pcg():
    m = M.box_hexa8(10, 8, 6)
    s = O.structure(m)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    x1, i1 = O.pcg(s, ad, al, b, tol=1e-10)
    x2, i2 = O.pcg_omp(s, ad, al, b, tol=1e-10, nthreads=4)
    assert abs(i1["iters"] - i2["iters"]) <= 2
    assert np.abs(x1 - x2).max() <= 1e-10 * np.abs(x1).max()
    y1 = O.matvec(s, ad, al, b)
    y2, _ = O.matvec_omp(s, ad, al, b, nthreads=3)
    assert np.abs(y1 - y2).max() <= 1e-14 * np.abs(y1).max()


def test_matvec_is_the_symmetric_product():
    m = M.box2d(9, 7, etype=M.TRIA3_STRESS)
    s = O.structure(m)
    ad, al, _ = O.assemble(m, s)
    x = np.random.default_rng(1).standard_normal(s.neq)
    K = full_matrix(s, ad, al)
    assert np.abs(O.matvec(s, ad, al, x) - K @ x).max() <= 1e-13 * np.abs(K @ x).max()


def test_zero_diagonal_is_reported():
    m = M.box2d(3, 3)
    s = O.structure(m)
    ad, al, b = O.assemble(m, s)
    ad[2] = 0.0
    x, info = O.pcg(s, ad, al, np.ones(s.neq))
    assert info["status"] == 1
