"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

Bars (from the reference's own tolerances of the path):
  * ia/ja/perm/id bit-exact;
  * assembled ad/al within 1e-13 of the oracle, relative to each row's
    largest entry; b = b0 - K u within 1e-13 of max|b|;
  * SpMV within 1e-14 relative (inf-norm), different summation order only;
  * FP64 PCG displacements within 1e-10 relative, iterations within +-2.
"""
import json
import os
import sys

import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import relabel_nodes, rel_inf, rollers, row_scaled_error, two_components

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
ASSEMBLY_TOL = 1e-13
SPMV_TOL = 1e-14
U_TOL = 1e-10


def _setup(ctx, m, reorder=True):
    ctx.set_mesh(m)
    ctx.build_structure(reorder)
    return O.structure(m, reorder)


MESHES = {
    "tria3_strain": lambda: M.box2d(12, 9, 2.0, 1.0, etype=M.TRIA3_STRAIN, E=3.0, nu=0.25),
    "tria3_stress": lambda: M.box2d(12, 9, 2.0, 1.0, etype=M.TRIA3_STRESS, E=3.0, nu=0.25,
                                    thick=2.0),
    "quad4_strain": lambda: M.box2d(16, 8, 2.0, 1.0, etype=M.QUAD4_STRAIN),
    "quad4_stress": lambda: M.cantilever_quad4_64x16(),
    "tetra4": lambda: M.box_tetra4(7, 6, 5, jitter=0.2, lognormal_E=True, seed=4),
    "hexa8": lambda: M.box_hexa8(9, 8, 7, jitter=0.2, seed=5),
    "hexa8_scrambled": lambda: relabel_nodes(M.box_hexa8(6, 5, 4), 8),
    "tetra4_two_components": lambda: two_components(M.box_tetra4(3, 3, 3)),
    # partly fixed nodes: no node blocks, the scalar (two-sided gather) kernels
    "hexa8_rollers": lambda: rollers(M.box_hexa8(7, 6, 5, jitter=0.1, seed=6)),
}


@pytest.mark.parametrize("name", sorted(MESHES))
def test_assembly_parity(gpu_ctx, name):
    m = MESHES[name]()
    s = _setup(gpu_ctx, m)
    st = gpu_ctx.structure()
    assert np.array_equal(st.ia, s.ia) and np.array_equal(st.ja, s.ja)
    assert np.array_equal(st.perm, s.perm) and np.array_equal(st.id, s.id)
    rng = np.random.default_rng(1)
    u = rng.standard_normal((m.nnode, m.ndf)) * 1e-2
    b0 = rng.standard_normal(s.neq)
    ad_o, al_o, b_o = O.assemble(m, s, u, b0)
    b_g, ad_g, al_g = gpu_ctx.assemble(u, b0, want_matrix=True)
    assert row_scaled_error(s.ia, al_o, al_g, ad_o, ad_g) <= ASSEMBLY_TOL
    assert rel_inf(b_o, b_g) <= ASSEMBLY_TOL


def test_caller_supplied_structure_matches_built_structure(gpu_ctx):
    m = M.box_hexa8(5, 4, 4, jitter=0.1)
    s = O.structure(m, True)
    gpu_ctx.set_mesh(m)
    gpu_ctx.set_structure(s.id, s.ia, s.ja)
    b1, ad1, al1 = gpu_ctx.assemble(None, None, want_matrix=True)
    _setup(gpu_ctx, m)
    b2, ad2, al2 = gpu_ctx.assemble(None, None, want_matrix=True)
    assert np.array_equal(ad1, ad2) and np.array_equal(al1, al2)


@pytest.mark.parametrize("name", ["quad4_stress", "tetra4", "hexa8", "hexa8_rollers"])
def test_spmv_parity(gpu_ctx, name):
    m = MESHES[name]()
    s = _setup(gpu_ctx, m)
    _, ad, al = gpu_ctx.assemble(None, None, want_matrix=True)
    x = np.random.default_rng(2).standard_normal(s.neq)
    y_o = O.matvec(s, ad, al, x)
    y_g = gpu_ctx.spmv(x)
    assert rel_inf(y_o, y_g) <= SPMV_TOL


@pytest.mark.parametrize("name", ["quad4_stress", "tria3_stress", "tetra4", "hexa8",
                                  "hexa8_rollers"])
def test_pcg_parity(gpu_ctx, name):
    m = MESHES[name]()
    # every mesh gets a seeded nodal load (some generators carry none)
    m.f = np.random.default_rng(7).standard_normal(m.f.shape) * (m.id == 0)
    s = _setup(gpu_ctx, m)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    x_o, i_o = O.pcg(s, ad, al, b, tol=1e-10, maxit=20000)
    gpu_ctx.assemble(u0, b0)
    x_g, i_g = gpu_ctx.solve(b, tol=1e-10, maxit=20000)
    assert i_o["status"] == 0 and i_g["status"] == 0
    assert abs(i_o["iters"] - i_g["iters"]) <= 2
    assert rel_inf(x_o, x_g) <= U_TOL
    np.testing.assert_allclose(i_g["xkx"], i_o["xkx"], rtol=1e-10)
    np.testing.assert_allclose(i_g["conv"], i_o["conv"], rtol=1e-13)
    assert i_g["norm_m_r"] <= 3.16 * i_g["conv"]


@pytest.mark.parametrize("name", ["hexa8", "quad4_stress", "tetra4"])
def test_block_and_scalar_kernels_agree(gpu_ctx, name, monkeypatch):
    """The node-block product and the scalar two-sided gather (node blocks
    switched off) give the oracle's K x, and PCG the same solution."""
    m = MESHES[name]()
    s = _setup(gpu_ctx, m)
    _, ad, al = gpu_ctx.assemble(None, None, want_matrix=True)
    x = np.random.default_rng(3).standard_normal(s.neq)
    b = np.random.default_rng(4).standard_normal(s.neq)
    y_blocks = gpu_ctx.spmv(x)
    u_blocks, _ = gpu_ctx.solve(b, tol=1e-11, maxit=20000)
    bytes_blocks = gpu_ctx.device_bytes
    monkeypatch.setenv("ELX_BLOCKS", "0")
    _setup(gpu_ctx, m)
    gpu_ctx.assemble(None, None)
    y_scalar = gpu_ctx.spmv(x)
    u_scalar, _ = gpu_ctx.solve(b, tol=1e-11, maxit=20000)
    assert gpu_ctx.device_bytes != bytes_blocks  # a different matrix layout was resident
    y_o = O.matvec(s, ad, al, x)
    assert rel_inf(y_o, y_blocks) <= SPMV_TOL and rel_inf(y_o, y_scalar) <= SPMV_TOL
    assert rel_inf(u_blocks, u_scalar) <= U_TOL


def test_solvm_quad_known_answer(gpu_ctx):
    """The driver's solvm sequence on the library for the reference's quad
    deck model: sqrt(xKx) equals the oracle's (golden) and is within the
    discretisation error of the deck's exact 1.379745."""
    gold = json.load(open(os.path.join(GOLD, "golden.json")))["decks"]["quad_el"]
    m = M.square_quad4_100()
    u, info, _ = E.solvm(m, tol=1e-11, ctx=gpu_ctx)
    e = np.sqrt(info["xkx"])
    assert abs(e - gold["sqrt_xkx"]) <= 1e-10 * e
    assert abs(info["iters"] - gold["iters"]) <= 2
    assert abs(e - 1.379745) / 1.379745 < 1e-3
    np.testing.assert_allclose(np.abs(u).max(), gold["u_max_abs"], rtol=1e-10)


@pytest.mark.parametrize("key", ["hexa_nf", "tetra_nf"])
def test_solvm_reference_decks(gpu_ctx, key):
    sys.path.insert(0, GOLD)
    from make_golden import load_deck_mesh
    gold = json.load(open(os.path.join(GOLD, "golden.json")))["decks"][key]
    m = load_deck_mesh(key)
    u, info, _ = E.solvm(m, tol=1e-11, ctx=gpu_ctx)
    np.testing.assert_allclose(info["xkx"], gold["xkx"], rtol=1e-10)
    assert abs(info["iters"] - gold["iters"]) <= 2
    np.testing.assert_allclose(np.abs(u).max(), gold["u_max_abs"], rtol=1e-10)


def test_solve_is_deterministic(gpu_ctx):
    m = MESHES["tetra4"]()
    s = _setup(gpu_ctx, m)
    b0, u0 = O.loads(m, s)
    b = gpu_ctx.assemble(u0, b0)
    x1, i1 = gpu_ctx.solve(b, tol=1e-10)
    b2 = gpu_ctx.assemble(u0, b0)
    x2, i2 = gpu_ctx.solve(b2, tol=1e-10)
    assert np.array_equal(b, b2) and np.array_equal(x1, x2) and i1["iters"] == i2["iters"]


# ------------------------------------------------------------------ errors
def test_bad_determinant_reports_the_element(gpu_ctx):
    m = M.box_tetra4(3, 3, 2)
    m.ix[4, [0, 1]] = m.ix[4, [1, 0]]  # invert element 5
    _setup(gpu_ctx, m)
    with pytest.raises(E.ElasticError) as ei:
        gpu_ctx.assemble()
    assert ei.value.code == E.ERR_BAD_DET and "element 5" in str(ei.value)


def test_zero_diagonal_is_reported(gpu_ctx):
    m = M.box2d(4, 3)
    s = _setup(gpu_ctx, m)
    ad, al, _ = O.assemble(m, s)
    ad[3] = 0.0
    gpu_ctx.set_matrix(ad, al)
    with pytest.raises(E.ElasticError) as ei:
        gpu_ctx.solve(np.ones(s.neq))
    assert ei.value.code == E.ERR_ZERO_DIAG and "equation 4" in str(ei.value)


def test_no_convergence_is_reported(gpu_ctx):
    m = M.box_hexa8(6, 6, 6)
    s = _setup(gpu_ctx, m)
    b0, u0 = O.loads(m, s)
    b = gpu_ctx.assemble(u0, b0)
    x, info = gpu_ctx.solve(b, tol=1e-12, maxit=5, raise_on_error=False)
    assert info["status"] == E.ERR_NO_CONVERGENCE and info["iters"] == 5
    with pytest.raises(E.ElasticError):
        gpu_ctx.solve(b, tol=1e-12, maxit=5)


def test_bad_element_type_rejected(gpu_ctx):
    m = M.box2d(2, 2)
    m.ie[:] = 9
    with pytest.raises(E.ElasticError) as ei:
        gpu_ctx.set_mesh(m)
    assert ei.value.code == E.ERR_BAD_ELEMENT


def test_hbm_budget_is_enforced(built_lib):
    m = M.box_hexa8(10, 10, 10)
    with E.Context(hbm_budget=1 << 20) as c:
        c.set_mesh(m)
        with pytest.raises(E.ElasticError) as ei:
            c.build_structure(True)
        assert ei.value.code == E.ERR_OOM


# ------------------------------------------------------------ full size
def test_full_size_cube_solve_properties(gpu_ctx):
    """64^3 HEXA8 (811,200 equations) to 1e-8: size-independent properties of
    the result -- the explicit residual meets the stopping test, the energy
    equals (b, x), and a second run is bitwise identical."""
    m = M.cube_hexa8_64()
    gpu_ctx.set_mesh(m)
    neq, nad, _ = gpu_ctx.build_structure(True)
    assert (neq, nad) == (811200, 31442295)
    st = gpu_ctx.structure()
    b0, u0 = E.pload(m, st.id)
    b = gpu_ctx.assemble(u0, b0)
    x, info = gpu_ctx.solve(b, tol=1e-8, maxit=20000)
    assert info["norm_m_r"] <= 3.16 * info["conv"]
    np.testing.assert_allclose(info["xkx"], b @ x, rtol=1e-6)
    x2, info2 = gpu_ctx.solve(b, tol=1e-8, maxit=20000)
    assert np.array_equal(x, x2)


# ------------------------------------------------------------ mixed precision
FP32_SPMV_TOL = 1e-6


@pytest.mark.parametrize("name", ["quad4_stress", "tetra4", "hexa8"])
def test_fp32_spmv_parity(gpu_ctx, name):
    """The FP32 product of the mixed-precision inner iteration, against the
    FP64 oracle (FP32 values and vectors: relative error near 1e-7)."""
    m = MESHES[name]()
    s = _setup(gpu_ctx, m)
    _, ad, al = gpu_ctx.assemble(None, None, want_matrix=True)
    x = np.random.default_rng(3).standard_normal(s.neq)
    y_o = O.matvec(s, ad, al, x)
    y_g = gpu_ctx.spmv(x, precision=E.PREC_MIXED)
    assert rel_inf(y_o, y_g) <= FP32_SPMV_TOL


@pytest.mark.parametrize("env", [{"ELX_SELL_STREAM": "0"},
                                 {"ELX_SELL_STREAM": "1"},
                                 {"ELX_SELL_STREAM": "1", "ELX_SELL_D16": "0"}])
@pytest.mark.parametrize("name", ["quad4_stress", "hexa8"])
def test_fp32_spmv_kernel_choices(built_lib, monkeypatch, name, env):
    """Each FP32 node-block product (sliced copy with streaming loads and
    16-bit or 32-bit columns, or cached loads) against the FP64 oracle."""
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    m = MESHES[name]()
    ctx = E.Context(device=0)
    try:
        s = _setup(ctx, m)
        _, ad, al = ctx.assemble(None, None, want_matrix=True)
        x = np.random.default_rng(5).standard_normal(s.neq)
        assert rel_inf(O.matvec(s, ad, al, x), ctx.spmv(x, precision=E.PREC_MIXED)) <= FP32_SPMV_TOL
    finally:
        ctx.close()


@pytest.mark.parametrize("name", ["quad4_stress", "tetra4", "hexa8"])
def test_mixed_precision_refinement_matches_fp64(gpu_ctx, name):
    """FP32 inner PCG + FP64 refinement meets the reference's FP64 stopping
    test, and its solution agrees with the FP64 oracle's PCG solution to the
    accuracy both solves carry (tolerance 1e-10)."""
    m = MESHES[name]()
    m.f = np.random.default_rng(7).standard_normal(m.f.shape) * (m.id == 0)
    s = _setup(gpu_ctx, m)
    b0, u0 = O.loads(m, s)
    ad, al, b = O.assemble(m, s, u0, b0)
    x_o, i_o = O.pcg(s, ad, al, b, tol=1e-10, maxit=20000)
    gpu_ctx.assemble(u0, b0)
    x_g, i_g = gpu_ctx.solve(b, tol=1e-10, maxit=20000, precision=E.PREC_MIXED)
    assert i_g["status"] == 0 and i_g["refinements"] >= 1
    assert i_g["norm_m_r"] <= i_g["conv"] * (1 + 1e-6)
    assert rel_inf(x_o, x_g) <= 1e-7
