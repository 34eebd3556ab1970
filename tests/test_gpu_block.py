"""Block PCG (elx_solve_block): nrhs load cases over one read of the matrix
per iteration, each column the reference's Jacobi PCG (pcg, Iters.f:252-524)
with its own scalars and stopping test.

Bars: FP64 columns equal the oracle's single-RHS PCG solutions within 1e-10
relative with iterations within +-2; mixed-precision columns meet the
reference's FP64 stopping test and their error against the FP64 oracle is
reported and bounded (1e-6 relative at tol 1e-10); a column's result does not
depend on the block it is solved in beyond the PCG tolerance.
"""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import rel_inf, rollers

pytestmark = pytest.mark.gpu


def _system(ctx, m, nrhs, seed=5):
    ctx.set_mesh(m)
    ctx.build_structure(True)
    s = O.structure(m, True)
    ad, al, _ = O.assemble(m, s, np.zeros((m.nnode, m.ndf)), np.zeros(s.neq))
    ctx.assemble(None, None)
    B = np.random.default_rng(seed).standard_normal((s.neq, nrhs))
    return s, ad, al, B


@pytest.mark.parametrize("width", [1, 4, 16])
def test_block_fp64_columns_match_oracle(gpu_ctx, width):
    m = M.box_hexa8(9, 8, 7, jitter=0.2, seed=5)
    s, ad, al, B = _system(gpu_ctx, m, 5)
    X, infos = gpu_ctx.solve_block(B, precision=E.PREC_FP64, tol=1e-10, width=width)
    for c in range(B.shape[1]):
        x_o, i_o = O.pcg(s, ad, al, B[:, c], tol=1e-10, maxit=20000)
        assert infos[c]["status"] == 0
        assert abs(infos[c]["iters"] - i_o["iters"]) <= 2, (c, infos[c]["iters"], i_o["iters"])
        assert rel_inf(x_o, X[:, c]) <= 1e-10
        np.testing.assert_allclose(infos[c]["conv"], i_o["conv"], rtol=1e-13)
        np.testing.assert_allclose(infos[c]["xkx"], i_o["xkx"], rtol=1e-10)


@pytest.mark.parametrize("name", ["hexa8", "tetra4", "quad4"])
def test_block_mixed_meets_fp64_test(gpu_ctx, name):
    m = {"hexa8": lambda: M.box_hexa8(9, 8, 7, jitter=0.2, seed=5),
         "tetra4": lambda: M.box_tetra4(7, 6, 5, jitter=0.2, lognormal_E=True, seed=4),
         "quad4": lambda: M.cantilever_quad4_64x16()}[name]()
    s, ad, al, B = _system(gpu_ctx, m, 6)
    X, infos = gpu_ctx.solve_block(B, precision=E.PREC_MIXED, tol=1e-10, width=8)
    for c in range(B.shape[1]):
        x_o, _ = O.pcg(s, ad, al, B[:, c], tol=1e-12, maxit=50000)
        assert infos[c]["status"] == 0 and infos[c]["refinements"] >= 1
        assert infos[c]["norm_m_r"] <= 3.16 * infos[c]["conv"]
        assert rel_inf(x_o, X[:, c]) <= 1e-6


def test_block_column_independent_of_block(gpu_ctx):
    m = M.box_tetra4(6, 6, 5, jitter=0.15, seed=9)
    s, ad, al, B = _system(gpu_ctx, m, 7)
    X16, i16 = gpu_ctx.solve_block(B, precision=E.PREC_FP64, tol=1e-11, width=16)
    X1, i1 = gpu_ctx.solve_block(B[:, 3:4], precision=E.PREC_FP64, tol=1e-11, width=1)
    assert rel_inf(X1[:, 0], X16[:, 3]) <= 1e-10
    assert abs(i1[0]["iters"] - i16[3]["iters"]) <= 2
    Xm, _ = gpu_ctx.solve_block(B, precision=E.PREC_MIXED, tol=1e-11, width=4)
    Xm1, _ = gpu_ctx.solve_block(B[:, 5:6], precision=E.PREC_MIXED, tol=1e-11, width=1)
    assert rel_inf(Xm1[:, 0], Xm[:, 5]) <= 1e-7


def test_block_zero_column_and_ragged_count(gpu_ctx):
    m = M.box_hexa8(6, 5, 4)
    s, ad, al, B = _system(gpu_ctx, m, 5)
    B[:, 2] = 0.0
    X, infos = gpu_ctx.solve_block(B, precision=E.PREC_MIXED, tol=1e-10, width=4)
    assert infos[2]["status"] == 0 and infos[2]["iters"] == 0
    assert np.all(X[:, 2] == 0.0)
    for c in (0, 1, 3, 4):
        assert infos[c]["status"] == 0 and infos[c]["iters"] > 0


def test_block_no_convergence_reported(gpu_ctx):
    m = M.box_hexa8(6, 5, 4)
    _, _, _, B = _system(gpu_ctx, m, 3)
    X, infos = gpu_ctx.solve_block(B, precision=E.PREC_FP64, tol=1e-14, maxit=3,
                                   raise_on_error=False)
    assert all(i["status"] == E.ERR_NO_CONVERGENCE for i in infos)
    assert np.isfinite(X).all()


def test_block_needs_node_blocks(gpu_ctx):
    m = rollers(M.box_hexa8(5, 4, 4))
    _, _, _, B = _system(gpu_ctx, m, 2)
    with pytest.raises(E.ElasticError) as e:
        gpu_ctx.solve_block(B)
    assert e.value.code == E.ERR_ARG


def test_block_autotune(gpu_ctx):
    m = M.box_hexa8(12, 12, 10)
    _system(gpu_ctx, m, 1)
    for prec in (E.PREC_FP64, E.PREC_MIXED):
        w, t = gpu_ctx.autotune_block(prec, remeasure=True)
        assert w in (1, 2, 4, 8, 16)
        assert np.all(t > 0)
        assert gpu_ctx.autotune_block(prec)[0] == w


def test_mixed_falls_back_to_fp64_on_ill_conditioned_2d(gpu_ctx):
    """A 2-D mesh of ~10^5 dofs is ill-conditioned enough for its FP32 matrix
    to stall or diverge the FP32 iteration; the mixed solvers then solve the
    case in FP64 (refinements = -1).  Either way the answer meets the FP64
    stopping test and matches the FP64 solve."""
    m = M.box2d(240, 120, 2.0, 1.0, etype=M.QUAD4_STRESS, E=1.0, nu=0.3)
    gpu_ctx.set_mesh(m)
    gpu_ctx.build_structure(True)
    neq = gpu_ctx.sizes()[0]
    gpu_ctx.assemble(None, None)
    B = np.random.default_rng(12).standard_normal((neq, 3))
    X64, i64 = gpu_ctx.solve_block(B, precision=E.PREC_FP64, tol=1e-10, width=4)
    Xm, im = gpu_ctx.solve_block(B, precision=E.PREC_MIXED, tol=1e-10, width=4)
    x1, i1 = gpu_ctx.solve(B[:, 0], precision=E.PREC_MIXED, tol=1e-10, maxit=50000)
    for c in range(3):
        assert im[c]["status"] == 0 and im[c]["norm_m_r"] <= 3.16 * im[c]["conv"]
        bar = 1e-10 if im[c]["refinements"] == -1 else 1e-6
        assert rel_inf(X64[:, c], Xm[:, c]) <= bar
    assert i1["status"] == 0 and i1["norm_m_r"] <= 3.16 * i1["conv"]
    assert rel_inf(X64[:, 0], x1) <= (1e-10 if i1["refinements"] == -1 else 1e-6)


@pytest.mark.parametrize("precision", [E.PREC_MIXED, E.PREC_FP64])
def test_autotuned_tiling_gives_the_same_bits(built_lib, monkeypatch, precision):
    """The autotuner picks, per width, how many slot groups of matrix loads
    the block product keeps in flight (1-3 on 3x3 node blocks).  Each row's
    sums run in the block order whatever that number, so every tiling gives
    the same bits: the autotuned solve equals solves with the tiling fixed
    to 1 and to 3 (ELX_SPMM_UNROLL)."""
    m = M.box_hexa8(9, 8, 7, jitter=0.2, seed=5)
    results = []
    for fixed in (None, "1", "3"):
        if fixed is None:
            monkeypatch.delenv("ELX_SPMM_UNROLL", raising=False)
        else:
            monkeypatch.setenv("ELX_SPMM_UNROLL", fixed)
        with E.Context(device=0) as ctx:
            _, _, _, B = _system(ctx, m, 6)
            w, _ = ctx.autotune_block(precision, remeasure=True)
            tiling = ctx.block_tiling(precision)
            if fixed is None:
                assert all(1 <= u <= 3 for u in tiling), tiling
            else:
                assert tiling == [0] * 5  # a fixed tiling is not tuned
            X, infos = ctx.solve_block(B, precision=precision, tol=1e-10, width=8)
            assert all(i["status"] == 0 for i in infos)
            results.append(X)
    assert np.array_equal(results[0], results[1]) and np.array_equal(results[0], results[2])
