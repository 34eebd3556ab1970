"""The single-read tiled CSRC product (ELX_SPMV=tile: matvec_csrcsym1's
one-pass form, Matvec.f:528-621 -- each entry of al read once from HBM, the
mirrored half summed per tile column and through halo slots) against the
oracle, alone and inside PCG; and its bounded waits: with the producer of
the bulk-copy pipeline stalled on purpose (ELX_PIPE_STALL_TEST=1, nothing
arrives at the barriers) every wait runs out after about a second, the call
returns ELX_ERR_TIMEOUT, and the same context computes the product
correctly once the stall is lifted."""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import rel_inf

pytestmark = pytest.mark.gpu

MESHES = {
    "hexa8": lambda: M.box_hexa8(9, 8, 7, jitter=0.2, seed=5),
    "tetra4": lambda: M.box_tetra4(7, 6, 5, jitter=0.2, lognormal_E=True, seed=4),
    "quad4_stress": lambda: M.cantilever_quad4_64x16(),
}


def _tiled_ctx(monkeypatch, m):
    monkeypatch.setenv("ELX_SPMV", "tile")
    ctx = E.Context(device=0)
    ctx.set_mesh(m)
    ctx.build_structure(True)
    return ctx


@pytest.mark.parametrize("name", sorted(MESHES))
def test_tiled_product_and_pcg_match_oracle(built_lib, monkeypatch, name):
    m = MESHES[name]()
    rng = np.random.default_rng(13)
    m.f = rng.standard_normal(m.f.shape) * (m.id == 0)
    ctx = _tiled_ctx(monkeypatch, m)
    try:
        s = O.structure(m, True)
        b0, u0 = O.loads(m, s)
        ad, al, b = O.assemble(m, s, u0, b0)
        b_g = ctx.assemble(u0, b0)
        x = rng.standard_normal(s.neq)
        assert rel_inf(O.matvec(s, ad, al, x), ctx.spmv(x)) <= 1e-14
        x_o, i_o = O.pcg(s, ad, al, b, tol=1e-10, maxit=20000)
        x_g, i_g = ctx.solve(b_g, tol=1e-10, maxit=20000)
        assert i_g["status"] == 0 and abs(i_g["iters"] - i_o["iters"]) <= 2
        assert rel_inf(x_o, x_g) <= 1e-10
    finally:
        ctx.close()


def test_tiled_waits_time_out_and_context_recovers(built_lib, monkeypatch):
    m = MESHES["hexa8"]()
    ctx = _tiled_ctx(monkeypatch, m)
    try:
        s = O.structure(m, True)
        b0, u0 = O.loads(m, s)
        ad, al, _ = O.assemble(m, s, u0, b0)
        ctx.assemble(u0, b0)
        x = np.random.default_rng(3).standard_normal(s.neq)
        monkeypatch.setenv("ELX_PIPE_STALL_TEST", "1")
        with pytest.raises(E.ElasticError) as e:
            ctx.spmv(x)
        assert e.value.code == E.ERR_TIMEOUT
        monkeypatch.delenv("ELX_PIPE_STALL_TEST")
        assert rel_inf(O.matvec(s, ad, al, x), ctx.spmv(x)) <= 1e-14
    finally:
        ctx.close()
