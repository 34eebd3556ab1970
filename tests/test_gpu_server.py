"""Solve server (elx_server_*): continuous batching of many meshes.

Bars: every load case of every request equals the oracle's FP64 PCG solution
(pcg, Iters.f:252-524, tol 1e-10) within 1e-10 relative with iterations within
+-2; a request's result is bitwise the same alone and in a mix; admission
respects the HBM budget; a bad request fails alone without stopping the
server; requests above the size threshold, solved whole by the block PCG,
meet the same bars (FP64 block PCG: 1e-10; mixed: the FP64 stopping test and
1e-6 of the oracle) and are bitwise the same alone and in a mix.
"""
import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import rel_inf, rollers

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _requests(seed, count, dof_max=3e4):
    rng = np.random.default_rng(seed)
    return [M.serving_request(rng, dof_min=2e3, dof_max=dof_max, max_rhs=3)
            for _ in range(count)]


def _oracle(m, F):
    s = O.structure(m, True)
    out, iters = [], []
    for k in range(F.shape[0]):
        m.f = F[k]
        b0, u0 = O.loads(m, s)
        ad, al, b = O.assemble(m, s, u0, b0)
        x, info = O.pcg(s, ad, al, b, tol=TOL, maxit=50000)
        out.append(O.update(s, x, u0))
        iters.append(info["iters"])
    return np.array(out), iters


def test_mix_matches_oracle_and_solo(built_lib):
    reqs = _requests(3, 10)
    with E.Server(device=0) as srv:
        tickets = [srv.submit(m, F, tol=TOL, maxit=50000) for m, F in reqs]
        mixed = [srv.wait(t, timeout=300) for t in tickets]
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["peak_slots"] >= 2
        for (m, F), (U, infos, lat, status) in zip(reqs, mixed):
            assert status == 0 and lat > 0
            U_o, it_o = _oracle(m, F)
            for k in range(F.shape[0]):
                assert infos[k]["status"] == 0
                assert abs(infos[k]["iters"] - it_o[k]) <= 2, (m.name, k)
                assert rel_inf(U_o[k], U[k]) <= 1e-10, (m.name, k)
        # the same requests one at a time: bitwise the same results
        for (m, F), (U, infos, _, _) in zip(reqs[:4], mixed[:4]):
            U1, infos1, _, st1 = srv.wait(srv.submit(m, F, tol=TOL, maxit=50000), timeout=300)
            assert st1 == 0 and np.array_equal(U1, U)
            assert [i["iters"] for i in infos1] == [i["iters"] for i in infos]


def test_budget_admission(built_lib):
    reqs = _requests(5, 6)
    # find the largest single request's footprint with an unlimited server
    with E.Server(device=0) as srv:
        peaks = []
        for m, F in reqs:
            srv.wait(srv.submit(m, F, tol=1e-8), timeout=300)
            peaks.append(srv.stats()["peak_bytes"])
    budget = int(max(peaks) * 1.1)
    with E.Server(device=0, hbm_budget=budget) as srv:
        tickets = [srv.submit(m, F, tol=1e-8) for m, F in reqs]
        res = [srv.wait(t, timeout=300) for t in tickets]
        assert all(r[3] == 0 for r in res), ([r[3] for r in res], budget, peaks)
        st = srv.stats()
        assert st["peak_bytes"] <= budget and st["completed"] == len(reqs)
    # a request larger than the whole budget fails alone
    with E.Server(device=0, hbm_budget=1 << 20) as srv:
        m, F = reqs[0]
        _, _, _, status = srv.wait(srv.submit(m, F), timeout=300)
        assert status == E.ERR_OOM


def test_bad_request_does_not_stop_the_server(built_lib):
    good = _requests(7, 3)
    with E.Server(device=0) as srv:
        bad = rollers(M.box_hexa8(4, 4, 4))  # partly fixed nodes: no node blocks
        t_bad = srv.submit(bad, bad.f)
        tickets = [srv.submit(m, F, tol=1e-8) for m, F in good]
        assert srv.wait(t_bad, timeout=300)[3] == E.ERR_ARG
        assert all(srv.wait(t, timeout=300)[3] == 0 for t in tickets)


def test_no_convergence_reported(built_lib):
    m, F = _requests(9, 1)[0]
    with E.Server(device=0) as srv:
        U, infos, _, status = srv.wait(srv.submit(m, F, tol=1e-14, maxit=5), timeout=300)
        assert status == E.ERR_NO_CONVERGENCE
        assert all(i["iters"] == 5 for i in infos)
        assert np.isfinite(U).all()


@pytest.mark.parametrize("mode,bar", [(2, 1e-6), (1, 1e-10)])
def test_large_requests_solved_whole(built_lib, mode, bar):
    reqs = _requests(11, 6)
    with E.Server(device=0, large_dofs=1, large_mode=mode) as srv:
        tickets = [srv.submit(m, F, tol=TOL, maxit=50000) for m, F in reqs]
        res = [srv.wait(t, timeout=300) for t in tickets]
        assert srv.stats()["large_solved"] == len(reqs)
        for (m, F), (U, infos, lat, status) in zip(reqs, res):
            assert status == 0
            U_o, it_o = _oracle(m, F)
            for k in range(F.shape[0]):
                assert infos[k]["status"] == 0
                assert infos[k]["norm_m_r"] <= 3.16 * infos[k]["conv"]
                assert rel_inf(U_o[k], U[k]) <= bar, (m.name, k, mode)
                if mode == 1:
                    assert abs(infos[k]["iters"] - it_o[k]) <= 2
        # alone: bitwise the same
        for (m, F), (U, _, _, _) in zip(reqs[:3], res[:3]):
            U1, _, _, st1 = srv.wait(srv.submit(m, F, tol=TOL, maxit=50000), timeout=300)
            assert st1 == 0 and np.array_equal(U1, U)


def test_phase_statistics(built_lib):
    """The server times each finished request's phases (structure built,
    waiting for admission, admitted, waiting to start, solved); they add up
    to the request's latency, and the counts to the finished requests."""
    reqs = _requests(13, 8, dof_max=2e5)
    with E.Server(device=0, large_dofs=50000) as srv:
        tickets = [srv.submit(m, F, tol=1e-8) for m, F in reqs]
        res = [srv.wait(t, timeout=300) for t in tickets]
        assert all(r[3] == 0 for r in res)
        st = srv.stats()
    assert st["packed_finished"] + st["block_finished"] == len(reqs)
    assert st["block_finished"] == st["large_solved"]
    total = 0.0
    for kind in ("packed", "block"):
        n = st[f"{kind}_finished"]
        if not n:
            continue
        ph = st[f"{kind}_phases_mean_s"]
        assert set(ph) == {"prepare", "wait_admission", "admit", "wait_start", "solve"}
        assert all(v >= 0 for v in ph.values()) and ph["solve"] > 0 and ph["admit"] > 0
        total += n * sum(ph.values())
    lat = sum(r[2] for r in res)
    assert abs(total - lat) <= 1e-6 * lat, (total, lat)
