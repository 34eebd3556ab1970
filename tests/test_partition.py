"""Row-block partitions of the CSRC for a multi-GPU run (host side, no GPU):
the library's partition arrays equal the oracle's restatement of csrstruct
with lower = right = .true. (Csr.f:13-305) on the partition's local
numbering, bit for bit; the partitions' products through the oracle's
matvec_csrcrsym1 (Matvec.f:1090-1191) give the global product; and two gloo
ranks, each holding one partition and exchanging halo values, reproduce it
(the exchange a multi-GPU run does with NCCL)."""
import os
import socket

import numpy as np
import pytest

import elastic_gb300 as E
import oracle as O
from elastic_gb300 import meshgen as M
from helpers import rollers

MESHES = {
    "hexa8": lambda: M.box_hexa8(9, 8, 7, jitter=0.2, seed=5),
    "tetra4": lambda: M.box_tetra4(7, 6, 5, jitter=0.2, lognormal_E=True, seed=4),
    "quad4": lambda: M.box2d(40, 30, 2.0, 1.0, etype=M.QUAD4_STRESS),
    "rollers": lambda: rollers(M.box_hexa8(6, 5, 4)),  # partly fixed nodes: no node blocks
}


def _local_id(st, p):
    """The partition's local equation numbers: owned 1..neq, halo neq+1.."""
    g = st.id.astype(np.int64) - 1  # 0-based global, -1 fixed
    lid = np.zeros_like(st.id)
    own = (g >= p.eq0) & (g < p.eq0 + p.neq)
    lid[own] = g[own] - p.eq0 + 1
    h = np.searchsorted(p.halo, g)
    inh = (g >= 0) & ~own & (h < len(p.halo))
    inh[inh] = p.halo[h[inh]] == g[inh]
    lid[inh] = p.neq + 1 + h[inh]
    return lid


@pytest.mark.parametrize("nparts", [1, 2, 3, 5])
@pytest.mark.parametrize("name", sorted(MESHES))
def test_partition_structure_matches_oracle(name, nparts):
    m = MESHES[name]()
    st = E.host_structure(m, True)
    owned = 0
    for part in range(nparts):
        p = E.host_partition(m, nparts, part)
        assert p.eq0 == owned
        owned += p.neq
        ia, ja, ia1, ja1 = O.csr_right(m, _local_id(st, p), st.perm, p.neq)
        assert np.array_equal(p.ia, ia) and np.array_equal(p.ja, ja)
        assert np.array_equal(p.ia1, ia1) and np.array_equal(p.ja1, ja1)
        # values: every local entry points at its global entry
        for r in range(p.neq):
            g = p.eq0 + r
            for k in range(p.ia[r] - 1, p.ia[r + 1] - 1):
                q = p.pos[k]
                assert st.ja[q] - 1 == p.ja[k] - 1 + p.eq0 and st.ia[g] - 1 <= q < st.ia[g + 1] - 1
            for k in range(p.ia1[r] - 1, p.ia1[r + 1] - 1):
                q, c = p.pos1[k], p.halo[p.ja1[k] - p.neq - 1]
                row = np.searchsorted(st.ia - 1, q, side="right") - 1
                assert {row, st.ja[q] - 1} == {g, c}
    assert owned == st.neq


def _global(m):
    s = O.structure(m, True)
    b0, u0 = O.loads(m, s)
    ad, al, _ = O.assemble(m, s, u0, b0)
    x = np.random.default_rng(9).standard_normal(s.neq)
    return s, ad, al, x, O.matvec(s, ad, al, x)


def _part_product(m, ad, al, x, nparts, part):
    p = E.host_partition(m, nparts, part)
    xl = np.concatenate([x[p.eq0:p.eq0 + p.neq], x[p.halo]])
    y = O.matvec_csrcrsym1(p.neq, p.ia, p.ja, p.ia1, p.ja1, ad[p.eq0:p.eq0 + p.neq], al[p.pos],
                           al[p.pos1], xl)
    return p, y


@pytest.mark.parametrize("nparts", [2, 4])
@pytest.mark.parametrize("name", sorted(MESHES))
def test_partition_products_give_the_global_product(name, nparts):
    m = MESHES[name]()
    s, ad, al, x, y = _global(m)
    got = np.zeros_like(y)
    for part in range(nparts):
        p, yp = _part_product(m, ad, al, x, nparts, part)
        got[p.eq0:p.eq0 + p.neq] = yp
    assert np.abs(got - y).max() <= 1e-14 * np.abs(y).max()


def test_too_many_partitions_refused():
    m = M.box_hexa8(2, 2, 2)
    with pytest.raises(E.ElasticError) as e:
        E.host_partition(m, 4, 0)  # 27 nodes: one 32-node cut unit
    assert e.value.code == E.ERR_ARG


def _join_all(procs, timeout):
    """Joins the rank processes; a rank still running after `timeout` (hung
    in a collective) is terminated, so that it holds no port afterwards."""
    for pr in procs:
        pr.join(timeout)
    alive = [pr for pr in procs if pr.is_alive()]
    for pr in alive:
        pr.terminate()
        pr.join(5)
    assert not alive, "a rank did not finish"
    assert all(pr.exitcode == 0 for pr in procs), [pr.exitcode for pr in procs]


def _rank(rank, world, port, name, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = MESHES[name]()
        s, ad, al, x, y = _global(m)
        p = E.host_partition(m, world, rank)
        # each rank holds only its owned x; the halo comes from the others
        sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(sizes, torch.tensor([p.neq]))
        sizes = [int(n) for n in sizes]

        def gather(v):  # gloo gathers equal sizes: pad to the largest block
            pad = torch.zeros(max(sizes), dtype=torch.float64)
            pad[:len(v)] = torch.from_numpy(v)
            out = [torch.zeros(max(sizes), dtype=torch.float64) for _ in range(world)]
            dist.all_gather(out, pad)
            return np.concatenate([o[:n].numpy() for o, n in zip(out, sizes)])

        own = x[p.eq0:p.eq0 + p.neq].copy()
        xl = np.concatenate([own, gather(own)[p.halo]])
        yp = O.matvec_csrcrsym1(p.neq, p.ia, p.ja, p.ia1, p.ja1, ad[p.eq0:p.eq0 + p.neq],
                                al[p.pos], al[p.pos1], xl)
        got = gather(yp)
        if rank == 0:
            q.put(float(np.abs(got - y).max() / np.abs(y).max()))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["hexa8", "quad4"])
def test_two_gloo_ranks_exchange_halos(name):
    import torch.multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, name, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    _join_all(procs, 120)
    assert q.get(timeout=5) <= 1e-14


def _pcg_rank(rank, world, port, name, q):
    """Jacobi-PCG on row-block partitions, the reference's MPI form (pcg,
    Iters.f:252-524, with matvec_csrcrsym1 after the halo exchange and the
    dots summed over the ranks, Matvec.f:1258-1263)."""
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = MESHES[name]()
        m.f = np.random.default_rng(21).standard_normal(m.f.shape) * (m.id == 0)
        s = O.structure(m, True)
        b0, u0 = O.loads(m, s)
        ad, al, b = O.assemble(m, s, u0, b0)
        p = E.host_partition(m, world, rank)
        own = slice(p.eq0, p.eq0 + p.neq)
        sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(sizes, torch.tensor([p.neq]))
        sizes = [int(n) for n in sizes]

        def gather(v):
            pad = torch.zeros(max(sizes), dtype=torch.float64)
            pad[:len(v)] = torch.from_numpy(v)
            out = [torch.zeros(max(sizes), dtype=torch.float64) for _ in range(world)]
            dist.all_gather(out, pad)
            return np.concatenate([o[:n].numpy() for o, n in zip(out, sizes)])

        def dot(a, c):
            t = torch.tensor([float(np.dot(a, c))], dtype=torch.float64)
            dist.all_reduce(t)
            return float(t[0])

        adl, all_, arl = ad[own], al[p.pos], al[p.pos1]
        mi = 1.0 / adl
        bl = b[own]
        x = np.zeros(p.neq)
        r = bl.copy()
        z = mi * r
        pv = z.copy()
        d = dot(r, z)
        conv = 1e-10 * np.sqrt(abs(d))
        it = 0
        while it < 20000:
            xl = np.concatenate([pv, gather(pv)[p.halo]])
            qv = O.matvec_csrcrsym1(p.neq, p.ia, p.ja, p.ia1, p.ja1, adl, all_, arl, xl)
            alpha = d / dot(pv, qv)
            x += alpha * pv
            r -= alpha * qv
            z = mi * r
            dn = dot(r, z)
            it += 1
            if np.sqrt(abs(dn)) < conv:
                break
            pv = z + (dn / d) * pv
            d = dn
        xg = gather(x)
        if rank == 0:
            x_o, i_o = O.pcg(s, ad, al, b, tol=1e-10, maxit=20000)
            q.put((float(np.abs(xg - x_o).max() / np.abs(x_o).max()), it, i_o["iters"]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["hexa8", "tetra4"])
def test_two_gloo_ranks_partitioned_pcg(name):
    """The partitioned solve the multi-GPU design would run (one partition per
    rank, halo values exchanged before each product, the PCG dots all-reduced)
    reproduces the single solve: displacements within 1e-10, iterations within
    2 (the dots are summed in a different order)."""
    import torch.multiprocessing as mp
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_pcg_rank, args=(r, 2, port, name, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    _join_all(procs, 300)
    err, it, it_o = q.get(timeout=5)
    assert err <= 1e-10 and abs(it - it_o) <= 2, (err, it, it_o)
