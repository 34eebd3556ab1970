"""Benchmark of the linear-elasticity solve path on GB300.

Workload: 3-D HEXA8 cube 64x64x64 elements on [0,1]^3 (811,200 equations,
31,442,295 strict-lower CSRC entries), E=1, nu=0.3, z=0 face fixed, unit
pressure on z=1 as consistent nodal forces, RCM ordering, FP64 Jacobi-PCG to
1e-8 (the reference's M-norm test).  Synthetic, seeded-free structured mesh.

One step = one pass of the hot path: element integration + CSRC assembly
(pform_mec isw=2) and the PCG solve to tolerance (solv).  `value` is solves/s
with the mesh, structure and load vectors already resident on the device;
`e2e` is the same through the C ABI with host buffers (u, b0 in, b out;
b in, x out) copied every step.  Sub-objects: `mixed` (the same step with
the mixed-precision solver), `after_solve` (the device load step, stress
recovery and the result file on the solution, against the oracle's stress
recovery and writer; the product through 4 row-block partitions), `block`
(16 load cases of the 96x96x48 plate), `tetra` (FP64 and mixed PCG to 1e-10
on the 48^3 TETRA4 mesh with per-element materials, against the oracle's
FP64 solve) and `serve` (a served request stream against sequential plain
FP64 solves; `served.phases_mean_s` splits the packed and the block-solved
requests' mean latency into preparation, waiting for admission, admission,
waiting to start and solve).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --gpus N > 1 (torchrun, one rank per GPU) every rank solves its own copy
(the path has no data-parallel exchange: replicas, weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CSRC-PCG time-to-1e-8 & SpMV HBM GB/s; served solves/s, p99 vs plain FP64"
WORKLOAD = ("HEXA8 cube 64x64x64 on [0,1]^3, E=1, nu=0.3, z=0 fixed, unit pressure on z=1 "
            "(nodal forces), RCM, FP64 Jacobi-PCG to 1e-8: assembly + solve per step")
TOL = 1e-8
MAXIT = 20000


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, impl):
        self.ws, self.rank, self.local = _dist()
        self.pg = None
        if self.ws > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if (impl == "ours" and torch.cuda.is_available()) else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            td.init_process_group(backend)
            self.td = td
            self.backend = backend

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        dev = f"cuda:{self.local}" if self.backend == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        # the raw samples (ELX_CLOCKS_DIR, else the system's temporary folder)
        import tempfile
        folder = os.environ.get("ELX_CLOCKS_DIR", tempfile.gettempdir())
        self.path = os.path.join(folder, f"elx_clocks_bench_{gpu}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [v.strip() for v in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        load = [v for v in sm if v > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ helpers
def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled(key, name="sell_spmv_fp64_hexa8_cube64.md"):
    """A figure (`key: value` line) from a committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    m = re.search(key + r":\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


def make_workload():
    from elastic_gb300 import meshgen as M
    return M.cube_hexa8_64()


# ------------------------------------------------------------------ our arm
def run_ours(args, dist: Dist):
    import torch

    import elastic_gb300 as E

    dev = dist.local
    torch.cuda.set_device(dev)
    mesh = make_workload()
    ctx = E.Context(device=dev)
    ctx.set_mesh(mesh)
    neq, nad, ncolors = ctx.build_structure(True)
    st = ctx.structure()
    b0, u0 = E.pload(mesh, st.id)
    ext = torch.cuda.ExternalStream(ctx.stream, device=dev)

    # ---- device-resident steps
    ctx.set_state(u0, b0)
    infos = []
    for _ in range(args.warmup):
        ctx.assemble_resident()
        infos.append(ctx.solve_resident(tol=TOL, maxit=MAXIT))
    dist.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(dev)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev_a = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    launches0 = ctx.kernel_launches
    ev0.record(ext)
    t0 = time.perf_counter()
    for k in range(args.steps):
        ev_a[2 * k].record(ext)
        ctx.assemble_resident()
        ev_a[2 * k + 1].record(ext)
        infos.append(ctx.solve_resident(tol=TOL, maxit=MAXIT))
    ev1.record(ext)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
    launches = ctx.kernel_launches - launches0
    ms_total = ev0.elapsed_time(ev1)
    asm_ms = statistics.median(ev_a[2 * k].elapsed_time(ev_a[2 * k + 1])
                               for k in range(args.steps))
    dist.barrier()
    ms_total = dist.max(ms_total)
    ms_step = ms_total / args.steps
    iters = infos[-1]["iters"]

    x64 = ctx.solution()

    # ---- the SpMV as the solver launches it (the dominant kernel), timed on
    # its own stream; the matrix (400 MB FP64, 252 MB FP32 two-sided) is
    # larger than L2, so every launch streams it from HBM
    def time_spmv(prec, reps=50):
        ctx.spmv_resident(precision=prec, reps=5)
        torch.cuda.synchronize(dev)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(ext)
        ctx.spmv_resident(precision=prec, reps=reps)
        s1.record(ext)
        torch.cuda.synchronize(dev)
        return s0.elapsed_time(s1) / reps

    spmv_ms = time_spmv(E.PREC_FP64)
    spmv_bytes = 12 * nad + 28 * neq
    spmv_gbs = spmv_bytes / (spmv_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    iter_bytes = 12 * nad + 116 * neq
    pcg_ms = ms_step - asm_ms
    iter_gbs = iter_bytes * iters / (pcg_ms * 1e-3) / 1e9

    # ---- the same step with the mixed-precision solver (FP32 inner PCG with
    # FP64 reliable updates, the FP64 stopping test)
    mixed_ms, mixed_pcg_ms, minfo = [], [], None
    for k in range(args.warmup + args.steps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(ext)
        ctx.assemble_resident()
        e2.record(ext)
        minfo = ctx.solve_resident(precision=E.PREC_MIXED, tol=TOL, maxit=MAXIT)
        e1.record(ext)
        torch.cuda.synchronize(dev)
        if k >= args.warmup:
            mixed_ms.append(e0.elapsed_time(e1))
            mixed_pcg_ms.append(e2.elapsed_time(e1))
    xm = ctx.solution()
    spmv32_ms = time_spmv(E.PREC_MIXED)
    # device bytes the context holds with both solvers' data resident: mesh,
    # structure, CSRC ad / al, the sliced FP64 and FP32 copies, vectors
    device_bytes = ctx.device_bytes
    spmv32_bytes = 8 * nad + 16 * neq
    clk = clocks.stop()
    mixed_step = dist.max(statistics.median(mixed_ms))

    # ---- end to end through the C ABI with host buffers (pinned)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    u_h, b0_h = pin(u0), pin(b0)
    e2e_times = []
    for k in range(args.warmup + args.steps):
        dist.barrier()
        t = time.perf_counter()
        b_h = ctx.assemble(u_h, b0_h)
        x_h, info = ctx.solve(b_h, tol=TOL, maxit=MAXIT)
        dt = time.perf_counter() - t
        if k >= args.warmup:
            e2e_times.append(dt)
    e2e_s = dist.max(sum(e2e_times)) / args.steps
    h2d = (u0.size + 2 * neq) * 8
    d2h = 2 * neq * 8

    # ---- the rows after the solve: the load step on the device (pload_mec:
    # f up, b0 and u formed there) and stress recovery (tform_mec with the
    # elements' isw = 3, nodal stresses back to the host), each through its
    # C ABI call on the resident solution
    f_h = pin(mesh.f)
    ctx.set_state(None, None)
    ctx.set_loads(f_h)
    ctx.assemble_resident()
    ctx.solve_resident(tol=TOL, maxit=MAXIT)
    ctx.update_resident()
    ld_s, sr_s = [], []
    for k in range(args.warmup + args.steps):
        t = time.perf_counter()
        ctx.set_loads(f_h)
        t1 = time.perf_counter()
        stresses = ctx.stress(None)
        t2 = time.perf_counter()
        if k >= args.warmup:
            ld_s.append(t1 - t)
            sr_s.append(t2 - t1)
    u_sol, _ = ctx.state()
    # the result file (write_mesh_res_mec, XML VTU ASCII with u and stresses)
    # formatted on the device, copied back and written to a scratch file
    import tempfile
    vtk_dir = tempfile.mkdtemp(prefix="elx_vtk_")
    vtk_path = os.path.join(vtk_dir, "res.vtu")
    vt_s = []
    for k in range(args.warmup + args.steps):
        t = time.perf_counter()
        vtk_bytes = ctx.write_vtk(vtk_path)
        if k >= args.warmup:
            vt_s.append(time.perf_counter() - t)
    # the partitioned product: 4 row blocks with their halo gathers (the data
    # path of a 4-GPU run, all partitions on this GPU), against the single
    # product timed above
    ctx.partition_spmv_resident(4, 3)
    torch.cuda.synchronize(dev)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(ext)
    ctx.partition_spmv_resident(4, 20)
    p1.record(ext)
    torch.cuda.synchronize(dev)
    part = {"nparts": 4, "ms": p0.elapsed_time(p1) / 20, "single_ms": spmv_ms,
            "halo_equations": sum(ctx.partition_info(4, q)[2] for q in range(4))}
    nxt = {"loads_ms": 1e3 * statistics.median(ld_s), "loads_h2d_bytes": mesh.f.size * 8,
           "stress_ms": 1e3 * statistics.median(sr_s),
           "stress_d2h_bytes": stresses.size * 8, "elements": mesh.numel,
           "vtk_ms": 1e3 * statistics.median(vt_s), "vtk_bytes": vtk_bytes,
           "partitioned_spmv": part}

    # the FP64 product's floor on this part: one DFMA per stored entry of the
    # full matrix (2 nad + neq) at the FP64 pipe's rate, measured here by the
    # library's register-only probe (elx_fp64_fma_rate), scaled to the SM
    # clock sampled during the run
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz")
    fma_rate, per_clk = E.fp64_fma_rate(dev)
    fp64_floor = None
    if mhz:
        dfma = 2 * nad + neq
        floor_us = dfma / (per_clk * sms * mhz * 1e6) * 1e6
        # the pipe's nominal rate (2 per clock per SM: what ncu counts as
        # 100 % busy) gives the hard floor; the probe reaches 84 % of it
        nominal_us = dfma / (2.0 * sms * mhz * 1e6) * 1e6
        fp64_floor = {"dfma_per_launch": dfma, "dfma_per_clock_per_sm_probe": per_clk,
                      "probe_fma_per_s": fma_rate, "sms": sms,
                      "sm_mhz": mhz, "floor_us_probe": floor_us,
                      "floor_frac_of_hbm_probe": spmv_bytes / (floor_us * 1e-6) / 1e9 / peak,
                      "frac_of_floor_probe": floor_us / (spmv_ms * 1e3),
                      "floor_us_nominal": nominal_us,
                      "floor_frac_of_hbm_nominal": spmv_bytes / (nominal_us * 1e-6) / 1e9 / peak,
                      "frac_of_floor_nominal": nominal_us / (spmv_ms * 1e3)}

    out = None
    if dist.rank == 0:
        n = dist.ws
        value = n * 1000.0 / ms_step
        out = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": n,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (structured mesh generated in-process)",
            "config": bench_config(neq, nad, n), "colors": ncolors,
            "time_to_tol_ms": ms_step, "pcg_iters": iters, "assembly_ms": asm_ms,
            "pcg_ms": pcg_ms, "pcg_iter_gbs": iter_gbs, "spmv_ms": spmv_ms,
            "spmv_gbs": spmv_gbs, "wall_s": wall,
            "roofline": {"bound": "hbm",
                         "kernel": "sell_spmv_kernel<double> (FP64 sliced node-block SpMV + fused (p, Kp))",
                         "achieved": spmv_gbs, "peak": peak, "unit": "GB/s",
                         "frac": spmv_gbs / peak, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": spmv_bytes,
                         "traffic": profiled("traffic_bytes_per_launch"),
                         "fp64_pipe_frac_ncu": profiled("fp64_pipe_frac"),
                         "fp64_floor": fp64_floor},
            "mixed": {"ms_per_step": mixed_step, "solves_per_s": n * 1000.0 / mixed_step,
                      "speedup_vs_fp64": ms_step / mixed_step,
                      "pcg_ms": statistics.median(mixed_pcg_ms),
                      "pcg_speedup_vs_fp64": pcg_ms / statistics.median(mixed_pcg_ms),
                      "pcg_iters": minfo["iters"], "refinements": minfo["refinements"],
                      "rel_err_vs_fp64": float(np.abs(xm - x64).max() / np.abs(x64).max()),
                      "norm_m_r": minfo["norm_m_r"], "conv": minfo["conv"],
                      "spmv32_ms": spmv32_ms,
                      "spmv32_gbs": spmv32_bytes / (spmv32_ms * 1e-3) / 1e9,
                      "spmv32_frac": spmv32_bytes / (spmv32_ms * 1e-3) / 1e9 / peak},
            "e2e": {"value": n / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "device_bytes": device_bytes,
            "csrc_bytes": 8 * (nad + neq) + 4 * (nad + neq + 1),
            "clocks": clk,
        }
        if n == 1 and not args.no_cpu_baseline:
            import oracle as O
            s_o = O.structure(mesh, True)
            b0_o, u0_o = O.loads(mesh, s_o)
            out["cpu_baseline"] = cpu_baseline(mesh, s_o, b0_o, u0_o, keep=True)
            # the FP64 and mixed solutions against the oracle's pcg_omp solve
            # (the same equations: the structures are the same bit for bit)
            x_o = out["cpu_baseline"].pop("_x")
            same = all(np.array_equal(a, b) for a, b in
                       ((s_o.perm, st.perm), (s_o.id, st.id), (s_o.ia, st.ia), (s_o.ja, st.ja)))
            rel = lambda a: float(np.abs(a - x_o).max() / np.abs(x_o).max())
            out["parity_vs_oracle"] = {
                "structure_bit_exact": same, "oracle_pcg_iters": out["cpu_baseline"]["pcg_iters"],
                "gpu_pcg_iters": iters, "rel_err_fp64": rel(x64), "rel_err_mixed": rel(xm),
                "bars": ("FP64 <= 1e-9 with iterations +-2 at tol 1e-8 (the oracle's own "
                         "pcg_omp moves by 4.4e-10 between 8 and 5 threads here); mixed <= 1e-7")}
            # the oracle's stress recovery (one host thread) on the same u,
            # and how far the device's nodal stresses are from it
            t = time.perf_counter()
            t_o = O.tform(mesh, u_sol)
            nxt["stress_cpu_oracle_ms"] = 1e3 * (time.perf_counter() - t)
            nxt["stress_cpu_cores"] = 1
            nxt["stress_max_rel_diff_vs_oracle"] = float(
                np.abs(t_o - stresses).max() / np.abs(t_o).max())
            # the oracle's writer (one host thread) on the same u and stresses
            ref_path = os.path.join(vtk_dir, "ref.vtu")
            t = time.perf_counter()
            O.write_mesh_res(ref_path, mesh, u_sol, stresses, 0)
            nxt["vtk_cpu_oracle_ms"] = 1e3 * (time.perf_counter() - t)
            with open(vtk_path, "rb") as a, open(ref_path, "rb") as b:
                nxt["vtk_identical_to_oracle"] = a.read() == b.read()
        out["after_solve"] = nxt
    import shutil
    shutil.rmtree(vtk_dir, ignore_errors=True)
    ctx.close()
    return out


def run_spmv_only(args):
    """Assemble the workload once, then time `steps` SpMVs (after `warmup`)."""
    import torch

    import elastic_gb300 as E

    mesh = make_workload()
    ctx = E.Context(device=0)
    ctx.set_mesh(mesh)
    neq, nad, _ = ctx.build_structure(True)
    st = ctx.structure()
    b0, u0 = E.pload(mesh, st.id)
    ctx.set_state(u0, b0)
    ctx.assemble_resident()
    try:  # a short solve leaves a non-trivial search direction p behind
        ctx.solve_resident(tol=1e-2, maxit=50)
    except E.ElasticError:
        pass
    ext = torch.cuda.ExternalStream(ctx.stream, device=0)
    prec = E.PREC_MIXED if args.precision == "mixed" else E.PREC_FP64
    ctx.spmv_resident(precision=prec, reps=args.warmup)
    torch.cuda.synchronize(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    ctx.spmv_resident(precision=prec, reps=args.steps)
    e1.record(ext)
    torch.cuda.synchronize(0)
    ms = e0.elapsed_time(e1) / args.steps
    byts = 12 * nad + 28 * neq if prec == E.PREC_FP64 else 8 * nad + 16 * neq
    peak, kind = measured_peak()
    ctx.close()
    return {"mode": "spmv", "precision": args.precision, "neq": neq, "nad": nad, "spmv_ms": ms,
            "spmv_gbs": byts / (ms * 1e-3) / 1e9, "frac": byts / (ms * 1e-3) / 1e9 / peak,
            "peak": peak, "peak_kind": kind}


def run_block(args):
    """Batched load cases (the 96x96x48 HEXA8 plate, 16 cases of N(0,1) top-face
    forces, tol 1e-8): block PCG with the autotuned width (FP32 inner, FP64
    replacements) against single-RHS FP64 PCG solves, both on the device."""
    import torch

    import elastic_gb300 as E
    from elastic_gb300 import meshgen as M

    mesh, F = M.plate_hexa8_96(16)
    ctx = E.Context(device=0)
    ctx.set_mesh(mesh)
    neq, nad, _ = ctx.build_structure(True)
    st = ctx.structure()
    B = np.zeros((neq, 16), order="F")
    free = st.id > 0
    for c in range(16):
        B[st.id[free] - 1, c] = F[c][free]
    ctx.assemble(None, None)
    width, tt = ctx.autotune_block(E.PREC_MIXED, remeasure=True)
    tiling = ctx.block_tiling(E.PREC_MIXED)
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dX = torch.zeros_like(dB)
    ext = torch.cuda.ExternalStream(ctx.stream, device=0)
    times = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        infos = ctx.solve_block_device(dB.data_ptr(), dX.data_ptr(), 16,
                                       precision=E.PREC_MIXED, tol=TOL, maxit=MAXIT)
        e1.record(ext)
        torch.cuda.synchronize()
        if k >= args.warmup:
            times.append(e0.elapsed_time(e1))
    X = dX.cpu().numpy().T
    ms = statistics.median(times)
    # single-RHS FP64 PCG on two of the cases, timed the same way, and the
    # oracle's FP64 pcg_omp of the same two cases on this host's cores
    import oracle as O
    nth = len(os.sched_getaffinity(0))
    s = O.Structure(perm=st.perm, id=st.id, neq=st.neq, nad=st.nad, ia=st.ia, ja=st.ja)
    ad_o, al_o, _ = O.assemble_omp(mesh, s, np.zeros((mesh.nnode, mesh.ndf)), np.zeros(neq),
                                   nthreads=nth)
    single, err_block, err_single, o_iters, o_s = [], {}, {}, {}, []
    for c in range(2):
        ctx.solve(B[:, c], tol=TOL, maxit=MAXIT)  # warm
        t = time.perf_counter()
        x, info = ctx.solve(B[:, c], tol=TOL, maxit=MAXIT)
        single.append((time.perf_counter() - t) * 1000.0)
        x_o, i_o = O.pcg_omp(s, ad_o, al_o, B[:, c], tol=TOL, maxit=MAXIT, nthreads=nth)
        o_s.append(i_o["seconds"])
        o_iters[str(c)] = [i_o["iters"], info["iters"]]
        rel = lambda a: float(np.abs(a - x_o).max() / np.abs(x_o).max())
        err_block[str(c)] = rel(X[:, c])
        err_single[str(c)] = rel(x)
    its = [i["iters"] for i in infos]
    ctx.close()
    single_ms = statistics.mean(single)
    # the block product's roofline: FP32 algorithmic bytes of one product of
    # the autotuned width (8 nad + 8 neq + 8 W neq) over its timed launch
    peak, peak_kind = measured_peak()
    w_us = dict(zip([1, 2, 4, 8, 16], tt))[width]
    spmm_bytes = 8 * nad + 8 * neq + 8 * width * neq
    spmm_gbs = spmm_bytes / (w_us * 1e-6) / 1e9
    return {"mode": "block", "workload": "HEXA8 plate 96x96x48, 16 load cases, tol 1e-8",
            "spmm_roofline": {"kernel": f"sell_spmm_kernel<float, 3, {width}>",
                              "bound": "hbm", "achieved": spmm_gbs, "peak": peak,
                              "unit": "GB/s", "frac": spmm_gbs / peak, "peak_kind": peak_kind,
                              "algorithmic_bytes_per_launch": spmm_bytes, "us": w_us,
                              "traffic": profiled("traffic_bytes_per_launch",
                                                  "sell_spmm_fp32_w16_hexa8_plate96.md")
                              if width == 16 else None},
            "neq": neq, "nad": nad, "block_width": width,
            "spmm32_us_by_width": dict(zip(["1", "2", "4", "8", "16"], np.round(tt, 1).tolist())),
            "spmm32_groups_in_flight_by_width": dict(zip(["1", "2", "4", "8", "16"], tiling)),
            "ms_16_cases": ms, "ms_per_case": ms / 16, "iters_min_max": [min(its), max(its)],
            "replacements": infos[0]["refinements"],
            "single_fp64_ms_per_case": single_ms,
            "speedup_per_case_vs_single_fp64": single_ms / (ms / 16),
            "rel_err_block_mixed_vs_oracle_by_case": err_block,
            "rel_err_single_fp64_vs_oracle_by_case": err_single,
            "oracle_vs_single_fp64_iters_by_case": o_iters,
            "oracle_pcg_omp_s_per_case": statistics.mean(o_s), "oracle_cores": nth}


def run_fp64peak(args):
    """The FP64 pipe's FMA rate (the library's register-only probe kernel),
    the denominator of the FP64 product's floor."""
    import torch

    import elastic_gb300 as E

    p = torch.cuda.get_device_properties(0)
    E.fp64_fma_rate(0)  # warm
    clocks = ClockSampler(0)
    clocks.start()
    runs = [E.fp64_fma_rate(0) for _ in range(max(args.steps, 8))]
    clk = clocks.stop()
    rate = max(r for r, _ in runs)
    out = {"mode": "fp64peak", "fma_per_s": rate, "tflops": 2 * rate / 1e12,
           "fma_per_clock_per_sm_at_max_clock": max(c for _, c in runs),
           "sms": p.multi_processor_count, "clocks": clk}
    if clk and clk.get("sm_mhz"):
        out["fma_per_clock_per_sm_at_sampled_clock"] = (
            rate / (p.multi_processor_count * clk["sm_mhz"] * 1e6))
    return out


def run_spmm(args):
    """The block products of the 96x96x48 plate alone: the autotuner's times
    of every width (FP32 and FP64, with the fused dots), for profiling."""
    import elastic_gb300 as E
    from elastic_gb300 import meshgen as M

    mesh, _ = M.plate_hexa8_96(16)
    ctx = E.Context(device=0)
    ctx.set_mesh(mesh)
    neq, nad, _ = ctx.build_structure(True)
    ctx.assemble(None, None)
    out = {"mode": "spmm", "neq": neq, "nad": nad}
    for _ in range(max(1, args.steps)):
        for name, prec in (("fp32", E.PREC_MIXED), ("fp64", E.PREC_FP64)):
            w, tt = ctx.autotune_block(prec, remeasure=True)
            out[name] = {"width": w, "us_by_width": dict(zip(["1", "2", "4", "8", "16"],
                                                             np.round(tt, 1).tolist())),
                         "groups_in_flight_by_width": dict(zip(["1", "2", "4", "8", "16"],
                                                               ctx.block_tiling(prec)))}
    ctx.close()
    return out


def run_tetra(args):
    """The TETRA4 mesh of a 48^3 cube (6 tetrahedra per hex, interior nodes
    jittered, one lognormal E and uniform nu per element: 345,744 equations),
    z=0 fixed, unit pressure on z=1, tol 1e-10: FP64 PCG and the mixed-
    precision solver on the device (assembly excluded, CUDA events), each
    solution against the oracle's FP64 pcg_omp solve on this host's cores
    (timed: the CPU baseline of this mesh)."""
    import torch

    import elastic_gb300 as E
    import oracle as O
    from elastic_gb300 import meshgen as M

    tol = 1e-10
    mesh = M.cube_tetra4_48_mixed()
    ctx = E.Context(device=0)
    ctx.set_mesh(mesh)
    neq, nad, _ = ctx.build_structure(True)
    st = ctx.structure()
    b0, u0 = E.pload(mesh, st.id)
    ctx.set_state(u0, b0)
    ctx.assemble_resident()
    ext = torch.cuda.ExternalStream(ctx.stream, device=0)

    def timed(prec):
        ms, info = [], None
        for k in range(args.warmup + args.steps):
            e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
            e0.record(ext)
            info = ctx.solve_resident(precision=prec, tol=tol, maxit=MAXIT)
            e1.record(ext)
            torch.cuda.synchronize(0)
            if k >= args.warmup:
                ms.append(e0.elapsed_time(e1))
        return statistics.median(ms), info, ctx.solution()

    ms64, i64, x64 = timed(E.PREC_FP64)
    msm, im, xm = timed(E.PREC_MIXED)
    ctx.close()
    # the oracle's FP64 solve on the same equations (numbering, ia/ja identical)
    nth = len(os.sched_getaffinity(0))
    s = O.Structure(perm=st.perm, id=st.id, neq=st.neq, nad=st.nad, ia=st.ia, ja=st.ja)
    ad, al, b = O.assemble_omp(mesh, s, u0, b0, nthreads=nth)
    xo, io = O.pcg_omp(s, ad, al, b, tol=tol, maxit=MAXIT, nthreads=nth)
    rel = lambda a, ref: float(np.abs(a - ref).max() / np.abs(ref).max())
    return {"mode": "tetra",
            "workload": ("TETRA4 of a 48^3 cube (6 per hex), jittered interior nodes, lognormal E "
                         "per element, z=0 fixed, unit pressure on z=1, RCM, tol 1e-10"),
            "neq": neq, "nad": nad,
            "fp64": {"pcg_ms": ms64, "iters": i64["iters"]},
            "mixed": {"pcg_ms": msm, "inner_iters": im["iters"],
                      "refinements": im["refinements"], "speedup_vs_fp64": ms64 / msm},
            "rel_err_fp64_vs_oracle": rel(x64, xo), "rel_err_mixed_vs_oracle": rel(xm, xo),
            "rel_err_mixed_vs_fp64": rel(xm, x64),
            "cpu_baseline": {"value": 1.0 / io["seconds"], "unit": "solves/s (PCG only)",
                             "cores": nth, "kind": "port", "iters": io["iters"],
                             "sample": "the full pcg_omp solve (matvec_csrcsym_omp)"}}


def run_serve(args):
    """The served stream: N requests (box meshes of the four element types,
    2k-2M dofs log-uniform, 1-8 load cases, tol 1e-8) with Poisson arrivals at
    1.5x the sequential service rate, through the solve server with a 150 GB
    admission budget, against the same stream solved one request at a time
    with plain FP64 PCG (library single solves; its latencies follow from the
    measured service times and the arrival times, a FIFO queue)."""
    import threading

    import elastic_gb300 as E
    from elastic_gb300 import meshgen as M

    rng = np.random.default_rng(20261203)
    n = args.requests
    reqs = [M.serving_request(rng, dof_max=args.max_dof) for _ in range(n)]
    cases = sum(F.shape[0] for _, F in reqs)
    # ---- sequential plain FP64 (service time per request, back to back);
    # with --rate the arrival rate is given and this half is left out
    service, ref_u = [], {}
    for i, (m, F) in enumerate(reqs if not getattr(args, "rate", None) else []):
        t0 = time.perf_counter()
        ctx = E.Context(device=0)
        ctx.set_mesh(m)
        ctx.build_structure(True)
        st = ctx.structure()
        ctx.assemble(None, None)
        free = st.id > 0
        us = []
        for k in range(F.shape[0]):
            b = np.zeros(st.neq)
            b[st.id[free] - 1] = F[k][free]
            x, _ = ctx.solve(b, tol=TOL, maxit=MAXIT)
            if i % 8 == 0:
                u = np.zeros_like(F[k])
                u[free] = x[st.id[free] - 1]
                us.append(u)
        ctx.close()
        service.append(time.perf_counter() - t0)
        if us:
            ref_u[i] = np.array(us)
    rate = args.rate if getattr(args, "rate", None) else 1.5 / statistics.mean(service)
    arrivals = np.cumsum(np.random.default_rng(7).exponential(1.0 / rate, n))
    arrivals -= arrivals[0]
    t, lat_seq = 0.0, []
    for a, sv in zip(arrivals, service):
        t = max(t, a) + sv
        lat_seq.append(t - a)
    seq_span = t
    # ---- served
    srv = E.Server(device=0, hbm_budget=int(150e9), prep_threads=len(os.sched_getaffinity(0)),
                   large_workers=getattr(args, "large_workers", 0))
    tickets = [None] * n
    t_start = time.perf_counter() + 0.5

    def submitter():
        for i, (m, F) in enumerate(reqs):
            dt = t_start + arrivals[i] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            tickets[i] = (srv.submit(m, F, tol=TOL, maxit=MAXIT), time.perf_counter())

    th = threading.Thread(target=submitter)
    th.start()
    lat, done_at, errs, bad, served_u = [], [], [], 0, {}
    for i in range(n):
        while tickets[i] is None:
            time.sleep(0.001)
        tk, t_sub = tickets[i]
        U, infos, latency, status = srv.wait(tk, timeout=3600)
        bad += status != 0
        lat.append(latency)
        done_at.append(t_sub - t_start + latency)
        if i in ref_u:
            errs.append(float(np.abs(U - ref_u[i]).max() / max(np.abs(ref_u[i]).max(), 1e-300)))
        if i % 8 == 0:
            served_u[i] = U
    th.join()
    stats = srv.stats()
    sat_span = None
    if args.all_at_once:
        # the same requests all at once (a closed batch): the server's capacity
        t0 = time.perf_counter()
        tks = [srv.submit(m, F, tol=TOL, maxit=MAXIT) for m, F in reqs]
        for tk in tks:
            srv.wait(tk, timeout=3600)
        sat_span = time.perf_counter() - t0
    srv.close()
    # sampled served results against the oracle's FP64 solves (pcg_omp on this
    # host's cores, the oracle's own structure and assembly): requests of up
    # to 3e5 dofs among the sampled ones; the packed loop solves them in FP64
    # (<= 1e5 dofs), the block solver in mixed precision for 3-D meshes above
    import oracle as O
    nth = len(os.sched_getaffinity(0))
    err_o = {"fp64_packed": [], "block": []}
    for i in sorted(served_u) if not getattr(args, "quick", False) else []:
        m, F = reqs[i]
        if m.nnode * m.ndf > 3e5:
            continue
        s = O.structure(m, True)
        ad, al, _ = O.assemble_omp(m, s, np.zeros((m.nnode, m.ndf)), np.zeros(s.neq),
                                   nthreads=nth)
        free = s.id > 0
        for k in range(F.shape[0]):
            b = np.zeros(s.neq)
            b[s.id[free] - 1] = F[k][free]
            x, _ = O.pcg_omp(s, ad, al, b, tol=TOL, maxit=MAXIT, nthreads=nth)
            u = np.zeros_like(F[k])
            u[free] = x[s.id[free] - 1]
            d = float(np.abs(served_u[i][k] - u).max() / max(np.abs(u).max(), 1e-300))
            err_o["block" if s.neq >= 1e5 else "fp64_packed"].append(d)
    span = max(done_at)
    pct = lambda v, q: float(np.percentile(np.array(v), q))
    return {"mode": "serve", "requests": n, "load_cases": cases,
            "dof_range": [2e3, args.max_dof], "arrival_rate_per_s": rate,
            "served": {"solves_per_s": cases / span, "requests_per_s": n / span,
                       "p50_latency_s": pct(lat, 50), "p99_latency_s": pct(lat, 99),
                       "span_s": span, "failed": int(bad),
                       "peak_device_bytes": stats["peak_bytes"],
                       "peak_load_cases_in_pack": stats["peak_slots"],
                       "packed_iterations": stats["iterations"],
                       "phases_mean_s": {k: stats[f"{k}_phases_mean_s"]
                                         for k in ("packed", "block")},
                       "all_at_once_solves_per_s": cases / sat_span if sat_span else None},
            "sequential_fp64": {"solves_per_s": cases / seq_span, "requests_per_s": n / seq_span,
                                "p50_latency_s": pct(lat_seq, 50),
                                "p99_latency_s": pct(lat_seq, 99), "span_s": seq_span,
                                "mean_service_s": statistics.mean(service)} if service else None,
            "max_rel_diff_vs_sequential_sample": max(errs) if errs else None,
            "vs_oracle_fp64": {
                "requests": sum(1 for i in served_u if reqs[i][0].nnode * reqs[i][0].ndf <= 3e5),
                "load_cases": {k: len(v) for k, v in err_o.items()},
                "max_rel_err": {k: (max(v) if v else None) for k, v in err_o.items()},
                "bars": ("tol 1e-8: packed FP64 <= 1e-8 (the oracle's own pcg_omp moves by up to "
                         "1.5e-9 between thread counts at this tolerance); block (mixed for "
                         "3-D) <= 1e-6")}}


# ------------------------------------------------------------------ CPU side
def cpu_model() -> str:
    """The host CPU's model name (lscpu), with the logical CPUs this process
    may use."""
    name = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return f"{name or 'unknown'} ({len(os.sched_getaffinity(0))} logical CPUs usable)"


def bench_config(neq, nad, n_ranks):
    """The workload description both arms print (the same keys and values)."""
    return {"workload": WORKLOAD, "neq": neq, "nad": nad, "tol": TOL,
            "parallelism": "replicas" if n_ranks > 1 else "single",
            "l2": "inputs larger than L2 (CSRC matrix 400 MB + vectors > 129 MB L2)"}


def cpu_baseline(mesh, s, b0, u0, nthreads=None, sequential=True, keep=False):
    """The reference's OpenMP CPU path (oracle restatement of pform_mec's
    colour loop and pcg_omp with matvec_csrcsym_omp) on this host's cores:
    one full assembly and one full PCG solve, timed; with `sequential`, also
    the one-thread path (pform_mec's element loop, matvec_csrcsym1, pcg);
    with `keep`, the OpenMP solve's x under "_x"."""
    import oracle as O

    nth = nthreads or len(os.sched_getaffinity(0))
    colors = O.colormsh(mesh)
    t = time.perf_counter()
    ad, al, b = O.assemble_omp(mesh, s, u0, b0, nthreads=nth, colors=colors)
    t_asm = time.perf_counter() - t
    x_o, info = O.pcg_omp(s, ad, al, b, tol=TOL, maxit=MAXIT, nthreads=nth)
    t_pcg = info["seconds"]
    total = t_asm + t_pcg
    out = {"value": 1.0 / total, "unit": "solves/s", "cores": nth, "kind": "port",
           "cpu": cpu_model(),
           "sample": f"one full OpenMP assembly + one full pcg_omp solve ({info['iters']} "
                     "iterations), no extrapolation",
           "seconds_per_solve": total, "assembly_s": t_asm, "pcg_s": t_pcg,
           "pcg_iters": info["iters"]}
    if sequential:
        t = time.perf_counter()
        O.assemble(mesh, s, u0, b0)
        t_asm1 = time.perf_counter() - t
        _, info1 = O.pcg(s, ad, al, b, tol=TOL, maxit=MAXIT)
        out["sequential_1thread"] = {
            "value": 1.0 / (t_asm1 + info1["seconds"]), "unit": "solves/s", "cores": 1,
            "assembly_s": t_asm1, "pcg_s": info1["seconds"], "pcg_iters": info1["iters"],
            "sample": "one full assembly + one full pcg solve on one thread"}
    if keep:
        out["_x"] = x_o  # the solution (the caller's parity check; not printed)
    return out


def run_reference(args, dist: Dist):
    """--impl reference: the reference's CPU implementation of the path (the
    oracle port, with its own structure: graph, RCM, numeq, csrstruct; then
    per step the OpenMP assembly and the full pcg_omp solve) on this host's
    cores.  Under torchrun only rank 0 runs."""
    if dist.rank != 0:
        return None
    import oracle as O

    mesh = make_workload()
    s = O.structure(mesh, True)
    b0, u0 = O.loads(mesh, s)
    nth = len(os.sched_getaffinity(0))
    per_step, iters = [], None
    for k in range(args.warmup + args.steps):
        r = cpu_baseline(mesh, s, b0, u0, nthreads=nth, sequential=False)
        iters = r["pcg_iters"]
        if k >= args.warmup:
            per_step.append(r["seconds_per_solve"])
    sec = statistics.median(per_step)
    value = 1.0 / sec
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": dist.ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1000.0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (structured mesh generated in-process)",
        "config": bench_config(s.neq, s.nad, dist.ws),
        "pcg_iters": iters,
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nth, "kind": "port",
                         "cpu": cpu_model(),
                         "sample": ("per step: one full OpenMP assembly + one full pcg_omp "
                                    f"solve ({iters} iterations); median of {args.steps} steps "
                                    f"after {args.warmup}")},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="full mode: skip the block, tetra and serve sub-benchmarks")
    ap.add_argument("--mode", choices=["full", "spmv", "spmm", "block", "tetra", "serve",
                                       "fp64peak"],
                    default="full",
                    help="spmv: only the SpMV of the workload (for profiling); spmm: only the "
                         "block products of the 96x96x48 plate (profiling); block: 16 load "
                         "cases on the 96x96x48 plate; tetra: FP64 and mixed PCG on the "
                         "48^3 TETRA4 mesh; serve: the served request stream")
    ap.add_argument("--requests", type=int, default=512, help="serve: requests in the stream")
    ap.add_argument("--max-dof", type=float, default=2e6, help="serve: largest request")
    ap.add_argument("--rate", type=float, default=None,
                    help="serve: arrival rate in requests/s (leaves out the sequential "
                         "FP64 half, whose mean service time sets the rate otherwise)")
    ap.add_argument("--large-workers", type=int, default=0,
                    help="serve: block-solve worker threads (0: the server's default, 2)")
    ap.add_argument("--quick", action="store_true",
                    help="serve: the open stream only (no all-at-once submission of the same "
                         "requests, no oracle check of the served results)")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64",
                    help="solver precision (mixed: FP32 inner PCG + FP64 refinement)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist = Dist(args.impl)
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        elif args.mode == "spmv":
            out = run_spmv_only(args)
        elif args.mode == "block":
            out = run_block(args)
        elif args.mode == "spmm":
            out = run_spmm(args)
        elif args.mode == "fp64peak":
            out = run_fp64peak(args)
        elif args.mode == "tetra":
            out = run_tetra(args)
        elif args.mode == "serve":
            args.all_at_once = not args.quick
            out = run_serve(args)
        else:
            out = run_ours(args, dist)
            if out is not None and dist.ws == 1 and not args.no_extras:
                # the other headline workloads at their own sizes: block, tetra
                # and the served stream (512 requests, 2k-2M dofs; --mode serve
                # also measures the same requests submitted all at once)
                # (a failure in one of them is recorded in its sub-object and
                # the line is still printed)
                blk = argparse.Namespace(**vars(args))
                blk.steps, blk.warmup = 3, 3
                srv = argparse.Namespace(**vars(args))
                srv.all_at_once = False
                for key, fn, a in (("block", run_block, blk), ("tetra", run_tetra, blk),
                                   ("serve", run_serve, srv)):
                    try:
                        out[key] = fn(a)
                    except Exception as e:  # noqa: BLE001 -- reported, not hidden
                        out[key] = {"error": f"{type(e).__name__}: {e}"}
                        print(f"bench: {key} failed: {e}", file=sys.stderr)
    finally:
        dist.close()
    if out is not None and dist.rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
