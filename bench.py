"""Benchmark of the finite-volume hot path on GB300.

Workload: the 2,097,152-cell 3D channel with a bump, coupled (u, v, w, p) + k-omega SST
(``aquaflux_gb300.workloads.channel3d(128)``: 6,340,608 faces, seeded bump / jitter, randomly
permuted then RCM-renumbered cells).  One step (default ``--step vjp``) = one evaluation of the
residual and its vector-Jacobian product (hand-written adjoint kernels) at a fixed state;
``--step jvp`` times the residual + Jacobian-vector product (dual numbers) instead, and
``--step jvp-linearised`` the Newton solve's Krylov operator (the product at a held
linearisation).  ``value`` is faces processed per second (Gfaces/s) with inputs resident in HBM;
``e2e`` is the same step through the C ABI with host (pinned) inputs / outputs copied inside the
timed region.

``--impl reference`` times the reference algorithm on the host CPU instead (the float64 CPU
oracle restating the reference's residual, autograd JVP, all host threads) on a bounded sample of
the same workload.

The line also carries the Newton block (each preconditioner in fp64, fp32 and fp32 + fp32
tangents), the adjoint objectives, the CPU baseline, and ``cpu_ilu``: the reference's compiled
ILU(0) kernel (built from its source; its plain-C restatement where that build is absent; one
core) timed beside the GPU's fp64 ILU(0) on a 48^3 Jacobian.

Run: ``python bench.py [--gpus N] [--steps K] [--warmup W] [--size 128]``.  Profiling modes
(one JSON line each): ``--newton-only KIND:PREC:TANGENTS`` (one Newton solve inside the NVTX
range "newton"), ``--vcycle-only PREC`` (the AMG V-cycle, one inside the NVTX range "vcycle").
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton-solve s & residual+VJP Gfaces/s at 2M cells: FP32-precond vs FP64, 1 GB300"
UNIT = "Gfaces/s"
STEP_DESC = {"vjp": "residual + VJP (hand-written adjoint) at a fixed state",
             "jvp": "residual + JVP (dual numbers) at a fixed state",
             "jvp-linearised": "JVP at a held linearisation, the held residual copied out (the "
                               "Newton solve's Krylov operator: fv_linearise once, then "
                               "fv_jvp_linearised)"}
CLOCK_QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=128, help="cells per axis of the 3D channel")
    ap.add_argument("--cpu-sample", type=int, default=40,
                    help="cells per axis of the CPU sample (a reference-arm step)")
    ap.add_argument("--no-reference-full-size", dest="reference_full_size", action="store_false",
                    help="skip the reference arm's one full-size CPU evaluation")
    ap.add_argument("--ilu-sample", type=int, default=48,
                    help="cells per axis of the ILU(0) CPU-vs-GPU sample (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--step", default="vjp", choices=["vjp", "jvp", "jvp-linearised"])
    ap.add_argument("--cell-order", default="coherent", choices=["coherent", "natural"],
                    help="thread-to-cell order of the cell stages (fv_case_set_cell_order): "
                         "grouped by face-list pattern (default) or the mesh's natural order")
    ap.add_argument("--no-newton", action="store_true", help="skip the Newton-solve timing")
    ap.add_argument("--newton-kinds", default="amg,ilu",
                    help="preconditioners timed in the Newton block (comma list of amg (fine "
                         "order by dimension: coloured in 3D), amg-natural, amg-colour, ilu)")
    ap.add_argument("--workload", default="channel3d", choices=["channel3d", "batched"],
                    help="channel3d: the 128^3 SST channel (the headline); batched: the 64-instance "
                         "calibration sweep (its own JSON line)")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the adjoint objectives' gradients after the Newton solves")
    ap.add_argument("--no-newton-oracle", action="store_true",
                    help="skip the CPU oracle's residual of the converged Newton states")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched sweep's residual + VJP timing (graph vs persistent)")
    ap.add_argument("--no-harder-start", action="store_true",
                    help="skip the nu = 2.5e-4 channel (direct Newton beside Reynolds continuation)")
    ap.add_argument("--no-config1", action="store_true",
                    help="skip the config-1 cavity Newton solve (GPU beside the CPU oracle)")
    ap.add_argument("--newton-only", default=None, metavar="KIND:PREC:TANGENTS",
                    help="run one Newton solve of that form (e.g. amg:32:32) on the channel and "
                         "print its timings only (for profiling the solve's kernels)")
    ap.add_argument("--vcycle-only", default=None, metavar="PREC", type=int, choices=[32, 64],
                    help="time the AMG V-cycle of that precision on the channel's plug-flow "
                         "Jacobian and run one more in an NVTX range \"vcycle\" (for profiling)")
    return ap.parse_args()


def run_newton_only(args) -> dict:
    """One Newton solve of the given form on the --size channel after one warm-up solve on a 16^3
    channel (library initialisation), with no other GPU work in the process."""
    import torch

    from aquaflux_gb300 import solve, workloads

    kind, prec, tan = args.newton_only.split(":")
    warm = workloads.channel3d(16)
    solve.newton_solve(warm.device_case(), warm.initial_state(), kind=kind, precision=int(prec),
                       tangents=int(tan))
    wl = workloads.channel3d(args.size)
    case = wl.device_case()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("newton")  # the profiled region (ncu --nvtx-include "newton/")
    res = solve.newton_solve(case, wl.initial_state(), kind=kind, precision=int(prec),
                             tangents=int(tan))
    torch.cuda.nvtx.range_pop()
    return {"newton_only": args.newton_only, "cells": wl.mesh.n_cells, "seconds": res.seconds,
            "converged": res.converged, "newton_steps": res.steps,
            "krylov_iterations": res.krylov_iterations,
            "phase_seconds": {k: round(v, 4) for k, v in res.phase_seconds.items()}}


def run_vcycle_only(args) -> dict:
    """The AMG preconditioner (coloured fine order, the Newton default in 3D) of the --size
    channel's plug-flow Jacobian: per-level sizes, the V-cycle's time (CUDA events over 20 graph
    replays after 3 warm-up applications), then one eager V-cycle in the NVTX range "vcycle"."""
    import torch

    from aquaflux_gb300 import workloads
    from aquaflux_gb300.amg import AmgPreconditioner
    from aquaflux_gb300.solve import BlockJacobian

    prec = args.vcycle_only
    wl = workloads.channel3d(args.size)
    case = wl.device_case()
    s = torch.tensor(wl.initial_state(noise=0.02), device="cuda")
    pc = AmgPreconditioner(BlockJacobian(case, precision=prec), prec)
    pc.refresh(s)
    r = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(0))
    for _ in range(3):
        pc.apply(r)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        pc.apply(r)
    e1.record()
    torch.cuda.synchronize()
    pc.graph = False
    torch.cuda.nvtx.range_push("vcycle")  # the profiled region (ncu --nvtx-include "vcycle/")
    y = pc.apply(r)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    return {"vcycle_only": prec, "cells": wl.mesh.n_cells, "levels": pc.h.sizes,
            "blocks": [lv.nnzb for lv in pc.h.levels], "ms_per_vcycle": e0.elapsed_time(e1) / 20,
            "finite": bool(torch.isfinite(y).all())}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """``nvidia-smi`` sampled every 200 ms while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            with open(self.path, "w") as out:  # the child keeps its own descriptor
                self.proc = subprocess.Popen(
                    ["nvidia-smi", "-i", str(self.index), f"--query-gpu={CLOCK_QUERY}",
                     "--format=csv,noheader,nounits", "-lms", "200"],
                    stdout=out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        power = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(power) if power else None}


# ----------------------------------------------------------------------------- algorithmic bytes
def step_bytes_per_face(wl, step: str = "vjp") -> float:
    """Compulsory bytes of one residual + VJP (or residual + JVP) evaluation per face.

    Per face: owner + neighbour indices (8 B) and the area vector and centroid (2 dim 8 B).  Per
    cell: the state (n_f 8 B), centroid (dim 8 B), volume (8 B), wall distance (8 B, SST) in and
    the residual (n_f 8 B) out; the VJP (or JVP) adds its input vector (n_f 8 B) in and its result
    (n_f 8 B) out.  Each distinct value counted once.  On the 128^3 SST channel: 132.7 B/face.
    """
    m = wl.mesh
    dim, nf = m.dim, m.dim + (3 if wl.sst else 1)
    per_face = 8 + 2 * dim * 8
    per_cell = nf * 8 + dim * 8 + 8 + (8 if wl.sst else 0) + nf * 8 + 2 * nf * 8
    return per_face + per_cell * m.n_cells / m.n_faces


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ----------------------------------------------------------------------------- CPU reference
def cpu_residual_jvp_rate(size: int, min_seconds: float = 8.0, step: str = "vjp") -> dict:
    """Faces/s of the float64 CPU oracle (the reference algorithm restated; residual + autograd
    VJP or JVP) on a ``size^3`` sample of the channel workload, all host threads."""
    import numpy as np
    import torch

    from aquaflux_gb300 import workloads
    from oracle import fv_oracle as fo

    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    wl = workloads.channel3d(size, renumber="host")
    walls = wl.sst["walls"]
    case = fo.make_case(wl.mesh, mu=wl.mu, rho=wl.rho, flow_bc=wl.flow_bc,
                        sst={"nu": wl.mu / wl.rho, "walls": walls, "k": wl.sst["k"],
                             "omega": wl.sst["omega"]})
    orc = fo.Oracle(case)
    s = wl.initial_state(seed=1, noise=0.05)
    v = np.random.default_rng(2).standard_normal(s.size)
    def one():
        if step == "vjp":
            x = torch.as_tensor(s).requires_grad_(True)
            r = orc.residual(x)
            torch.autograd.grad(r, x, torch.as_tensor(v))
        else:
            orc.residual(torch.as_tensor(s))
            orc.jvp(s, v)

    one()  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        one()
        n += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    return {"faces_per_s": n * wl.mesh.n_faces / el, "cores": threads,
            "sample": f"{size}^3 channel ({wl.mesh.n_cells} cells, {wl.mesh.n_faces} faces), "
                      f"{n} residual+{step.upper()} evaluations in {el:.1f} s"}


def bsr_to_scalar_csr(blocks, indptr, indices):
    """``(indptr, indices, data)`` of the scalar CSR holding every entry of the BSR operator
    ``blocks`` (nnzb, b, b) on a sorted block pattern: scalar row ``i b + a`` holds entries
    ``(a, 0..b-1)`` of block row i's blocks, blocks in pattern order (the cell-major scalar layout
    the reference's ILU(0) kernel factors)."""
    import numpy as np

    b = blocks.shape[1]
    ip = np.asarray(indptr, dtype=np.int64)
    ix = np.asarray(indices, dtype=np.int64)
    k = np.diff(ip)
    data = np.empty(blocks.size, dtype=blocks.dtype)
    cols = np.empty(blocks.size, dtype=np.int32)
    for kk in np.unique(k):
        rows = np.flatnonzero(k == kk)
        q = ip[rows][:, None] + np.arange(kk)  # the rows' blocks, (m, kk)
        pos = ip[rows][:, None] * b * b + np.arange(kk * b * b)  # their scalar entries
        data[pos] = blocks[q].transpose(0, 2, 1, 3).reshape(len(rows), -1)
        c = ix[q][:, None, :, None] * b + np.arange(b)  # (m, 1, kk, b) scalar columns
        cols[pos] = np.broadcast_to(c, (len(rows), b, kk, b)).reshape(len(rows), -1)
    sptr = np.concatenate([[0], np.cumsum(np.repeat(k * b, b))]).astype(np.int32)
    return sptr, cols, data


def cpu_ilu0(sptr, scols, sdata, rhs) -> dict:
    """Factor + solve of the reference's own ILU(0) kernel (``aquaflux/solve/_ilu0.pyx`` built from
    its source into ``oracle/_ref`` by ``oracle/build_ref.py``; one core, the kernel is sequential)
    on a scalar CSR operator; where that build is absent, the plain-C restatement of the same
    kernel.  Factor, solution and which one ran are returned."""
    import ctypes

    import numpy as np

    from oracle.build_ref import load_ref

    mod = load_ref()
    if mod is not None:
        n = len(sptr) - 1
        diag = np.asarray(mod.diagonal_positions(sptr, scols, n))
        data = np.array(sdata, dtype=np.float64)
        t0 = time.perf_counter()
        mod.factor(sptr, scols, data, diag, n)
        t1 = time.perf_counter()
        x = np.array(rhs, dtype=np.float64)
        t2 = time.perf_counter()
        mod.solve(sptr, scols, data, diag, x, n)
        t3 = time.perf_counter()
        return {"factor_s": t1 - t0, "solve_s": t3 - t2, "factor": data, "x": x,
                "kind": "reference", "what": "the reference's compiled ILU(0) kernel "
                                             "(aquaflux/solve/_ilu0.pyx, built from its source)"}

    from oracle.build_oracle import build_c_oracle

    L = ctypes.CDLL(build_c_oracle())
    vp = ctypes.c_void_p

    def p(a):
        return a.ctypes.data_as(vp)

    n = len(sptr) - 1
    diag = np.zeros(n, dtype=np.int32)
    bad = ctypes.c_int(-1)
    if L.ilu0_diagonal_positions(p(sptr), p(scols), n, p(diag), ctypes.byref(bad)) != 0:
        raise ValueError(f"row {bad.value} stores no diagonal entry")
    data = np.array(sdata, dtype=np.float64)
    t0 = time.perf_counter()
    rc = L.ilu0_factor(p(sptr), p(scols), p(data), p(diag), n, ctypes.byref(bad))
    t1 = time.perf_counter()
    if rc != 0:
        raise ZeroDivisionError(f"ILU(0) met an exactly zero pivot at row {bad.value}")
    x = np.array(rhs, dtype=np.float64)
    t2 = time.perf_counter()
    L.ilu0_solve(p(sptr), p(scols), p(data), p(diag), p(x), n)
    t3 = time.perf_counter()
    return {"factor_s": t1 - t0, "solve_s": t3 - t2, "factor": data, "x": x, "kind": "port",
            "what": "plain-C restatement of the reference's ILU(0) kernel"}


def ilu_cpu_vs_gpu(size: int) -> dict:
    """The reference's ILU(0) factor + solve (its C restatement, one core; the kernel is
    sequential) beside the GPU's fp64 block ILU(0) on the same operator: the fp64 equilibrated
    cell-major Jacobian of a ``size^3`` sample of the channel at its plug-flow state.  Also checks
    that the two factors are bitwise equal."""
    import numpy as np
    import torch

    from aquaflux_gb300 import workloads
    from aquaflux_gb300.ilu0 import Ilu0
    from aquaflux_gb300.solve import BlockJacobian, ShiftedCellMajorOperator

    wl = workloads.channel3d(size)
    case = wl.device_case()
    state = torch.tensor(wl.initial_state(noise=0.02), device="cuda")
    jac = BlockJacobian(case)
    vals, _ = ShiftedCellMajorOperator(jac, equilibrate=True).assemble(jac.materialize(state))
    b = jac.b
    ilu = Ilu0.__new__(Ilu0)
    ilu._setup(jac.indptr, jac.indices, b, 64)
    r = torch.randn(jac.n * b, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(0))
    for _ in range(2):  # warm: the level schedules' graphs are captured on first use
        ilu.refactor(vals)
        x_gpu = ilu.solve(r)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ilu.refactor(vals)
    torch.cuda.synchronize()
    factor_ms = (time.perf_counter() - t0) * 1e3
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        x_gpu = ilu.solve(r)
    e1.record()
    torch.cuda.synchronize()
    solve_ms = e0.elapsed_time(e1) / 5
    blocks = vals.cpu().numpy().reshape(-1, b, b)
    sptr, scols, sdata = bsr_to_scalar_csr(blocks, jac.indptr, jac.indices)
    cpu = cpu_ilu0(sptr, scols, sdata, r.cpu().numpy())
    _, _, gfac = bsr_to_scalar_csr(ilu.factor_values().cpu().numpy().reshape(-1, b, b),
                                   jac.indptr, jac.indices)
    xg = x_gpu.cpu().numpy()
    return {"sample": f"{size}^3 channel, fp64 equilibrated cell-major Jacobian at the plug-flow "
                      f"state ({jac.n} cells, {jac.n * b} rows, {sdata.size} entries)",
            "cpu": {"factor_s": round(cpu["factor_s"], 4), "solve_s": round(cpu["solve_s"], 4),
                    "cores": 1, "kind": cpu["kind"], "what": cpu["what"]},
            "gpu_fp64": {"factor_ms": round(factor_ms, 3), "solve_ms": round(solve_ms, 3)},
            "factor_speedup": round(cpu["factor_s"] * 1e3 / factor_ms, 1),
            "solve_speedup": round(cpu["solve_s"] * 1e3 / solve_ms, 1),
            "factor_bitwise_equal": bool(np.array_equal(gfac, cpu["factor"])),
            "solve_max_rel_diff": float(np.abs(xg - cpu["x"]).max() / np.abs(cpu["x"]).max())}


# ----------------------------------------------------------------------------- GPU arm
def replica_throughput(ms: float, faces: int, steps: int, world: int, dist, device) -> tuple:
    """The replicas' timing contract: the slowest rank's time (max over ranks) and the whole job's
    throughput in Gfaces/s, every rank having processed `faces` faces per step (weak scaling, no
    data-path collective)."""
    import torch

    t = torch.tensor([ms], device=device, dtype=torch.float64)
    if dist is not None and world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t)
    return ms, world * faces * steps / (ms * 1e-3) / 1e9


def run_gpu(args, rank: int, world: int, local_rank: int) -> dict | None:
    import numpy as np
    import torch

    from aquaflux_gb300 import workloads

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    wl = workloads.channel3d(args.size)
    case = wl.device_case()
    n_cell_classes = case.set_cell_order(args.cell_order == "coherent")
    F = wl.mesh.n_faces
    state = torch.tensor(wl.initial_state(seed=rank, noise=0.05), device="cuda")
    vec = torch.tensor(np.random.default_rng(100 + rank).standard_normal(state.numel()),
                       device="cuda")
    r = torch.empty_like(state)
    jv = torch.empty_like(state)

    from aquaflux_gb300._lib import check, lib, ptr

    L = lib()
    stream = torch.cuda.current_stream()

    fn = {"vjp": L.fv_vjp, "jvp": L.fv_jvp, "jvp-linearised": L.fv_jvp_linearised}[args.step]
    if args.step == "jvp-linearised":
        case.linearise(state)  # held for every timed step (the same state values throughout)

    def step():
        check(fn(case.handle, ptr(state), ptr(vec), ptr(r), ptr(jv), stream.cuda_stream))

    # the stage kernels' block sizes, picked stage by stage by the library's autotuner (untimed)
    case.autotune(state, vec)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    case.profile_begin(args.steps)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        torch.cuda.synchronize()
        start.record(stream)
        for _ in range(args.steps):
            step()
        end.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    stage_ms, runs = case.profile_end()
    if not torch.isfinite(jv).all() or not torch.isfinite(r).all():
        raise RuntimeError("non-finite residual / derivative in the benchmark step")
    ms, value = replica_throughput(ms, F, args.steps, world, dist, "cuda")

    # end to end through the C ABI with pinned host buffers (copies inside the timed region): every
    # step copies its inputs in and its results out; the copies of neighbouring steps overlap the
    # step's compute (double-buffered device inputs / outputs, one stream each for host-to-device
    # copies, compute and device-to-host copies, ordered by events)
    h_state = state.cpu().pin_memory()
    h_vec = vec.cpu().pin_memory()
    h_r = torch.empty_like(h_state).pin_memory()
    h_jv = torch.empty_like(h_state).pin_memory()
    d_in = [(torch.empty_like(state), torch.empty_like(vec)) for _ in range(2)]
    d_out = [(torch.empty_like(state), torch.empty_like(state)) for _ in range(2)]
    s_h2d, s_d2h = torch.cuda.Stream(), torch.cuda.Stream()
    ev_in = [torch.cuda.Event() for _ in range(2)]     # inputs b copied in
    ev_used = [torch.cuda.Event() for _ in range(2)]   # step on buffer b computed
    ev_out = [torch.cuda.Event() for _ in range(2)]    # results b copied out
    pending = [False, False]

    def e2e_step(k):
        b = k % 2
        ds, dv = d_in[b]
        dr, dj = d_out[b]
        with torch.cuda.stream(s_h2d):
            if pending[b]:
                s_h2d.wait_event(ev_used[b])  # the step two back has read these inputs
            ds.copy_(h_state, non_blocking=True)
            dv.copy_(h_vec, non_blocking=True)
            ev_in[b].record(s_h2d)
        stream.wait_event(ev_in[b])
        if pending[b]:
            stream.wait_event(ev_out[b])  # the step two back's results are out
        check(fn(case.handle, ptr(ds), ptr(dv), ptr(dr), ptr(dj), stream.cuda_stream))
        ev_used[b].record(stream)
        with torch.cuda.stream(s_d2h):
            s_d2h.wait_event(ev_used[b])
            h_r.copy_(dr, non_blocking=True)
            h_jv.copy_(dj, non_blocking=True)
            ev_out[b].record(s_d2h)
        pending[b] = True

    for k in range(3):
        e2e_step(k)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s_h2d)  # before the first step's input copies
    for k in range(args.steps):
        e2e_step(k)
    for b in range(2):
        s_d2h.wait_event(ev_out[b])
    e1.record(s_d2h)  # after the last step's result copies
    torch.cuda.synchronize()
    e2e_ms, _ = replica_throughput(e0.elapsed_time(e1), F, args.steps, world, dist, "cuda")
    if dist is not None:
        dist.barrier()
    if rank != 0:
        return None

    peaks = measured_peaks()
    dom = max(stage_ms, key=stage_ms.get)
    # roofline of the dominant kernel of this step: the step's algorithmic bytes (each distinct
    # input read once, each output written once: 132.7 B/face for residual + VJP on the SST
    # channel) over that kernel's average CUDA-event launch duration; DRAM traffic and FP64-pipe
    # utilisation of the same kernel from the committed ncu capture
    bpf = step_bytes_per_face(wl, args.step)
    alg_bytes = bpf * F
    kname = {"vjp": "a_flux<3, SST> (adjoint face fluxes)",
             "jvp": "k_flux<Dual, 3, SST> (JVP face fluxes)",
             "jvp-linearised": "k_flux_tangent<3, SST> (JVP face-flux tangents)"}[args.step]
    kstage, tkey = {"vjp": ("a_flux", "a_flux"), "jvp": ("flux", "k_flux_dual"),
                    "jvp-linearised": ("flux", "k_flux_tangent")}[args.step]
    k_avg_ms = stage_ms[kstage] / max(runs, 1)
    achieved = alg_bytes / (k_avg_ms * 1e-3) / 1e9
    step_gbs = alg_bytes / (ms / args.steps * 1e-3) / 1e9
    traffic, fp64 = None, None
    traffic_path = os.path.join(ROOT, "profiles", "flux_traffic.json")
    if os.path.exists(traffic_path) and args.size == 128:
        with open(traffic_path) as f:
            tr = json.load(f).get(tkey, {})
        traffic = tr.get("bytes_128")
        fp64 = tr.get("fp64_pipe_active_pct")
    clk = clk.summary()
    # the FP64 pipe's roofline of the step: FP64-pipe instructions per face (ncu) x faces over the
    # step's time, against 2 instructions per clock per SM at the sampled SM clock
    fp64_roof = None
    instr_path = os.path.join(ROOT, "profiles", "fp64_instructions.json")
    per_face = None
    if os.path.exists(instr_path):
        with open(instr_path) as f:
            ins = json.load(f)
        per_face = ins.get({"vjp": "vjp_step_instr_per_face", "jvp": "jvp_step_instr_per_face",
                            "jvp-linearised": "jvp_linearised_step_instr_per_face"}[args.step])
    if per_face:
        mhz = clk.get("sm_mhz") or 2070.0
        peak_gi = ins["pipe_instr_per_clock_per_sm"] * ins["sms"] * mhz * 1e6 / 1e9
        ach_gi = per_face * F / (ms / args.steps * 1e-3) / 1e9
        fp64_roof = {"instr_per_face": per_face,
                     "achieved_ginstr_s": round(ach_gi, 1), "peak_ginstr_s": round(peak_gi, 1),
                     "frac": round(ach_gi / peak_gi, 4),
                     "bound_gfaces_s": round(peak_gi / per_face, 4),
                     "source": "profiles/fp64_%s_channel3d_64.md (ncu, 64^3)"
                               % {"vjp": "residual_vjp", "jvp": "jvp",
                                  "jvp-linearised": "jvp_linearised"}[args.step]}
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"channel3d {args.size}^3 k-omega SST (u,v,w,p,k,omega), "
                               f"{wl.mesh.n_cells} cells, {F} faces",
                   "step": STEP_DESC[args.step],
                   "cells": wl.mesh.n_cells, "faces": F,
                   "l2": "working set > 2 GB per step (inputs larger than the 129 MB L2)",
                   "cell_order": f"{args.cell_order} ({n_cell_classes} face-list patterns)",
                   "stage_block_size": dict(zip(case.STAGES, case.block_sizes())),
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(world * F * args.steps / (e2e_ms * 1e-3) / 1e9, 4), "unit": UNIT,
                "h2d_bytes_per_step": 2 * state.numel() * 8,
                "d2h_bytes_per_step": 2 * state.numel() * 8,
                "copies": "every step's inputs in and results out over pinned host memory, "
                          "overlapping the neighbouring steps' compute (double-buffered, "
                          "three streams)"},
        # stage kernels per step: 6 forward (+ 5 adjoint for the VJP; + the boundary faces'
        # coefficient and flux launches of the linearised JVP)
        "gpu_launches": (6 + {"vjp": 5, "jvp": 0, "jvp-linearised": 2}[args.step]) * args.steps,
        "stage_ms_per_step": {k: round(v / max(runs, 1), 4) for k, v in stage_ms.items()},
        "algorithmic_bytes_per_face": round(bpf, 2),
        "roofline": {"bound": "hbm", "kernel": kname, "dominant_stage": dom,
                     "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": round(traffic) if traffic else None,
                     "algorithmic_bytes": round(alg_bytes), "kernel_ms": round(k_avg_ms, 4),
                     "bytes_rule": f"{bpf:.1f} B/face x {F} faces: the whole step's compulsory "
                                   "bytes, charged to its dominant kernel's launch duration",
                     "step_achieved_gbs": round(step_gbs, 1),
                     "step_frac": round(step_gbs / peaks["hbm_gbs"], 4),
                     "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs)",
                     "fp64_pipe_active_pct_ncu": fp64,
                     "binding_limit": "fp64 pipe (profiles/fp64_residual_vjp_channel3d_64.md)",
                     "fp64_pipe": fp64_roof},
        "clocks": clk,
    }
    if not args.no_newton:
        out["newton"] = newton_block(args, wl, case)
    if not args.no_cpu_baseline:
        cb = cpu_residual_jvp_rate(args.cpu_sample, step=args.step)
        out["cpu_baseline"] = {"value": round(cb["faces_per_s"] / 1e9, 6), "unit": UNIT,
                               "cores": cb["cores"], "kind": "port", "sample": cb["sample"]}
        if args.ilu_sample > 0:
            try:
                out["cpu_ilu"] = ilu_cpu_vs_gpu(args.ilu_sample)
            except Exception as e:  # reported, never allowed to lose the headline line
                out["cpu_ilu"] = {"error": f"{type(e).__name__}: {e}"[:300]}
        if not args.no_config1:
            try:
                out["config1_newton"] = config1_newton(args)
            except Exception as e:  # reported, never allowed to lose the headline line
                out["config1_newton"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if not args.no_batched:
        try:
            out["batched"] = batched_step_timing()
        except Exception as e:  # reported, never allowed to lose the headline line
            out["batched"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if not args.no_cpu_baseline:
        try:
            out["renumbering"] = renumbering_block(args.size)
        except Exception as e:  # reported, never allowed to lose the headline line
            out["renumbering"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if not args.no_newton and not args.no_harder_start:
        try:
            out["harder_start"] = harder_start_block(args)
        except Exception as e:  # reported, never allowed to lose the headline line
            out["harder_start"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if "newton" in out:  # the headline Newton numbers last, where a truncated tail keeps them
        out["newton_summary"] = newton_summary(out["newton"], args.newton_kinds.split(","))
        hs = out.get("harder_start", {})
        if "direct" in hs:
            out["newton_summary"]["harder_start_nu_2.5e-4"] = {
                "direct_converged": hs["direct"]["converged"],
                "direct_s": hs["direct"]["seconds"],
                "continuation_converged": hs["reynolds_continuation"].get("converged"),
                "continuation_s": hs["reynolds_continuation"].get("seconds")}
    return out


def _field_errors(a, b, n_fields: int) -> dict:
    """max |a - b| / max |b| per field (field-major states) and over all fields."""
    av, bv = a.view(n_fields, -1), b.view(n_fields, -1)
    per = [float((av[q] - bv[q]).abs().max() / bv[q].abs().max().clamp_min(1e-300))
           for q in range(n_fields)]
    return {"max": max(per), "per_field": [float(f"{e:.3g}") for e in per]}


def newton_block(args, wl, case) -> dict:
    """Newton-solve seconds for each preconditioner kind (aggregation-AMG V-cycle, ILU(0)) in three
    forms: fp64 throughout; an fp32 preconditioner (its frozen Jacobian assembled by fp32 dual
    numbers, factored and applied in fp32) with the fp64 Krylov operator J v; the same with J v
    in fp32 as well ("fp32 tangents").  The AMG preconditioner's connectivity-only plan is made
    once per mesh before the timed solves and reported as ``mesh_plan``.

    Every form: fp64 residual, fp64 FGMRES(30) with Krylov orthogonalisation, fp64 Newton update
    and line search, so every form converges to the fp64 root.  Each solve is timed whole, from
    the initial state and including the preconditioner's setup on the case's kept plan (device
    levels, ILU(0) structures, factors; the "setup" phase).  Stops at ||R|| <= 1e-12 + 1e-10 ||R0||.  Every converged state is then checked
    against the FP64 CPU oracle (its residual relative to the oracle's ||R(s0)||) and against a
    tightly converged FP64 root (per-field relative field error).
    """
    import numpy as np
    import torch

    from aquaflux_gb300 import solve

    out = {}
    # one materialisation of the frozen block Jacobian: direct face assembly vs coloured probes
    s0 = torch.tensor(wl.initial_state(), device="cuda")
    jt = {}
    for method in ("assemble", "probe"):
        jac = solve.BlockJacobian(case, method=method)
        jac.materialize(s0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        jac.materialize(s0)
        torch.cuda.synchronize()
        jt[method] = round((time.perf_counter() - t0) * 1e3, 2)
        if method == "probe":
            jt["n_probes"] = jac.n_probes
        del jac
    out["jacobian_ms"] = jt
    # the Krylov operator at the plug-flow state: the dual-number JVP, the linearisation (one
    # residual keeping its face intermediates) and the linearised JVP the fp64-tangent forms use
    v0 = torch.randn(s0.numel(), dtype=torch.float64, device="cuda",
                     generator=torch.Generator(device="cuda").manual_seed(3))

    def per_call_ms(fn, k=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return round(e0.elapsed_time(e1) / k, 3)

    kops = {"jvp_dual_numbers": per_call_ms(lambda: case.jvp(s0, v0)),
            "jvp_fp32_tangents": per_call_ms(lambda: case.jvp(s0, v0, precision=32)),
            "linearise": per_call_ms(lambda: case.linearise(s0))}
    kops["jvp_linearised"] = per_call_ms(lambda: case.jvp_linearised(s0, v0))
    ref = case.jvp(s0, v0)
    kops["linearised_max_rel_diff"] = float((case.jvp_linearised(s0, v0) - ref).abs().max()
                                            / ref.abs().max())
    out["krylov_operator_ms"] = kops
    # untimed warm-up of every solver path on a small channel (library initialisation, graph
    # captures), so that the timed solves below measure steady-state work
    from aquaflux_gb300 import workloads

    kinds = args.newton_kinds.split(",")
    warm = workloads.channel3d(16)
    warm_case = warm.device_case()
    forms = ((64, 64), (32, 64), (32, 32))  # (preconditioner precision, tangent precision)
    for kind in kinds:
        for prec, tan in forms:
            solve.newton_solve(warm_case, warm.initial_state(), precision=prec, tangents=tan,
                               kind="amg" if kind.startswith("amg") else kind, max_steps=40)
    del warm_case
    # the AMG preconditioner's connectivity-only plan (fine colour order, aggregation hierarchy:
    # host work), made by the first preconditioner built on this case and kept for every later
    # solve on it, as the mesh geometry is (FlowCase.pattern_plan): timed here, once per mesh, as
    # the first build minus a second one; the timed solves below reuse it
    from aquaflux_gb300.amg import AmgPreconditioner

    plan_s = {}
    for kind in kinds:
        if not kind.startswith("amg"):
            continue
        fine = {"amg-colour": "colour", "amg-natural": "natural"}.get(kind, "auto")
        builds = []
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pc = AmgPreconditioner(solve.BlockJacobian(case, precision=32), 32, fine_order=fine)
            torch.cuda.synchronize()
            builds.append(time.perf_counter() - t0)
            del pc
        plan_s[kind] = {"first_build_s": round(builds[0], 3), "later_build_s": round(builds[1], 3),
                        "plan_s": round(builds[0] - builds[1], 3)}
    if plan_s:
        out["mesh_plan"] = dict(plan_s, what="the AMG preconditioner's connectivity-only host plan "
                                "(fine colour order, aggregation, coarse patterns and colourings), "
                                "made once per mesh; every Newton solve below reuses it and "
                                "includes the rest of its setup")
    # one untimed two-step solve at full size: the first full-size Krylov iterations of a process
    # pay one-off costs (allocator growth to FGMRES(30)'s bases, first large-shape library calls)
    # that no timed form should carry alone
    solve.newton_solve(case, wl.initial_state(), precision=64, kind="amg", max_steps=2)
    torch.cuda.synchronize()
    states = {}
    for kind in kinds:
        for prec, tan in forms:
            torch.cuda.synchronize()
            opts = ({"fine_order": "colour"} if kind == "amg-colour" else
                    {"fine_order": "natural"} if kind == "amg-natural" else None)
            res = solve.newton_solve(case, wl.initial_state(), precision=prec, tangents=tan,
                                     kind="amg" if kind.startswith("amg") else kind,
                                     precond_options=opts, max_steps=40)
            key = f"{kind}_fp{prec}" + ("_fp32_tangents" if tan == 32 else "")
            out[key] = {
                "seconds": round(res.seconds, 3), "converged": bool(res.converged),
                "newton_steps": res.steps, "krylov_iterations": int(sum(res.krylov_iterations)),
                "final_rel_residual": res.residual_norms[-1] / res.residual_norms[0],
                "phase_seconds": {k: round(v, 3) for k, v in res.phase_seconds.items()}}
            states[(kind, prec, tan)] = res.state
            del res
        for prec, tan in forms[1:]:
            key = f"{kind}_fp{prec}" + ("_fp32_tangents" if tan == 32 else "")
            out[f"{key}_speedup_vs_fp64"] = round(
                out[f"{kind}_fp64"]["seconds"] / out[key]["seconds"], 3)
    if not args.no_adjoint:
        out["adjoint"] = adjoint_block(case, states[(kinds[0], 32, 64)])
    # the default kind's forms solved on to 1e-13 relative: the fields converged to the root
    # (the reference's 1e-10 leaves every form, fp64 included, ~1e-4 from the root on this mesh)
    for prec, tan in forms:
        torch.cuda.synchronize()
        res = solve.newton_solve(case, wl.initial_state(), precision=prec, tangents=tan,
                                 kind="amg" if kinds[0].startswith("amg") else kinds[0],
                                 rtol=1e-13, atol=0.0, max_steps=40)
        key = f"{kinds[0]}_fp{prec}" + ("_fp32_tangents" if tan == 32 else "") + "_to_1e-13"
        out[key] = {"seconds": round(res.seconds, 3), "converged": bool(res.converged),
                    "newton_steps": res.steps,
                    "krylov_iterations": int(sum(res.krylov_iterations)),
                    "final_rel_residual": res.residual_norms[-1] / res.residual_norms[0]}
        states[(kinds[0] + "_to_1e-13", prec, tan)] = res.state
        del res
    # a tight FP64 root, reached along another path: the last kind's fp64 solution refined by
    # Newton with tight linear solves until the residual stops falling; every form's fields are
    # compared with it
    nfld = case.n_unknowns // wl.mesh.n_cells
    tight = solve.newton_solve(case, states[(kinds[-1], 64, 64)], precision=64, kind="amg",
                               rtol=1e-14, atol=0.0, linear_rtol=1e-8, max_steps=4)
    r0 = float(torch.linalg.vector_norm(case.residual(s0)))
    out["tight_root"] = {"rel_residual": tight.residual_norms[-1] / r0,
                         "newton_steps": tight.steps, "from": f"{kinds[-1]}_fp64"}
    for (kind, prec, tan), st in states.items():
        key = f"{kind}_fp{prec}" + ("_fp32_tangents" if tan == 32 else "")
        if kind.endswith("_to_1e-13"):
            key = f"{kind[:-len('_to_1e-13')]}_fp{prec}" + \
                ("_fp32_tangents" if tan == 32 else "") + "_to_1e-13"
        out[key]["field_error_vs_tight_root"] = _field_errors(st, tight.state, nfld)
    # the FP64 CPU oracle's residual of every converged state, relative to its ||R(s0)||
    if not args.no_newton_oracle:
        from oracle import fv_oracle as fo

        torch.set_num_threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        c = fo.make_case(wl.mesh, mu=wl.mu, rho=wl.rho, flow_bc=wl.flow_bc,
                         sst={"nu": wl.mu / wl.rho, "walls": wl.sst["walls"], "k": wl.sst["k"],
                              "omega": wl.sst["omega"]})
        orc = fo.Oracle(c)
        r0o = float(np.linalg.norm(orc.residual(torch.as_tensor(wl.initial_state())).numpy()))
        for (kind, prec, tan), st in states.items():
            if kind.endswith("_to_1e-13"):
                continue
            key = f"{kind}_fp{prec}" + ("_fp32_tangents" if tan == 32 else "")
            ro = float(np.linalg.norm(orc.residual(st.cpu()).numpy()))
            out[key]["oracle_rel_residual"] = ro / r0o
        out["oracle_check_seconds"] = round(time.perf_counter() - t0, 1)
    return out


def config1_newton(args) -> dict:
    """Config 1 (64 x 64 lid-driven cavity, Re = 100, from rest): the GPU Newton solve in fp64 and
    with the fp32 ILU(0) preconditioner, beside the CPU oracle's Newton (exact sparse Jacobian,
    sparse LU; one process, all host threads for the residual products) to the same tolerance,
    and each GPU root against the CPU root."""
    import numpy as np
    import torch

    from aquaflux_gb300 import solve, workloads
    from oracle import fv_oracle as fo
    from oracle.newton_oracle import OracleJacobian, newton

    wl = workloads.cavity(64)
    case = wl.device_case()
    z = np.zeros(case.n_unknowns)
    out = {"workload": "64 x 64 lid-driven cavity, Re = 100, zero start, to 1e-10 relative"}
    states = {}
    for prec in (64, 32):
        solve.newton_solve(case, z, precision=prec, max_steps=40)  # warm
        torch.cuda.synchronize()
        res = solve.newton_solve(case, z, precision=prec, max_steps=40)
        states[prec] = res.state.cpu().numpy()
        out[f"gpu_ilu_fp{prec}"] = {"seconds": round(res.seconds, 3), "newton_steps": res.steps,
                                   "converged": bool(res.converged)}
    torch.set_num_threads(os.cpu_count() or 1)
    orc = fo.Oracle(fo.make_case(wl.mesh, mu=wl.mu, rho=wl.rho, flow_bc=wl.flow_bc,
                                 pressure_pin=wl.pressure_pin))
    jac = OracleJacobian(orc, wl.mesh.owner, wl.mesh.neighbour, wl.mesh.n_cells, 3)
    cpu = newton(orc, jac, z)
    out["cpu_oracle"] = {"seconds": round(cpu["seconds"], 2), "newton_steps": cpu["steps"],
                         "converged": bool(cpu["converged"]), "cores": os.cpu_count() or 1,
                         "kind": "port", "what": "oracle residual, exact sparse Jacobian from "
                                                 "reverse-mode products, SuperLU solves"}
    root = cpu["state"]
    for prec, st in states.items():
        out[f"gpu_ilu_fp{prec}"]["field_max_rel_diff_vs_cpu_root"] = float(
            np.abs(st - root).max() / np.abs(root).max())
    out["gpu_fp32_speedup_vs_cpu"] = round(cpu["seconds"] / out["gpu_ilu_fp32"]["seconds"], 1)
    return out


def newton_summary(nb: dict, kinds: list) -> dict:
    """The headline Newton numbers, repeated at the end of the JSON line."""
    out = {}
    for kind in kinds:
        f64, f32, t32 = (nb.get(f"{kind}_fp64"), nb.get(f"{kind}_fp32"),
                         nb.get(f"{kind}_fp32_fp32_tangents"))
        if not f64:
            continue
        out[kind] = {"fp64_s": f64["seconds"], "fp32_precond_s": f32["seconds"],
                     "fp32_precond_speedup": nb.get(f"{kind}_fp32_speedup_vs_fp64"),
                     "fp32_precond_fp32_tangents_s": t32["seconds"],
                     "fp32_precond_fp32_tangents_speedup":
                         nb.get(f"{kind}_fp32_fp32_tangents_speedup_vs_fp64"),
                     "max_oracle_rel_residual": max(
                         (nb[k].get("oracle_rel_residual", float("nan"))
                          for k in (f"{kind}_fp64", f"{kind}_fp32", f"{kind}_fp32_fp32_tangents")),
                         default=None),
                     "max_field_error_vs_tight_root": max(
                         nb[k]["field_error_vs_tight_root"]["max"]
                         for k in (f"{kind}_fp64", f"{kind}_fp32", f"{kind}_fp32_fp32_tangents"))}
        tight = [nb.get(f"{kind}_fp{p}{t}_to_1e-13") for p, t in
                 (("64", ""), ("32", ""), ("32", "_fp32_tangents"))]
        if all(tight):
            out[kind]["to_1e-13"] = {
                "fp64_s": tight[0]["seconds"], "fp32_precond_s": tight[1]["seconds"],
                "fp32_precond_fp32_tangents_s": tight[2]["seconds"],
                "fp32_precond_speedup": round(tight[0]["seconds"] / tight[1]["seconds"], 3),
                "fp32_precond_fp32_tangents_speedup":
                    round(tight[0]["seconds"] / tight[2]["seconds"], 3),
                "max_field_error_vs_tight_root": max(
                    t["field_error_vs_tight_root"]["max"] for t in tight)}
    return out


def adjoint_block(case, state) -> dict:
    """The 3D channel's adjoint objectives at the converged fp32-preconditioned state: the outlet
    mass flux and the wall shear force, each differentiated with respect to viscosity, inlet
    velocity and every node coordinate by the implicit function theorem (the transposed fp32
    V-cycle preconditioning FGMRES on the hand-written VJP, 1e-10)."""
    import torch

    from aquaflux_gb300 import solve
    from aquaflux_gb300.amg import AmgPreconditioner

    dim = case.dim
    out = {}
    pc = AmgPreconditioner(solve.BlockJacobian(case), 32)
    for name, spec, visc in (("outlet_mass_flux", {"right": {dim: 1.0}}, False),
                             ("wall_shear_x", {w: {0: 1.0} for w in
                                               ("bottom", "top", "back", "front")}, True)):
        w = case.functional_weights(spec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = solve.functional_gradient(case, state, w, viscous_only=visc, preconditioner=pc)
        torch.cuda.synchronize()
        out[name] = {"seconds": round(time.perf_counter() - t0, 3), "value": g.value,
                     "dJ_dmu": float(g.dparams[0]), "dJ_dinlet_scale": float(g.dparams[1]),
                     "dJ_dnodes_norm": float(torch.linalg.vector_norm(g.dnodes)),
                     "krylov_iterations": g.adjoint.krylov_iterations,
                     "converged": bool(g.adjoint.converged)}
    # the mesh-coordinate VJP alone
    lam = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda")
    case.node_vjp(state, lam)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    case.node_vjp(state, lam)
    torch.cuda.synchronize()
    out["node_vjp_ms"] = round((time.perf_counter() - t0) * 1e3, 2)
    return out


def harder_start_block(args) -> dict:
    """A harder start: the --size channel at nu = 2.5e-4 (twice the headline Reynolds number)
    from the plug-flow state, with the fp32 AMG preconditioner and the fp64 Krylov operator -- a
    direct Newton solve beside Reynolds continuation with one lower point (nu = 5e-4, converged to
    1e-6; solve_reynolds_continuation, aquaflux/turbulence/reynolds.py:144-338), both to 1e-10.
    The roots are checked by their relative residual on the GPU."""
    import torch

    from aquaflux_gb300 import solve, workloads

    nu = 2.5e-4
    wl = workloads.channel3d(args.size, nu=nu)
    case = wl.device_case()
    s0 = wl.initial_state()
    opts = dict(precision=32, tangents=64, kind="amg", max_steps=25)
    out = {"workload": f"channel3d {args.size}^3 SST, nu = {nu:g}, plug-flow start",
           "form": "fp32 AMG preconditioner, fp64 J v, to 1e-10"}
    r0 = float(torch.linalg.vector_norm(case.residual(torch.as_tensor(s0, device="cuda"))))
    torch.cuda.synchronize()
    d = solve.newton_solve(case, s0, **opts)
    rel = float(torch.linalg.vector_norm(case.residual(d.state))) / r0
    out["direct"] = {"converged": bool(d.converged), "newton_steps": d.steps,
                     "krylov_iterations": int(sum(d.krylov_iterations)),
                     "seconds": round(d.seconds, 3),
                     "final_rel_residual": rel if math.isfinite(rel) else None}
    try:
        # the rung converged to 1e-6: at 1e-2 relative the first Newton step (which only sets the
        # near-wall omega rows) already passes and leaves an undeveloped seed
        c = solve.reynolds_continuation(case, s0, 1, ratio=2.0, intermediate_rtol=1e-6, **opts)
        rel = float(torch.linalg.vector_norm(case.residual(c.state))) / r0
        out["reynolds_continuation"] = {
            "converged": c.converged, "seconds": round(c.seconds, 3), "points": c.points,
            "final_rel_residual": rel if math.isfinite(rel) else None}
    except RuntimeError as e:
        out["reynolds_continuation"] = {"converged": False, "error": str(e)[:300]}
    return out


def renumbering_block(size: int) -> dict:
    """Reverse Cuthill-McKee of the randomly relabelled ``size^3`` channel: on the GPU (the cell
    graph and the level-by-level sweeps; host argsort of the degrees and the copies included)
    beside scipy's ``reverse_cuthill_mckee`` on the host (the reference's own call, one core),
    with the permutations compared."""
    import numpy as np
    import torch

    from aquaflux_gb300 import mesh as fm
    from aquaflux_gb300 import workloads
    from aquaflux_gb300.reorder import mesh_rcm_permutation

    m = workloads.channel3d(size, renumber=False).mesh
    m = fm.permute_cells(m, fm.random_permutation(m.n_cells, 0))
    mesh_rcm_permutation(m)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gpu = mesh_rcm_permutation(m)
    torch.cuda.synchronize()
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = workloads.rcm_permutation(m)
    t_cpu = time.perf_counter() - t0
    return {"cells": m.n_cells, "gpu_ms": round(t_gpu * 1e3, 1),
            "scipy_ms": round(t_cpu * 1e3, 1), "cpu_kind": "reference",
            "bitwise_equal": bool(np.array_equal(gpu, ref))}


def batched_step_timing(steps: int = 20, warmup: int = 5) -> dict:
    """The batched calibration sweep's residual + VJP over all 64 instances (one disjoint-union
    case): the stage-per-launch step replayed as one CUDA graph, and the same step as one
    persistent cooperative launch (block size and per-thread chunk autotuned); results bitwise
    equal."""
    import torch

    from aquaflux_gb300 import workloads
    from aquaflux_gb300._lib import check, lib, ptr

    bw = workloads.batched_channels(64, seed=0)
    case = bw.workload.device_case()
    m = bw.workload.mesh
    s = torch.tensor(bw.initial_state(), device="cuda")
    w = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(0))
    best_tb = case.autotune(s, w)
    out_g = torch.empty_like(s)
    out_p = torch.empty_like(s)

    def step(out):
        check(lib().fv_vjp(case.handle, ptr(s), ptr(w), 0, ptr(out),
                           torch.cuda.current_stream().cuda_stream))

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    for _ in range(3):
        step(out_g)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step(out_g)
    ms_graph = timed(graph.replay)
    block, chunk, _ = case.autotune_persistent(s, w)
    case.set_persistent(True, block, chunk)
    ms_pers = timed(lambda: step(out_p))
    case.set_persistent(False)
    return {"workload": f"64 2D laminar channels, n in [{int(bw.sizes.min())}, "
                        f"{int(bw.sizes.max())}], {m.n_cells} cells, {m.n_faces} faces",
            "graph_of_stage_launches_ms": round(ms_graph, 4), "stage_block_size": best_tb,
            "persistent_launch_ms": round(ms_pers, 4), "persistent_block": block,
            "persistent_chunk": chunk,
            "gfaces_s_graph": round(m.n_faces / (ms_graph * 1e-3) / 1e9, 4),
            "gfaces_s_persistent": round(m.n_faces / (ms_pers * 1e-3) / 1e9, 4),
            "bitwise_equal": bool(torch.equal(out_g, out_p))}


def run_batched(args) -> dict:
    """The batched calibration sweep: 64 uneven 2D laminar channels side by side in one
    disjoint-union case.  Residual + VJP of all instances, one launch per stage, captured once in a
    CUDA graph and replayed (block size autotuned first); then the calibration itself: one Newton
    solve (fp32 AMG V-cycle) for every instance and one adjoint solve giving each instance's
    d(mean outlet velocity)/d(viscosity, inlet velocity)."""
    import numpy as np
    import torch

    from aquaflux_gb300 import solve, workloads
    from aquaflux_gb300.amg import AmgPreconditioner

    bw = workloads.batched_channels(64, seed=0)
    case = bw.workload.device_case()
    m = bw.workload.mesh
    s = torch.tensor(bw.initial_state(), device="cuda")
    w = torch.randn(case.n_unknowns, dtype=torch.float64, device="cuda")
    best_tb = case.autotune(s, w)
    out_buf = torch.empty_like(s)
    from aquaflux_gb300._lib import check, lib, ptr

    def step():
        check(lib().fv_vjp(case.handle, ptr(s), ptr(w), 0, ptr(out_buf),
                           torch.cuda.current_stream().cuda_stream))

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        graph.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ref = out_buf.clone()
    step()
    torch.cuda.synchronize()
    assert torch.equal(ref, out_buf)
    gfaces = m.n_faces / (ms * 1e-3) / 1e9
    # the same step as one persistent cooperative launch (autotuned block and chunk)
    pblock, pchunk, _ = case.autotune_persistent(s, w)
    case.set_persistent(True, pblock, pchunk)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms_p = e0.elapsed_time(e1) / args.steps
    persistent = {"ms_per_step": round(ms_p, 4), "block": pblock, "chunk": pchunk,
                  "gfaces_s": round(m.n_faces / (ms_p * 1e-3) / 1e9, 4),
                  "bitwise_equal_graph": bool(torch.equal(ref, out_buf))}
    case.set_persistent(False)
    # the calibration: Newton for all instances at once, then one adjoint for all gradients
    warm = workloads.batched_channels(4, n_min=8, n_max=16, seed=1)
    wc = warm.workload.device_case()
    wres = solve.newton_solve(wc, warm.initial_state(), kind="amg", precision=32, max_steps=60)
    solve.batched_gradients(wc, wres.state, warm,
                            preconditioner=AmgPreconditioner(solve.BlockJacobian(wc), 32))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = solve.newton_solve(case, bw.initial_state(), kind="amg", precision=32, max_steps=60)
    torch.cuda.synchronize()
    t_newton = time.perf_counter() - t0
    t0 = time.perf_counter()
    g = solve.batched_gradients(case, res.state, bw,
                                preconditioner=AmgPreconditioner(solve.BlockJacobian(case), 32))
    torch.cuda.synchronize()
    t_adj = time.perf_counter() - t0
    return {
        "metric": "batched residual+VJP Gfaces/s (64 uneven instances, one launch per stage)",
        "value": round(gfaces, 4), "unit": "Gfaces/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"64 2D laminar channels, n x n with n in [{int(bw.sizes.min())}, "
                               f"{int(bw.sizes.max())}], {m.n_cells} cells, {m.n_faces} faces",
                   "graph": "one CUDA graph replay per step", "block_size": best_tb},
        "instances_per_s": round(64.0 / (ms * 1e-3), 1),
        "persistent_launch": persistent,
        "calibration": {"newton_seconds": round(t_newton, 3), "converged": bool(res.converged),
                        "newton_steps": res.steps,
                        "krylov_iterations": int(sum(res.krylov_iterations)),
                        "adjoint_seconds": round(t_adj, 3),
                        "adjoint_krylov_iterations": g.adjoint.krylov_iterations,
                        "mean_outlet_velocity_range": [float(g.value.min()), float(g.value.max())],
                        "dJ_dmu_range": [float(g.dmu.min()), float(g.dmu.max())],
                        "dJ_dvelocity_range": [float(g.dvelocity.min()),
                                               float(g.dvelocity.max())]},
    }


def cpu_full_size_rate(size: int, step: str = "vjp") -> dict:
    """One residual + VJP (or JVP) of the CPU oracle on the full ``size^3`` channel (all host
    threads), timed after one untimed evaluation: the reference algorithm's CPU throughput at the
    benchmark's own size."""
    import numpy as np
    import torch

    from aquaflux_gb300 import workloads
    from oracle import fv_oracle as fo

    torch.set_num_threads(os.cpu_count() or 1)
    wl = workloads.channel3d(size, renumber="host")
    case = fo.make_case(wl.mesh, mu=wl.mu, rho=wl.rho, flow_bc=wl.flow_bc,
                        sst={"nu": wl.mu / wl.rho, "walls": wl.sst["walls"], "k": wl.sst["k"],
                             "omega": wl.sst["omega"]})
    orc = fo.Oracle(case)
    s = wl.initial_state(seed=1, noise=0.05)
    v = np.random.default_rng(2).standard_normal(s.size)

    def one():
        if step == "vjp":
            x = torch.as_tensor(s).requires_grad_(True)
            r = orc.residual(x)
            torch.autograd.grad(r, x, torch.as_tensor(v))
        else:
            orc.residual(torch.as_tensor(s))
            orc.jvp(s, v)

    one()
    t0 = time.perf_counter()
    one()
    el = time.perf_counter() - t0
    return {"faces_per_s": wl.mesh.n_faces / el, "seconds": el, "cores": os.cpu_count() or 1,
            "faces": wl.mesh.n_faces}


def run_reference(args) -> dict:
    cb = cpu_residual_jvp_rate(args.cpu_sample, min_seconds=4.0, step=args.step)
    rates = [cb["faces_per_s"]]
    for _ in range(max(args.steps, 1) - 1):
        rates.append(cpu_residual_jvp_rate(args.cpu_sample, min_seconds=2.0,
                                           step=args.step)["faces_per_s"])
    v = statistics.median(rates) / 1e9
    full = None
    if args.reference_full_size:
        try:
            full = cpu_full_size_rate(args.size, step=args.step)
        except Exception as e:  # reported, never allowed to lose the line
            full = {"error": f"{type(e).__name__}: {e}"[:200]}
    return {
        "impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"channel3d {args.size}^3 k-omega SST; CPU sample "
                               f"{args.cpu_sample}^3 per step",
                   "step": STEP_DESC[args.step]},
        "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": cb["cores"], "kind": "port",
                         "sample": cb["sample"]},
        "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "full_size": None if full is None else (
            full if "error" in full else
            {"value": round(full["faces_per_s"] / 1e9, 6), "unit": UNIT,
             "seconds_per_evaluation": round(full["seconds"], 2), "faces": full["faces"],
             "cores": full["cores"],
             "what": f"one residual + {args.step.upper()} of the CPU oracle on the full "
                     f"{args.size}^3 channel"}),
    }


def main():
    args = _args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.gpus == 1 else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    import __graft_entry__

    __graft_entry__.build()
    if args.workload == "batched":
        if rank == 0:
            print(json.dumps(run_batched(args)))
        return
    if args.newton_only:
        if rank == 0:
            print(json.dumps(run_newton_only(args)))
        return
    if args.vcycle_only:
        if rank == 0:
            print(json.dumps(run_vcycle_only(args)))
        return
    out = run_gpu(args, rank, world, local_rank)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
