#!/usr/bin/env python
"""Benchmark of the Euler-2D explicit step on one GB300.

Headline workload: 2048 x 2048 cells, FP64, HLLC flux, MC slopes, reflective
walls, gamma 1.4, CFL 0.8, diagonal-discontinuity initial state,
implementationVersion 0 (fused), 100 steps.  A "step" is one time step of the
reference's HydroRun loop (compute_dt + godunov_unsplit) over the whole grid.

Metric: Mcell-updates/s = nx * ny * steps / time (interior cells; the
reference's own formula, which counts ghost cells, is reported beside it).

Library build (--arith): "fma" (default; multiply-adds fused as nvfortran's
GPU builds of the reference do, divisions and square roots faithfully
rounded, results within the specified 1e-12 relative L1 per variable and
1e-14 relative dt of the FP64 oracle, checked in the line's
`accuracy_vs_fp64_oracle`) or "exact" (no contraction, IEEE rounding,
bitwise the oracle).  Both builds appear in `variants`.

value       device time (CUDA events on the launching stream) of `steps`
            steps replayed from a CUDA graph, state resident in HBM.
e2e         wall time of the reference driver's call sequence through the C
            ABI with host buffers: upload of the initial state from pinned
            memory, compute_dt (dt read back to the host every step) and
            godunov_unsplit per step, download of the final state.
roofline    HBM roofline of the step kernel (64 B per cell update in FP64:
            read U, write U'), plus the FP64 pipe roof that actually binds it.
cpu_baseline  the CPU oracle (serial_ref restatement) on a bounded sample.

`--impl reference` times the CPU implementation of the reference's path (the
oracle port: no Fortran compiler exists on the GPU machine) with all host threads on
the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

BYTES_PER_CELL = {8: 64, 4: 32}  # read U (4 words) + write U' (4 words)


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--precision", type=int, choices=[4, 8], default=8)
    ap.add_argument("--version", type=int, choices=[0, 1, 2], default=0)
    ap.add_argument("--riemann", choices=["hllc", "approx"], default="hllc")
    ap.add_argument("--arith", choices=["exact", "fma"], default="fma",
                    help="library build: fma (multiply-adds fused; within 1e-12 relative L1 and 1e-14 relative dt "
                         "of the FP64 oracle) or exact (bitwise serial_ref arithmetic)")
    ap.add_argument("--cpu-steps", type=int, default=3, help="steps of the single-thread CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-steps", type=int, default=200)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adjoint-nx", type=int, default=512)
    ap.add_argument("--adjoint-steps", type=int, default=200)
    ap.add_argument("--adjoint-batch-steps", type=int, default=100, help="0 skips the batched adjoint")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed

def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Replicas only: each rank advances its own grid on its own GPU; the
    process group carries the barrier and the max of the timings, never data."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_info()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


def device_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except ImportError:
        pass


# ---------------------------------------------------------------- clocks

CLOCK_Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={CLOCK_Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        under = [s for s in sm if s > 0.5 * mx] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": under[len(under) // 2], "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


# ---------------------------------------------------------------- helpers

def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_value(precision: int, nx: int, version: int, key: str, arith: str = "exact"):
    """A per-launch figure of the step kernel (`dram_bytes_per_launch`,
    `fp64_warp_inst_per_launch`, `thread_inst_per_cell`) from the committed
    ncu summary of the same workload and library build, if there is one."""
    suffix = "_fma" if arith == "fma" else ""
    name = f"k_fused_{nx}_{'fp64' if precision == 8 else 'fp32'}{suffix}_traffic.txt" if version == 0 else None
    if not name:
        return None
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            return float(line.split(":")[1])
    return None


def profiled_traffic(precision: int, nx: int, version: int, arith: str = "exact"):
    return profiled_value(precision, nx, version, "dram_bytes_per_launch", arith)


def workload_name(a):
    prec = "FP64" if a.precision == 8 else "FP32"
    return (f"euler2d {a.nx}x{a.nx} {prec}, {a.riemann.upper()} flux, MC slopes, reflective walls, "
            f"gamma 1.4, CFL 0.8, diagonal discontinuity, implementationVersion {a.version}")


def oracle_params(a):
    from oracle import oracle as O
    return O.Params(nx=a.nx, ny=a.nx, gamma0=1.4, cfl=0.8, riemann=2 if a.riemann == "hllc" else 0)


def time_oracle(a, nsteps: int, nthreads: int):
    """Wall time of nsteps oracle steps (after one untimed step)."""
    from oracle import oracle as O
    p = oracle_params(a)
    prec = "f64" if a.precision == 8 else "f32"
    u = O.init_implode(p, prec)
    _, _, u, u2 = O.run(p, 1, prec=prec, u0=u, nthreads=nthreads)  # warm-up step: state after 1 step in u2
    t0 = time.perf_counter()
    O.run(p, nsteps, prec=prec, u0=u2, nthreads=nthreads)
    return time.perf_counter() - t0


# ---------------------------------------------------------------- reference arm

def bench_config(a, ws: int):
    """The workload description both arms print (identical dicts)."""
    isz = a.nx + 4
    return {"workload": workload_name(a), "nx": a.nx, "ny": a.nx, "steps": a.steps,
            "parallelism": "replicas" if ws > 1 else "single GPU",
            "l2": "inputs larger than L2 (u and u2: 2 x %.1f MB ping-pong per step)"
                  % (4 * isz * isz * a.precision / 1e6)}


def run_reference(a, dist):
    if dist.rank != 0:
        return
    from oracle import oracle as O
    O.build()
    nthreads = os.cpu_count() or 1
    cells = a.nx * a.nx
    if a.warmup:
        time_oracle(a, a.warmup, nthreads)
    t = time_oracle(a, a.steps, nthreads)
    v = cells * a.steps / t / 1e6
    line = {
        "impl": "reference", "metric": "Mcell-updates/s", "value": round(v, 3), "unit": "Mcell-updates/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(1e3 * t / a.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if a.precision == 8 else "f32", "data": "synthetic",
        "config": bench_config(a, dist.ws),
        "cpu_baseline": {"value": round(v, 3), "unit": "Mcell-updates/s", "cores": nthreads, "kind": "port",
                         "sample": f"{a.nx}x{a.nx}, {a.steps} steps after {a.warmup} warm-up steps: CPU "
                                   f"restatement of serial_ref (no Fortran compiler on the box) with OpenMP on "
                                   f"the do-concurrent loops of stdpar"},
        "e2e": {"value": round(v, 3), "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- batched ensemble

def measure_batched(E, a):
    """64 seeded problems (sides 128..1024, offsets, states and walls at random)
    advanced together by one launch per step from a captured graph, against the
    same problems advanced one after another: with the single-run kernel's
    device-resident graphs (plain) and with the reference's per-call loop
    (compute_dt with dt read back, then godunov_unsplit, every step)."""
    from euler2d_cudafortran_gb300.ensemble import diagonal_ensemble
    ens = diagonal_ensemble(64, 12345)
    n = a.batched_steps
    riemann = E.RIEMANN_HLLC if a.riemann == "hllc" else E.RIEMANN_APPROX
    init = (ens.offset, ens.rho_hi, ens.p_hi, ens.rho_lo, ens.p_lo)
    with E.Batch(ens.sizes, ens.bcs, gamma0=1.4, cfl=0.8, riemann_solver=riemann, precision=a.precision,
                 arith=a.arith) as b:
        b.init_diagonal(*init)
        t0 = time.perf_counter()
        b.tune(steps=3)
        tune_s = time.perf_counter() - t0
        sched = b.schedule()
        b.advance(0, n, log=False)  # captures the graph of the timed sequence
        b.init_diagonal(*init)
        b.advance(0, n, log=False)
        batched_ms = b.last_advance_ms()
        health = [b.health(k) for k in range(b.nprob)]
    plain_ms = 0.0
    percall_s = 0.0
    for k, (nx, ny) in enumerate(ens.sizes):
        bc = ens.bcs[k]
        p = E.make_params(nx=nx, ny=ny, gamma0=1.4, cfl=0.8, riemann_solver=riemann, precision=a.precision,
                          boundary_type_xmin=bc[0], boundary_type_xmax=bc[1], boundary_type_ymin=bc[2],
                          boundary_type_ymax=bc[3])
        with E.HydroRun(p, arith=a.arith) as run:
            run.init_diagonal(*(x[k] for x in init))
            run.advance(0, n, log=False)
            plain_ms += run.last_advance_ms()
            # the reference's own loop (serial_ref/main.f90:66-74): compute_dt
            # with dt back on the host, then godunov_unsplit, every step
            run.init_diagonal(*(x[k] for x in init))
            run.synchronize()
            t0 = time.perf_counter()
            run.compute_dt(0)
            run.make_boundaries(0)
            for step in range(n):
                dt = run.compute_dt(step % 2)
                run.godunov_unsplit(step, dt)
            run.synchronize()
            percall_s += time.perf_counter() - t0
    cells = ens.cells
    return {"workload": f"64 problems, sides uniform in {{128..1024 step 64}} (total {cells} cells), "
                        f"seed 12345, {n} steps per graph", "steps": n,
            "mcells_per_s": round(cells * n / (batched_ms * 1e-3) / 1e6, 2),
            "plain_problem_by_problem_mcells_per_s": round(cells * n / (plain_ms * 1e-3) / 1e6, 2),
            "speedup_vs_problem_by_problem": round(plain_ms / batched_ms, 3),
            "percall_problem_by_problem_mcells_per_s": round(cells * n / percall_s / 1e6, 2),
            "speedup_vs_percall_problem_by_problem": round(percall_s * 1e3 / batched_ms, 3),
            "batched_ms": round(batched_ms, 3), "plain_ms": round(plain_ms, 3),
            "percall_ms": round(percall_s * 1e3, 3),
            "schedule": sched, "autotune_s": round(tune_s, 2), "health_flags_nonzero": int(sum(1 for h in health if h))}


# ---------------------------------------------------------------- adjoints

def measure_adjoint(E, a, full_tape: bool = True):
    """dJ/d(initial density) of J = sum rho^2 w (Gaussian of width 0.1 at
    (0.6, 0.6)) on the diagonal-interface problem, FP64 HLLC: the gradient
    (one captured graph: forward sweep, reverse sweep) against the forward
    run alone.  full_tape: the forward sweep keeps every state and its tape
    when they fit in memory; otherwise (and with full_tape False, the
    sqrt(N)-checkpoint method) a state copy every ceil(sqrt(N)) steps and the
    segments recomputed during the reverse sweep."""
    n, ns = a.adjoint_nx, a.adjoint_steps
    p = E.make_params(nx=n, ny=n, gamma0=1.4, cfl=0.8, riemann_solver=E.RIEMANN_HLLC)
    old = os.environ.get("E2D_ADJ_FULL_TAPE")
    os.environ["E2D_ADJ_FULL_TAPE"] = "1" if full_tape else "0"
    try:
        with E.Adjoint(p, arith=a.arith) as A:
            A.gradient(ns, dt_mode=1)  # captures the graph
            grads = []
            for _ in range(3):
                A.gradient(ns, dt_mode=1)
                grads.append(A.last_ms()[1])
            kseg, tape = A.layout()
            fwd = []
            for _ in range(3):
                A.objective(ns)
                fwd.append(A.last_ms()[0])
    finally:
        if old is None:
            os.environ.pop("E2D_ADJ_FULL_TAPE", None)
        else:
            os.environ["E2D_ADJ_FULL_TAPE"] = old
    fd = adjoint_fd_check(E, a, p) if full_tape else None
    g, f = min(grads), min(fwd)
    layout = ("every state and its tape kept by the forward sweep, nothing recomputed" if kseg >= ns
              else f"sqrt(N) checkpoints (every {kseg} steps), segments recomputed during the reverse sweep")
    layout += "" if tape else ", reverse steps recomputing their forward values"
    line = {"workload": f"{n}x{n} FP64 HLLC, {ns} steps, dt through the running CFL maximum, {layout}",
            "segment_steps": kseg, "gradient_ms": round(g, 3), "forward_ms": round(f, 3),
            "adjoint_over_forward": round(g / f, 3),
            "forward_mcells_per_s": round(n * n * ns / (f * 1e-3) / 1e6, 2)}
    if fd is not None:
        line["finite_difference_check"] = fd
    return line


def adjoint_fd_check(E, a, p, eps=1e-6, ndir=2):
    """Central finite differences of J along smooth seeded directions against
    the adjoint's directional derivative, dt frozen (the logged dt of the
    gradient).  The state is the implode state with a 1 % smooth density
    modulation: on the implode state itself the MC limiter (dlft*drgt = 0 on
    its flat sides) and the CFL maximum (every flat cell ties) are not
    differentiable."""
    import numpy as np
    n, ns = a.adjoint_nx, a.adjoint_steps
    with E.HydroRun(p, arith=a.arith) as r:
        r.init_implode()
        u0 = r.get_state(0)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x)
    u0[0, 2:-2, 2:-2] *= 1.0 + 0.01 * np.sin(2 * np.pi * (X + 0.13)) * np.cos(4 * np.pi * Y + 0.3)
    rng = np.random.default_rng(4242)
    errs = []
    with E.Adjoint(p, arith=a.arith) as A:
        _, g, dts = A.gradient(ns, u0, dt_mode=0)
        for _ in range(ndir):
            d = np.zeros((n, n))
            for _ in range(4):
                kx, ky = rng.integers(1, 4, 2)
                d += rng.normal() * np.sin(np.pi * kx * X + rng.uniform(0, 6)) * np.sin(np.pi * ky * Y + rng.uniform(0, 6))
            up, um = u0.copy(), u0.copy()
            up[0, 2:-2, 2:-2] += eps * d
            um[0, 2:-2, 2:-2] -= eps * d
            fdv = (A.objective(ns, up, dt_fixed=dts) - A.objective(ns, um, dt_fixed=dts)) / (2 * eps)
            errs.append(abs(fdv - float(np.sum(g * d))) / abs(fdv))
    return {"max_rel_err": float(max(errs)), "directions": ndir, "eps": eps, "dt": "frozen",
            "state": "implode state with a 1 % smooth density modulation (flat states are not differentiable)"}


def measure_adjoint_batch(E, a):
    """32 seeded problems (sides 256..1024, states and walls as the ensemble
    workload), FP64 HLLC, per-problem gradients from one forward/backward
    graph; the forward-only graph of the same batch beside it."""
    from euler2d_cudafortran_gb300.ensemble import diagonal_ensemble
    ens = diagonal_ensemble(32, 2024, sides=tuple(range(256, 1025, 64)))
    ns = a.adjoint_batch_steps
    init = (ens.offset, ens.rho_hi, ens.p_hi, ens.rho_lo, ens.p_lo)
    with E.AdjointBatch(ens.sizes, ens.bcs, gamma0=1.4, cfl=0.8, arith=a.arith) as B:
        B.init_diagonal(*init)
        B.gradient(ns, dt_mode=1)  # captures the graph
        B.gradient(ns, dt_mode=1)
        g = B.last_ms()[1]
        B.objective(ns)
        B.objective(ns)
        f = B.last_ms()[0]
    cells = ens.cells
    return {"workload": f"32 problems, sides uniform in {{256..1024 step 64}} (total {cells} cells), seed 2024, "
                        f"{ns} steps, dt through the running CFL maximum",
            "gradient_ms": round(g, 3), "forward_ms": round(f, 3), "adjoint_over_forward": round(g / f, 3),
            "gradients_per_s": round(32 / (g * 1e-3), 3),
            "forward_mcells_per_s": round(cells * ns / (f * 1e-3) / 1e6, 2)}


# ---------------------------------------------------------------- our arm

def time_run(E, p, arith, steps, warmup=3, keep=True):
    """Device time (ms) of `steps` steps replayed from a captured graph, after
    `warmup` steps and one untimed pass that captures the graph."""
    old_keep = os.environ.get("E2D_KEEP_PRIMS")
    os.environ["E2D_KEEP_PRIMS"] = "1" if keep else "0"
    try:
        with E.HydroRun(p, arith=arith) as r:
            r.init_implode()
            r.advance(0, warmup, log=False)
            r.advance(warmup, steps, log=False)
            r.advance(warmup + steps, steps, log=False)
            return r.last_advance_ms()
    finally:
        if old_keep is None:
            os.environ.pop("E2D_KEEP_PRIMS", None)
        else:
            os.environ["E2D_KEEP_PRIMS"] = old_keep


def rel_l1(u, ref):
    """Relative L1 difference per conservative variable (interior cells)."""
    import numpy as np
    u, ref = u[:, 2:-2, 2:-2].astype(np.float64), ref[:, 2:-2, 2:-2].astype(np.float64)
    return {k: float(np.abs(u[v] - ref[v]).sum() / np.abs(ref[v]).sum())
            for v, k in enumerate(("rho", "E", "rho_u", "rho_v"))}


def run_ours(a, dist):
    import numpy as np
    import euler2d_cudafortran_gb300 as E
    E.load_library(a.arith)
    cells = a.nx * a.nx
    riemann = E.RIEMANN_HLLC if a.riemann == "hllc" else E.RIEMANN_APPROX
    params = E.make_params(nx=a.nx, ny=a.nx, gamma0=1.4, cfl=0.8, implementation_version=a.version,
                           riemann_solver=riemann, precision=a.precision)
    run = E.HydroRun(params, arith=a.arith)
    run.init_implode()
    # warm-up: W steps (also builds and uploads the graphs)
    run.advance(0, a.warmup, log=False)
    run.advance(a.warmup, a.steps, log=False)  # untimed pass that captures the timed graph
    run.synchronize()
    n0 = a.warmup + a.steps
    dist.barrier()
    device_sync()
    clocks = ClockSampler(dist.local)
    clocks.start()
    dist.barrier()
    device_sync()
    run.advance(n0, a.steps, log=False)
    ms = run.last_advance_ms()
    device_sync()
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(ms)
    value = dist.ws * cells * a.steps / (ms * 1e-3) / 1e6
    n0 += a.steps

    # step-kernel time for the roofline: steps launched one by one with events
    per_step = run.time_steps(n0, 10)
    n0 += 10
    kern_ms = float(np.mean(per_step[1:]))
    hbm_peak, peak_kind = measured_peaks()
    bytes_per_launch = BYTES_PER_CELL[a.precision] * cells
    achieved = bytes_per_launch / (kern_ms * 1e-3) / 1e9
    traffic = profiled_traffic(a.precision, a.nx, a.version, a.arith)
    dfma, ddiv = E.measure_fp64_peak()
    health = run.health()
    run.close()

    # e2e through the C ABI with host buffers, as serial_ref/main.f90 drives the path
    e2e = None
    if not a.no_e2e:
        try:
            import torch
            host_u = torch.empty((4, a.nx + 4, a.nx + 4), dtype=torch.float64 if a.precision == 8 else torch.float32,
                                 pin_memory=True).numpy()
            host_out = torch.empty_like(torch.from_numpy(host_u)).pin_memory().numpy()
        except Exception:
            host_u = np.empty((4, a.nx + 4, a.nx + 4), dtype=np.float64 if a.precision == 8 else np.float32)
            host_out = np.empty_like(host_u)
        with E.HydroRun(params, arith=a.arith) as r2:
            r2.init_implode()
            host_u[...] = r2.get_state(0)
        with E.HydroRun(params, arith=a.arith) as r2:
            # one untimed pass of the same sequence (graph-free path, kernels loaded)
            for rep in range(2):
                dist.barrier()
                device_sync()
                t0 = time.perf_counter()
                r2.set_state(0, host_u)
                r2.compute_dt(0)
                r2.make_boundaries(0)
                for n in range(a.steps):
                    dt = r2.compute_dt(n % 2)
                    r2.godunov_unsplit(n, dt)
                r2.get_state(a.steps % 2, out=host_out)
                device_sync()
                t = time.perf_counter() - t0
            t = dist.max(t)
        sb = host_u.nbytes
        e2e = {"value": round(dist.ws * cells * a.steps / t / 1e6, 3), "unit": "Mcell-updates/s",
               "h2d_bytes_per_step": round(sb / a.steps, 1),
               "d2h_bytes_per_step": round((sb + a.precision * a.steps) / a.steps, 1),
               "sequence": "upload u (pinned) -> per step compute_dt (dt read back) + godunov_unsplit -> "
                           "download final state"}

    # CPU baseline: single-thread restatement of serial_ref on a bounded sample
    cpu = cpu_mc = None
    if dist.rank == 0 and not a.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        t = time_oracle(a, a.cpu_steps, 1)
        cpu = {"value": round(cells * a.cpu_steps / t / 1e6, 3), "unit": "Mcell-updates/s", "cores": 1,
               "kind": "port", "sample": f"{a.nx}x{a.nx}, {a.cpu_steps} steps after 1 warm-up step, single thread: "
                                         "C restatement of serial_ref (-O2 -ffp-contract=off)"}
        nt = os.cpu_count() or 1
        steps_mc = 10
        t = time_oracle(a, steps_mc, nt)
        cpu_mc = {"value": round(cells * steps_mc / t / 1e6, 3), "unit": "Mcell-updates/s", "cores": nt,
                  "kind": "port", "sample": f"{a.nx}x{a.nx}, {steps_mc} steps, OpenMP on the stdpar do-concurrent "
                                            "loops (stand-in for the unavailable -stdpar=multicore build)"}

    # Every build against the FP64 oracle on the headline workload: the exact
    # FP64 build bit for bit, the FMA FP64 build and both FP32 builds by
    # relative L1 per variable and relative dt.
    accuracy = None
    if dist.rank == 0 and not a.no_variants and a.precision == 8:
        from oracle import oracle as O
        O.build()
        po = oracle_params(a)
        ref, dts_ref, _, _ = O.run(po, a.steps, prec="f64", nthreads=os.cpu_count() or 1)
        accuracy = {"workload": f"{a.nx}x{a.nx}, {a.steps} steps, implementationVersion 0, against the FP64 oracle"}
        for arith in ("exact", "fma"):
            for prec in (8, 4):
                p = E.make_params(nx=a.nx, ny=a.nx, gamma0=1.4, cfl=0.8, implementation_version=0,
                                  riemann_solver=riemann, precision=prec)
                u, dts = E.run_steps(a.steps, p, arith=arith)
                dr = float(np.max(np.abs(dts.astype(np.float64) - dts_ref) / dts_ref))
                key = f"{'fp64' if prec == 8 else 'fp32'}_{arith}"
                row = {"rel_l1_per_variable": rel_l1(u, ref), "dt_max_rel": dr}
                if prec == 8:
                    row["bitwise"] = bool(np.array_equal(u[:, 2:-2, 2:-2], ref[:, 2:-2, 2:-2]) and
                                          np.array_equal(dts, dts_ref))
                    row["within_1e-12_l1_1e-14_dt"] = bool(max(row["rel_l1_per_variable"].values()) <= 1e-12
                                                           and dr <= 1e-14)
                accuracy[key] = row
        del ref

    variants = None
    if dist.rank == 0 and not a.no_variants:
        variants = []
        # keep=False: implementationVersion 0 without the primitive arrays kept
        # beside the states (E2D_KEEP_PRIMS=0: every step converts its box, the
        # primitives never leave shared memory)
        rows = [(nx, prec, ver, True, ar) for ar in ("exact", "fma") for nx in (2048, 4096) for prec in (8, 4)
                for ver in (0, 1)]
        rows.insert(1, (2048, 8, 0, False, "exact"))
        for (nx, prec, ver, keep, ar) in rows:
            p = E.make_params(nx=nx, ny=nx, gamma0=1.4, cfl=0.8, implementation_version=ver,
                              riemann_solver=riemann, precision=prec)
            vms = time_run(E, p, ar, a.steps, keep=keep)
            mc = nx * nx * a.steps / (vms * 1e-3) / 1e6
            gbs = mc * 1e6 * BYTES_PER_CELL[prec] / 1e9
            row = {"nx": nx, "precision": "FP64" if prec == 8 else "FP32", "implementationVersion": ver,
                   "arith": ar, "steps": a.steps, "mcells_per_s": round(mc, 2),
                   "hbm": {"bytes_per_cell": BYTES_PER_CELL[prec], "achieved_gbs": round(gbs, 1),
                           "frac": round(gbs / hbm_peak, 5)}}
            if ver == 0:
                row["primitives_kept"] = keep
            inst = profiled_value(prec, nx, ver, "thread_inst_per_cell", ar)
            if inst and prec == 4 and clk.get("sm_mhz"):
                # FP32 is bound by instruction issue: 4 schedulers x 32 lanes per SM per clock
                issue_peak = 152 * 4 * 32 * clk["sm_mhz"] * 1e6
                row["binding_roof"] = {"roof": "instruction issue", "thread_inst_per_cell": inst,
                                       "frac": round(inst * mc * 1e6 / issue_peak, 4),
                                       "frac_of": "152 SMs x 4 schedulers x 32 lanes x the sampled SM clock"}
            fp64_inst = profiled_value(prec, nx, ver, "fp64_warp_inst_per_launch", ar)
            if fp64_inst and prec == 8:
                inst_s = 32 * fp64_inst / (nx * nx) * mc * 1e6
                row["binding_roof"] = {"roof": "fp64 pipe", "fp64_inst_per_cell": round(32 * fp64_inst / (nx * nx), 1),
                                       "frac": round(inst_s / dfma, 4), "frac_of": "the live DFMA probe"}
            variants.append(row)

    batched = None
    if dist.rank == 0 and not a.no_batched:
        batched = measure_batched(E, a)
        single = value / dist.ws
        batched["ceiling"] = {
            "single_run_mcells_per_s": round(single, 2),
            "fraction_of_single_run": round(batched["mcells_per_s"] / single, 4),
            "note": "both the ensemble and the single run are bound by the FP64 pipe, so the single run's rate on "
                    "the largest grid is the ensemble's ceiling; batching can only recover the small-problem tail"}
        if a.precision == 8:
            inst = profiled_value(8, 2048, 0, "fp64_warp_inst_per_launch", a.arith)
            if inst:
                per_cell = 32 * inst / (2048 * 2048)
                batched["ceiling"]["fp64_pipe_frac"] = round(per_cell * batched["mcells_per_s"] * 1e6 / dfma, 4)
    adjoint = adjoint_ckpt = adjoint_batch = None
    if dist.rank == 0 and not a.no_adjoint:
        adjoint = measure_adjoint(E, a, full_tape=True)
        adjoint_ckpt = measure_adjoint(E, a, full_tape=False)
        if a.adjoint_batch_steps > 0:
            adjoint_batch = measure_adjoint_batch(E, a)

    fp64_roof = {"pipe": "fp64", "dfma_per_s": dfma, "ddiv_per_s": ddiv,
                 "note": "the FP64 step is bound by the FP64 pipe (two Riemann solves, traces, slopes per cell), "
                         "not by HBM"}
    warp_inst = profiled_value(a.precision, a.nx, a.version, "fp64_warp_inst_per_launch", a.arith)
    if warp_inst and a.precision == 8 and a.riemann == "hllc":
        inst_s = 32 * warp_inst / (kern_ms * 1e-3)  # FP64 thread instructions per second, this run
        fp64_roof.update({"fp64_inst_per_cell": round(32 * warp_inst / (a.nx * a.nx), 1),
                          "achieved_per_s": inst_s, "frac": round(inst_s / dfma, 4),
                          "frac_of": "the live DFMA probe (independent FP64 instructions per second)"})
    if dist.rank == 0:
        isz = a.nx + 4
        line = {
            "metric": "Mcell-updates/s", "value": round(value, 3), "unit": "Mcell-updates/s",
            "n_gpus": dist.ws, "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms / a.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if a.precision == 8 else "f32", "data": "synthetic",
            "config": bench_config(a, dist.ws),
            "arith": a.arith,
            "value_reference_formula": round(dist.ws * isz * isz * a.steps / (ms * 1e-3) / 1e6, 3),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm_peak, "unit": "GB/s",
                         "frac": round(achieved / hbm_peak, 5), "peak_kind": peak_kind,
                         "traffic": traffic,
                         "bytes_per_launch": bytes_per_launch, "kernel_ms": round(kern_ms, 4),
                         "binding_roof": fp64_roof},
            "e2e": e2e,
            "cpu_baseline": cpu,
            "cpu_baseline_multicore": cpu_mc,
            "clocks": clk,
            # timed advance call: make_boundaries, (version 0 with kept primitives) the
            # primitives of both buffers, then the steps
            "gpu_launches": (a.steps + 1 + (0 if os.environ.get("E2D_KEEP_PRIMS") == "0" else 2)
                             if a.version == 0 else 4 * a.steps),
            "health_flags": health,
            "accuracy_vs_fp64_oracle": accuracy,
            "variants": variants,
            "batched": batched,
            "adjoint": adjoint,
            "adjoint_checkpointed": adjoint_ckpt,
            "adjoint_batched": adjoint_batch,
        }
        print(json.dumps(line), flush=True)

def main():
    a = parse_args()
    ws, rank, local = dist_info()
    if ws > 1:
        # one GPU per rank, visible to both this process's CUDA runtimes
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = Dist()
    try:
        if a.impl == "reference":
            run_reference(a, dist)
        else:
            run_ours(a, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
