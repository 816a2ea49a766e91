#!/usr/bin/env python
"""bench.py -- field-point z-steps/s of the gsolver_solid_qdht z-step on GB300.

A "step" is one accepted propagator() call (RK4 nonlinear increment, forward QDHT with
the fused linear step, inverse QDHT) on the 1024 x 16384 fused-silica workload
(R = 1.2 mm, 1.6 ps window, collimated 800 nm 50 fs 3 P_cr pulse, adaptive dz with
MAX_TOLERANCE 1e-6), set up by the library's own C++ from a reference-format config.
Synthetic: the pulse is generated (seeded 1e-4 complex Gaussian noise), no dataset.

  value   device throughput (inputs resident in HBM), CUDA events on the handle's stream
  e2e     the same metric through the public C ABI with pinned host buffers: every step
          copies FIELD and BIGBUFFER2 in and out (the host globals propagator() works on),
          gs_step_host (BIGBUFFER2's copy in overlapping the NL attempt)
  fp64    the plain FP64 GPU path on the same workload, and the mixed path's relative L2
          error against it after 5, 100, 1000 and 2000 fixed-dz steps from the same start
  roofline  the dominant kernel, nl_row16k_kernel (the four RK4 stages of every row in one
          launch): the NL increment's algorithmic bytes, 16 B per field point (read FIELD,
          write BIGBUFFER1, complex64), over its CUDA-event launch time; its DRAM traffic and
          instruction counts from an ncu capture of one launch of this workload (the kernel
          is bound by SM instruction issue, not by HBM); roofline_qdht the tensor-core QDHT,
          algorithmic 8 N_r flop per field-point step
  adjoint the gradient workload (256 x 4096, 1000 steps): forward vs forward+adjoint time
          and the gradient's accuracy (see adjoint_leg)
  batch   64 pulses with uneven grids, one CUDA graph launch per z-step (see batch_leg), and
          the same grids with every pulse's adaptive controller on the device, one graph launch
          per attempt (gs_batch_advance, batch.adaptive)
  argon   16 argon pulses on the gas build (PPT, third harmonic), 512 x 32768 (see argon_leg),
          fixed steps and adaptive (argon.adaptive)
  cpu_baseline  the CPU oracle (a port of the reference algorithm) on a bounded sample

Multi-GPU: replicas only (one independent pulse per rank), value = total / max time.
``--impl reference`` times the reference algorithm's CPU implementation (the oracle port,
the reference itself needs MPI/FFTW/GSL) on the host cores, same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "field-point z-steps/s"
UNIT = "field-point z-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "c2r256", "c2r512"])
    ap.add_argument("--only", default=None, choices=["adjoint", "batch", "argon"],
                    help="run one leg alone and print its JSON object (profiling captures)")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--err-steps", default="5,100,1000,2000",
                    help="step counts at which the mixed path's error against FP64 is recorded")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-argon", action="store_true")
    ap.add_argument("--argon-pulses", type=int, default=16)
    ap.add_argument("--argon-steps", type=int, default=5)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--batch-pulses", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--batch-adaptive-calls", type=int, default=8,
                    help="accepted propagator() calls per pulse in the batch leg's adaptive part (0: skip it)")
    ap.add_argument("--adjoint-steps", type=int, default=1000)
    ap.add_argument("--adjoint-check-steps", type=int, default=100)
    ap.add_argument("--adjoint-dirs", type=int, default=2,
                    help="seeded random directions of the finite-difference check (the full check: 32 over 1000 steps)")
    return ap.parse_args()


def dist_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return r, w, lr


def whole_job(ms_local, units_per_rank, world):
    """Replicas: every rank advanced its own pulse (units_per_rank field-point z-steps) in
    ms_local; the job's time is the slowest rank's and its value all ranks' units over that
    time.  Returns (ms, value).  Under torch.distributed (world > 1) the max is an all-reduce
    over the process group (NCCL on GPUs, gloo on CPU)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(ms_local)], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_local = float(t.item())
    return ms_local, units_per_rank * world / (ms_local / 1e3)


def make_config(workload):
    from gsolver_gb300 import configs
    d = tempfile.mkdtemp(prefix="gs_bench_")
    if workload == "c2":
        return configs.fused_silica_c2(d), {"workload": "fused_silica_1024x16384", "n_r": 1024, "n_t": 16384,
                                             "r_max_m": 1.2e-3, "window_s": 1.6e-12, "z_max_m": 3e-3,
                                             "max_tolerance": 1e-6}
    if workload in ("c2r256", "c2r512"):
        nr = int(workload[3:])
        return configs.fused_silica_c2_rows(d, nr), {"workload": f"fused_silica_{nr}x16384 (profiling case)",
                                                     "n_r": nr, "n_t": 16384, "r_max_m": 1.2e-3 * nr / 1024,
                                                     "window_s": 1.6e-12, "z_max_m": 3e-3, "max_tolerance": 1e-6}
    return configs.fused_silica_c1(d), {"workload": "fused_silica_256x2048", "n_r": 256, "n_t": 2048,
                                         "r_max_m": 6e-4, "window_s": 4e-13, "z_max_m": 1e-3,
                                         "max_tolerance": 1e3}


class Clocks:
    """nvidia-smi sampler (200 ms) running during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = tempfile.mktemp(prefix="gs_clocks_", suffix=".csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 8:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[4:8]) if v.lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def run_z_steps(P, S, state, k):
    """k accepted propagator() calls continuing the z-loop (solver_main.cpp:202-225), through
    gs_advance: the step controller on the device, no host round trip per call (the workload's
    kernels read their step sizes from device memory; gs_step gives the same results bit for
    bit, tests/test_gpu_advance.py)."""
    znet = S["znet"]
    while k > 0:
        cz, n_z, zstep, step_n = state["z"], state["n_z"], state["zstep"], state["step_n"]
        if cz >= znet[n_z]:
            if n_z == len(znet) - 1:
                raise RuntimeError("workload ran past its last ZNET point")
            n_z += 1
        cz, zstep, step_n, calls, _ = P.advance(znet, n_z, cz, zstep, step_n, k)
        state.update(z=cz, n_z=n_z, zstep=zstep, step_n=step_n)
        k -= calls


def new_state(S):
    return {"z": float(S["znet"][0]), "n_z": 0, "zstep": float(S["init_zstep"]), "step_n": 0}


# Per field point of one launch on the 1024 x 16384 workload, from ncu captures of that
# workload (dram__bytes_read.sum + dram__bytes_write.sum, smsp__inst_executed.sum and
# smsp__issue_active.avg.pct_of_peak_sustained_active of one launch, divided by its n_r n_t field
# points); they are fixed properties of the kernels, re-measured whenever a kernel changes.
NCU_PER_POINT = {
    "nl_row16k": {"dram_bytes": 2.37, "warp_instructions": 30.1, "issue_active": 0.597},
    "qdht_pair": {"dram_bytes": 9.13},
}


def window_columns(S):
    """Real columns (2 per omega) inside calculate_Lstep's window: omega in [min, max] and some
    kt^2 <= Re(k^2) / 4 -- the columns the tensor-core QDHT transforms (propagator.cu:570-625)."""
    om = np.asarray(S["omega"])
    k = np.asarray(S["wavenum"])
    kt2 = np.asarray(S["kt2"])
    inwin = ~((om < S["omega_min"]) | (om > S["omega_max"]))
    lim = 0.25 * (k.real ** 2 - k.imag ** 2)
    return int(2 * np.count_nonzero(inwin & (kt2.min() <= lim)))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), d.get("bf16_tflops"), d.get("bf16_tflops_sustained"), "measured"
    except OSError:
        return 6800.0, 1900.0, 1700.0, "fallback"


def cpu_prepare(cfg_path):
    """Oracle set-up of the workload (numpy restatement of the reference start-up)."""
    from oracle import oracle, tables
    oracle.build()
    return tables.build(tables.Config.from_file(cfg_path), noise_seed=1234, noise_sigma=1e-4)


def cpu_sample(T, nthreads=None):
    """Oracle on the host cores: one RK4 NL step + linear step on a quarter of the rows
    and both QDHTs on a quarter of the omega columns of the full grid, extrapolated to a
    full step.  Returns (value, description, cores)."""
    from oracle import oracle, tables
    nr, nt = T["n_r"], T["n_t"]
    cores = nthreads or os.cpu_count() or 1
    rows = list(np.linspace(0, nr - 1, min(nr, max(2 * cores, nr // 4))).astype(int))
    Ts = dict(T)
    Ts["n_r"] = len(rows)
    Ts["kt2"] = T["kt2"][rows]
    O_rows = oracle.Oracle(Ts, nthreads=cores)
    sub = np.ascontiguousarray(T["field"][rows])
    dz = tables.init_zstep_kerr(T, T["field"])
    t0 = time.perf_counter()
    bb1, _, _ = O_rows.nl_step(sub, dz)
    O_rows.lstep(bb1, sub, dz)
    t_rows = time.perf_counter() - t0
    cols = min(nt, max(32 * cores, nt // 4))
    data = np.ascontiguousarray(T["field"][:, :cols])
    Tq = dict(T)
    Tq["n_t"] = cols
    Oq = oracle.Oracle(Tq, nthreads=cores)
    t0 = time.perf_counter()
    d1 = Oq.qdht(data)
    Oq.qdht(d1)
    t_cols = time.perf_counter() - t0
    t_step = t_rows * nr / len(rows) + t_cols * nt / cols
    desc = (f"oracle (C port of the reference z-step, agreeing with the reference solver itself to 1e-12 on every "
            f"hot-path function; OpenMP {cores} threads, radix-4 Stockham FFT): RK4 NL step + "
            f"linear step on {len(rows)} of {nr} rows, forward+inverse QDHT on {cols} of {nt} omega columns, "
            f"extrapolated to one {nr}x{nt} step ({t_step:.2f} s)")
    return nr * nt / t_step, desc, cores


def reference_arm(args, rank, world):
    if rank != 0:
        return
    cfg, conf = make_config(args.workload)
    T = cpu_prepare(cfg)
    vals = []
    desc, cores = "", 1
    for i in range(args.warmup + args.steps):
        v, desc, cores = cpu_sample(T)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": conf,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batch_leg(args, lrank):
    """The batched scan: 64 fused-silica pulses with uneven grids (N_r 128-512, N_t
    1024-8192) and parameters drawn from a seed, mixed precision, fixed 2 um steps; one CUDA
    graph launch advances every pulse one z-step.  Aggregate field-point z-steps/s over the
    batch (CUDA events on the batch stream), with and without the graph."""
    import torch
    import gsolver_gb300 as gs
    from gsolver_gb300 import configs
    d = tempfile.mkdtemp(prefix="gs_bench_batch_")
    cfgs = configs.c3_batch(d, seed=0, n=args.batch_pulses)
    t0 = time.perf_counter()
    S = [gs.Setup(p, noise_seed=100 + i, noise_sigma=1e-4, device=lrank).as_dict() for i, (p, _) in enumerate(cfgs)]
    t_setup = time.perf_counter() - t0                  # device set-up (gs_setup_from_config_dev)
    t0 = time.perf_counter()
    for i, (p, _) in enumerate(cfgs):
        gs.Setup(p, noise_seed=100 + i, noise_sigma=1e-4)
    t_setup_host = time.perf_counter() - t0             # the same on the host, for comparison
    P = [gs.Propagator(s, precision=gs.PREC_MIXED, device=lrank) for s in S]
    for s, p in zip(S, P):
        p.set_field(s["field"])
    B = gs.Batch(P)
    dz = np.array([float(s["init_zstep"]) for s in S])
    tuned = None
    if not args.no_autotune:
        # default shapes vs every grid's own tuned shape, timed on the whole batch
        ms_def, ms_tun, chose = B.autotune(dz)
        tuned = {"ms_per_zstep_default": ms_def, "ms_per_zstep_tuned_per_grid": ms_tun,
                 "chosen": "tuned per grid" if chose else "default",
                 "threads": {f"{s['n_r']}x{s['n_t']}": p.nl_threads() for s, p in zip(S, P)}}
    pts = sum(s["n_r"] * s["n_t"] for s in S)
    stream = torch.cuda.ExternalStream(B.stream_ptr(), device=lrank)
    out = {"workload": f"fused_silica_batch{len(P)}", "pulses": len(P), "points_per_zstep": pts,
           "grids": sorted({(s["n_r"], s["n_t"]) for s in S}), "precision": "mixed", "dz_m": 2e-6,
           "setup_s_device": t_setup, "setup_s_host": t_setup_host, "autotune": tuned or "off"}
    for graph in (True, False):
        B.step(dz, 2, graph=graph)   # warm-up (and graph capture)
        n0 = B.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e0.record(stream)
        B.step(dz, args.batch_steps, graph=graph)
        e1.record(stream)
        e1.synchronize()
        wall = time.perf_counter() - t1
        ms = e0.elapsed_time(e1)
        key = "graph" if graph else "streams"
        out[key] = {"value": pts * args.batch_steps / (ms / 1e3), "unit": UNIT, "ms_per_zstep": ms / args.batch_steps,
                    "wall_ms_per_zstep": wall * 1e3 / args.batch_steps, "steps": args.batch_steps,
                    "kernels_per_zstep": (B.launch_count() - n0) / args.batch_steps}
    B.close()
    for p in P:
        p.close()
    if args.batch_adaptive_calls > 0:
        out["adaptive"] = batch_adaptive(args, lrank, cfgs)
    return out


def batch_adaptive(args, lrank, cfgs):
    """The same 64 grids with each pulse's adaptive controller at MAX_TOLERANCE 1e-6 (the
    workload's own 1e3 lets ZNET clamp every step to 2 um), on the device: gs_batch_advance, one
    graph launch per attempt of all pulses, rejected attempts included; accepted field-point
    z-steps/s over the batch, wall clock of the call (graph capture and the host reads of the
    pulses' states included)."""
    import gsolver_gb300 as gs
    S = [gs.Setup(p, overrides={"MAX_TOLERANCE": "1e-6"}, noise_seed=100 + i, noise_sigma=1e-4, device=lrank).as_dict()
         for i, (p, _) in enumerate(cfgs)]
    P = [gs.Propagator(s, precision=gs.PREC_MIXED, device=lrank) for s in S]
    for s, p in zip(S, P):
        p.set_field(s["field"])
    B = gs.Batch(P)
    znets = [s["znet"] for s in S]
    n = len(P)
    cz = np.array([float(z[0]) for z in znets])
    dz = np.array([float(s["init_zstep"]) for s in S])
    sn = np.zeros(n, np.uint32)
    nz = [1] * n
    cz, dz, sn, _, _ = B.advance(znets, nz, cz, dz, sn, 2)   # warm-up: the first calls find each NL path
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cz1, dz1, sn1, calls, reached = B.advance(znets, nz, cz, dz, sn, args.batch_adaptive_calls)
    wall = time.perf_counter() - t0
    pts = sum(s["n_r"] * s["n_t"] * int(c) for s, c in zip(S, calls))
    attempts = int(np.sum(sn1 - sn))
    out = {"max_tolerance": 1e-6, "calls_per_pulse": args.batch_adaptive_calls, "accepted_calls": int(np.sum(calls)),
           "attempts": attempts, "rejected": attempts - int(np.sum(calls)), "value": pts / wall, "unit": UNIT,
           "ms_per_call_of_all_pulses": wall * 1e3 / max(1, args.batch_adaptive_calls),
           "api": "gs_batch_advance (every pulse's controller on the device, one graph launch per attempt)"}
    B.close()
    for p in P:
        p.close()
    return out


def argon_leg(args, lrank):
    """The gas workload: 16 argon pulses (gas build: PPT ionization, third harmonic) at
    512 x 32768, 3.9 um 80 fs w0 = 1 mm 4 P_cr, CEP swept over [0, 2 pi), mixed precision,
    one CUDA graph launch per z-step with each pulse's first controller step as its fixed
    dz; and the mixed path's field error against the FP64 path on one pulse after 3 steps."""
    import torch
    import gsolver_gb300 as gs
    from gsolver_gb300 import configs
    d = tempfile.mkdtemp(prefix="gs_bench_ar_")
    n = args.argon_pulses
    t0 = time.perf_counter()
    S = []
    for i in range(n):
        p = configs.argon_c5(d, cep=2 * np.pi * i / n, name=f"argon_c5_{i:02d}", build="gas_qdht")
        S.append(gs.Setup(p, noise_seed=200 + i, noise_sigma=1e-4, device=lrank).as_dict())
    t_setup = time.perf_counter() - t0                  # device set-up (gs_setup_from_config_dev)
    P = [gs.Propagator(s, precision=gs.PREC_MIXED, device=lrank) for s in S]
    for s, p in zip(S, P):
        p.set_field(s["field"])
    B = gs.Batch(P)
    dz = np.array([float(s["init_zstep"]) for s in S])
    pts = sum(s["n_r"] * s["n_t"] for s in S)
    stream = torch.cuda.ExternalStream(B.stream_ptr(), device=lrank)
    B.step(dz, 2, graph=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    B.step(dz, args.argon_steps, graph=True)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    out = {"workload": f"argon_gas_batch{n}", "build": "gas_qdht (PPT, third harmonic, IONRATE_DENOM 1e10)",
           "pulses": n, "n_r": 512, "n_t": 32768, "points_per_zstep": pts, "precision": "mixed",
           "dz_m": float(dz[0]), "setup_s_device": t_setup, "value": pts * args.argon_steps / (ms / 1e3),
           "unit": UNIT, "ms_per_zstep": ms / args.argon_steps, "steps": args.argon_steps,
           "path": "pair kernels (each row of 32768 over two CTAs)"}
    B.close()
    for p in P:
        p.close()
    # mixed vs FP64 on pulse 0, 3 steps of its first dz
    fields = []
    for prec in (gs.PREC_MIXED, gs.PREC_FP64):
        Q = gs.Propagator(S[0], precision=prec, device=lrank)
        Q.set_field(S[0]["field"])
        for _ in range(3):
            Q.nl_step(float(dz[0]))
            Q.lstep(float(dz[0]))
        fields.append(Q.get_field(want_spec=False))
        Q.close()
    out["mixed_rel_l2_field_err_vs_fp64"] = float(np.linalg.norm(fields[0] - fields[1]) / np.linalg.norm(fields[1]))
    out["err_steps"] = 3
    if args.batch_adaptive_calls > 0:
        # the same pulses with their own adaptive controllers (MAX_TOLERANCE 1e-3) on the device:
        # gs_batch_advance, one graph launch per attempt of all 16 pulses; wall clock of the call
        P = [gs.Propagator(s, precision=gs.PREC_MIXED, device=lrank) for s in S]
        for s, p in zip(S, P):
            p.set_field(s["field"])
        B = gs.Batch(P)
        znets = [s["znet"] for s in S]
        cz = np.array([float(z[0]) for z in znets])
        dz0 = np.array([float(s["init_zstep"]) for s in S])
        sn = np.zeros(n, np.uint32)
        cz, dz0, sn, _, _ = B.advance(znets, [1] * n, cz, dz0, sn, 1)   # warm-up: each NL path found
        K = max(1, args.batch_adaptive_calls // 2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, _, sn1, calls, _ = B.advance(znets, [1] * n, cz, dz0, sn, K)
        wall = time.perf_counter() - t0
        acc = int(np.sum(calls))
        out["adaptive"] = {"max_tolerance": 1e-3, "calls_per_pulse": K, "accepted_calls": acc,
                           "attempts": int(np.sum(sn1 - sn)), "value": S[0]["n_r"] * S[0]["n_t"] * acc / wall,
                           "unit": UNIT, "ms_per_call_of_all_pulses": wall * 1e3 / K,
                           "api": "gs_batch_advance (every pulse's controller on the device, one graph launch per attempt)"}
        B.close()
        for p in P:
            p.close()
    return out


def adjoint_leg(args, lrank):
    """The adjoint workload: fused silica 256 x 4096, 2 mm in 1000 fixed 2 um steps, seeded
    degree-6 spectral phase on the input, J = energy in the 500-600 nm band (average_spectrum
    radial weights).  Times gs_forward_fixed and gs_gradient (forward + checkpointed adjoint,
    the default stride: every step recorded when it fits in memory) on the mixed path, both through the C ABI with host fields, and checks the
    gradient on the first `adjoint_check_steps` steps against the FP64 adjoint and fourth-order
    central differences of the FP64 forward along the FP64 gradient and `adjoint_dirs` seeded
    random directions (max and median relative errors over those)."""
    import gsolver_gb300 as gs
    from gsolver_gb300 import configs
    d = tempfile.mkdtemp(prefix="gs_bench_adj_")
    S = gs.Setup(configs.fused_silica_c4(d), noise_seed=1234, noise_sigma=1e-4).as_dict()
    A0 = S["field"] * np.exp(1j * configs.spectral_phase(S["omega"], S["omega0"], 50e-15, seed=4))[None, :]
    w = configs.band_weights(S["omega"], S["qdht_x"], S["r_max"], 500e-9, 600e-9)
    n = args.adjoint_steps
    rk, lin = configs.clamp_schedule(S["znet"], S["init_zstep"], n)
    Pm = gs.Propagator(S, precision=gs.PREC_MIXED, device=lrank)
    Pm.set_field(A0)
    tuned = None if args.no_autotune else Pm.autotune()

    def timed(f, reps=2):
        f()   # warm-up: allocations, transposed-QDHT set-up
        t0 = time.perf_counter()
        for _ in range(reps):
            r = f()
        return (time.perf_counter() - t0) / reps * 1e3, r

    tf, (J, _) = timed(lambda: Pm.forward_fixed(A0, rk, lin, w))
    tg, (Jg, gm) = timed(lambda: Pm.gradient(A0, rk, lin, w))
    stride = Pm.adjoint_stride()
    ks = int(np.ceil(np.sqrt(n)))   # the sqrt(N) checkpointing: segments re-run from checkpoints
    tk, (_, gk) = timed(lambda: Pm.gradient(A0, rk, lin, w, checkpoint_stride=ks), reps=1)
    out = {"workload": "fused_silica_256x4096_adjoint", "n_r": 256, "n_t": 4096, "steps": n, "dz_m": 2e-6,
           "objective": "band energy 500-600 nm, average_spectrum radial weights",
           "checkpoint_stride": stride, "precision": "mixed",
           "nl_threads_per_row": tuned[0] if tuned else "default",
           "forward_ms": tf, "gradient_ms": tg, "cost_ratio": tg / tf,
           "sqrt_stride": {"checkpoint_stride": ks, "gradient_ms": tk, "cost_ratio": tk / tf,
                           "max_abs_diff_vs_default": float(np.abs(gk - gm).max() / np.abs(gm).max())},
           "note": "gradient_ms = forward + adjoint (one gs_gradient call); cost_ratio = gradient / forward; "
                   "sqrt_stride: the same gradient with checkpoints every ceil(sqrt(steps)) steps"}
    m = args.adjoint_check_steps
    if m > 0:
        P64 = gs.Propagator(S, precision=gs.PREC_FP64, device=lrank)
        J64, g64 = P64.gradient(A0, rk[:m], lin[:m], w)
        _, gmm = Pm.gradient(A0, rk[:m], lin[:m], w)
        h = 1e-5
        Jf = lambda A: P64.forward_fixed(A, rk[:m], lin[:m], w)[0]
        chk = {"steps": m, "grad_rel_l2_mixed_vs_fp64": float(np.linalg.norm(gmm - g64) / np.linalg.norm(g64)),
               "fd": "fourth-order central differences of the FP64 forward, h = 1e-5, along the FP64 gradient "
                     "(well conditioned) and along seeded random directions (complex Gaussian, seeds 11 + k)"}

        def fd_check(v):
            v = v * (np.linalg.norm(A0) / np.linalg.norm(v))
            fd = (-Jf(A0 + 2 * h * v) + 8 * Jf(A0 + h * v) - 8 * Jf(A0 - h * v) + Jf(A0 - 2 * h * v)) / (12 * h)
            d64 = float(np.sum((np.conj(g64) * v).real))
            dm = float(np.sum((np.conj(gmm) * v).real))
            # conditioning |g||v| / |<g, v>|: a gradient error e (relative L2) moves the
            # directional derivative by up to e times this
            cond = float(np.linalg.norm(g64) * np.linalg.norm(v) / abs(d64))
            return abs(d64 - fd) / abs(fd), abs(dm - fd) / abs(fd), cond

        e64, em, cd = fd_check(g64)
        chk["gradient_dir"] = {"fd_rel_err_fp64": e64, "fd_rel_err_mixed": em, "conditioning": cd}
        res = []
        for k in range(args.adjoint_dirs):
            r = np.random.default_rng(11 + k)
            res.append(fd_check(r.standard_normal(A0.shape) + 1j * r.standard_normal(A0.shape)))
        if res:
            a = np.asarray(res)
            stat = lambda x: {"max": float(np.max(x)), "median": float(np.median(x))}
            chk["random_dirs"] = {"n": len(res), "fd_rel_err_fp64": stat(a[:, 0]), "fd_rel_err_mixed": stat(a[:, 1]),
                                  "conditioning": stat(a[:, 2])}
        out["check"] = chk
        P64.close()
    Pm.close()
    return out


def main():
    args = parse()
    rank, world, lrank = dist_info()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    import torch
    import gsolver_gb300 as gs
    if args.only:
        torch.cuda.set_device(lrank)
        leg = {"adjoint": adjoint_leg, "batch": batch_leg, "argon": argon_leg}[args.only](args, lrank)
        if rank == 0:
            print(json.dumps({args.only: leg}), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(lrank)
    cfg, conf = make_config(args.workload)
    S = gs.Setup(cfg, noise_seed=1234 + rank, noise_sigma=1e-4).as_dict()
    nr, nt = S["n_r"], S["n_t"]
    prec = gs.PREC_MIXED if args.precision == "mixed" else gs.PREC_FP64
    try:
        P = gs.Propagator(S, precision=prec, device=lrank)
    except gs.GsError as e:
        if prec == gs.PREC_MIXED:
            print(f"# mixed path unavailable ({e}); timing the FP64 path", file=sys.stderr)
            prec = gs.PREC_FP64
            P = gs.Propagator(S, precision=prec, device=lrank)
        else:
            raise
    P.set_field(S["field"])
    tuned = None if args.no_autotune else P.autotune()   # fused NL launch shape (threads per row)
    state = new_state(S)
    run_z_steps(P, S, state, args.warmup)
    stream = torch.cuda.ExternalStream(P.stream_ptr(), device=lrank)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    P.qdht_timing(enable=True)
    P.nl_timing(enable=True)
    n0 = P.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(lrank) as clk:
        e0.record(stream)
        run_z_steps(P, S, state, args.steps)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = P.launch_count() - n0
    q_ms, q_n = P.qdht_timing(enable=False)
    st_ms, n_st, n_launch = P.nl_timing(enable=False)
    ms, value = whole_job(ms, nr * nt * args.steps, world)

    # roofline: the QDHT (forward + fused linear step, inverse), 2 N_r^2 flop per real column
    # of the spectral window each: outside it the linear step leaves BIGBUFFER2 untouched and
    # the masked inverse transforms zero columns, so neither is computed there
    hbm, bf16, bf16s, pk_kind = peaks()
    ncol_win = window_columns(S)
    flop_launch = 2.0 * nr * nr * ncol_win
    per_launch_ms = q_ms / max(q_n, 1)
    achieved = flop_launch / (per_launch_ms / 1e3) / 1e12 if q_n else None
    qt = NCU_PER_POINT["qdht_pair"]["dram_bytes"]
    roof_q = {"bound": "tensor", "kernel": "qdht_tc2 (split + GEMM)" if prec == gs.PREC_MIXED else "qdht64 (FP64 CUDA cores)",
              "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
              "frac": (achieved / bf16) if achieved else None,
              "traffic": (qt * nr * nt / 2) if (qt and prec == gs.PREC_MIXED) else None,
              "peak_kind": f"{pk_kind} cuBLAS bf16 burst", "launch_ms": per_launch_ms,
              "qdht_share_of_step": (q_ms / ms) if ms else None,
              "window_columns": ncol_win, "columns": 2 * nt,
              "note": "algorithmic flop 2 N_r^2 per real column of the spectral window per transform (launch_ms is "
                      "one transform: split, factor table when dz changes, GEMM); the split FP16 operands execute 3 "
                      "products (Hh Xh + Hh Xl + Hl Xh) at the FP16 rate, which equals the bf16 rate of the peak"}
    # the dominant kernel: nl_row16k_kernel (16384-point FP32 rows) or nl_stage4_kernel, one launch
    # per NL step (all four RK4 stages of a row in one CTA), or nl_stage_kernel once per stage on
    # smaller grids; algorithmic bytes per step
    # 16 per field point (read FIELD, write the NL increment BIGBUFFER1, complex64)
    esz = 8 if prec == gs.PREC_MIXED else 16
    four = n_st and n_launch < n_st
    step_ms_nl = st_ms / n_st * 4 if n_st else None
    nl_bytes = 2 * esz * nr * nt
    nl_ach = nl_bytes / (step_ms_nl / 1e3) / 1e9 if step_ms_nl else None
    ncu4 = NCU_PER_POINT["nl_row16k"]
    r16 = four and nt == 16384 and prec == gs.PREC_MIXED   # the shape the ncu figures describe
    kname = ("nl_row16k_kernel" if r16 else "nl_stage4_kernel") if four else "nl_stage_kernel"
    roof = {"bound": "hbm", "kernel": kname if n_st else "staged NL kernels (not timed)",
            "achieved": nl_ach, "peak": hbm, "unit": "GB/s", "frac": (nl_ach / hbm) if nl_ach and hbm else None,
            "traffic": (ncu4["dram_bytes"] * nr * nt) if r16 else None,
            "peak_kind": f"{pk_kind} HBM copy", "launch_ms": step_ms_nl,
            "algorithmic_bytes_per_launch": nl_bytes,
            "share_of_step": (st_ms / ms) if ms and n_st else None,
            "limiter": ({"kind": "SM instruction issue",
                         "warp_instructions_per_field_point": ncu4["warp_instructions"],
                         "issue_active_frac": ncu4["issue_active"]} if r16 else None),
            "note": "per NL step (one launch of all four RK4 stages), CUDA events around each launch on the handle's "
                    "stream; algorithmic bytes 16 per field point (FIELD in, BIGBUFFER1 out, complex64); traffic and "
                    "the limiter figures from an ncu capture of one launch of this workload"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+fp16x2" if prec == gs.PREC_MIXED else "f64",
            "data": "synthetic (seeded Gaussian pulse + 1e-4 complex noise; no dataset)",
            "config": dict(conf, precision="mixed" if prec == gs.PREC_MIXED else "fp64",
                           parallelism=f"replicas{world}", l2="inputs larger than L2 (state ~1 GB per pulse)",
                           z_reached_m=state["z"], dz_last_m=state["zstep"],
                           nl_threads_per_row=tuned[0] if tuned else "default"),
            "gpu_launches": launches, "roofline": roof, "roofline_qdht": roof_q,
            "clocks": clk.summary()}

    # e2e through the public API with pinned host buffers: propagator() on host-resident FIELD
    # and BIGBUFFER2 (gs_step_host: both in, one call's attempts, both out); also the same
    # through three calls (gs_set_field + gs_advance + gs_get_field), without the overlap
    if not args.no_e2e:
        f_h = torch.empty((nr, nt), dtype=torch.complex128, pin_memory=True)
        s_h = torch.empty((nr, nt), dtype=torch.complex128, pin_memory=True)
        P.get_field_ptr(f_h.data_ptr(), s_h.data_ptr())
        ke = max(2, min(args.steps, 10))
        znet = S["znet"]

        def host_call():
            if state["z"] >= znet[state["n_z"]]:
                if state["n_z"] == len(znet) - 1:
                    raise RuntimeError("workload ran past its last ZNET point")
                state["n_z"] += 1
            n_z = state["n_z"]
            zstep, step_n = P.step_host(f_h.data_ptr(), s_h.data_ptr(), state["z"], znet[n_z], znet[n_z - 1],
                                        state["zstep"], state["step_n"])
            state.update(z=state["z"] + zstep, zstep=zstep, step_n=step_n + 1)

        t0 = time.perf_counter()
        for _ in range(ke):
            host_call()
        te = time.perf_counter() - t0
        t1 = time.perf_counter()
        for _ in range(ke):
            P.set_field_ptr(f_h.data_ptr(), s_h.data_ptr())
            run_z_steps(P, S, state, 1)
            P.get_field_ptr(f_h.data_ptr(), s_h.data_ptr())
        t3 = time.perf_counter() - t1
        line["e2e"] = {"value": nr * nt * ke / te, "unit": UNIT, "h2d_bytes_per_step": 2 * nr * nt * 16,
                       "d2h_bytes_per_step": 2 * nr * nt * 16, "steps": ke,
                       "api": "gs_step_host (propagator() on host FIELD and BIGBUFFER2: both copied in and out "
                              "every call, pinned)",
                       "three_calls_value": nr * nt * ke / t3,
                       "three_calls_api": "gs_set_field + gs_advance (one call) + gs_get_field"}

    # FP64 path on the same workload + mixed-vs-FP64 field error after the same fixed-dz steps
    if prec == gs.PREC_MIXED and args.fp64_steps > 0:
        P64 = gs.Propagator(S, precision=gs.PREC_FP64, device=lrank)
        P64.set_field(S["field"])
        st64 = new_state(S)
        run_z_steps(P64, S, st64, 1)
        s64 = torch.cuda.ExternalStream(P64.stream_ptr(), device=lrank)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(s64)
        run_z_steps(P64, S, st64, args.fp64_steps)
        a1.record(s64)
        a1.synchronize()
        ms64 = a0.elapsed_time(a1)
        v64 = nr * nt * args.fp64_steps / (ms64 / 1e3)
        # accuracy: both paths from the start field, fixed dz = first ZSTEP, the mixed path's
        # relative L2 error of FIELD and BIGBUFFER2 against the FP64 path after each count of steps
        dz = float(S["init_zstep"])
        counts = sorted(int(c) for c in args.err_steps.split(",") if c)
        curve = []
        done = 0
        for Q in (P, P64):
            Q.set_field(S["field"])
        for c in counts:
            for Q in (P, P64):
                for _ in range(c - done):
                    Q.nl_step(dz)
                    Q.lstep(dz)
            done = c
            fm, sm = P.get_field(want_spec=True)
            fd, sd = P64.get_field(want_spec=True)
            curve.append({"steps": c, "field": float(np.linalg.norm(fm - fd) / np.linalg.norm(fd)),
                          "bigbuffer2": float(np.linalg.norm(sm - sd) / np.linalg.norm(sd))})
        line["fp64"] = {"value": v64, "unit": UNIT, "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps,
                        "mixed_speedup": value / world / v64,
                        "mixed_rel_l2_field_err": curve[-1]["field"] if curve else None,
                        "err_steps": done, "err_dz_m": dz, "error_curve": curve}
        P64.close()

    if prec == gs.PREC_MIXED and not args.no_adjoint and args.workload == "c2":
        line["adjoint"] = adjoint_leg(args, lrank)
    if prec == gs.PREC_MIXED and not args.no_batch and args.workload == "c2":
        line["batch"] = batch_leg(args, lrank)
    if prec == gs.PREC_MIXED and not args.no_argon and args.workload == "c2":
        line["argon"] = argon_leg(args, lrank)

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, desc, cores = cpu_sample(cpu_prepare(cfg))
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    P.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
