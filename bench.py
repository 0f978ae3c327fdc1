"""Benchmark of the dense Galerkin matrix fill on one GB300 (or N, one rank per GPU).

Workload (default, `--workload c2`): Maxwell3D single layer (EFIE, alpha = -ik, beta = 1/(-ik))
on RWG over an icosphere of level 5 (20,480 triangles, 30,720 RWG functions), k = 2 pi * 4,
default quadrature strategy (3 x 4-point far rule, Sauter-Schwab n = 4 for common
face/edge/vertex).  Synthetic, seeded mesh built by the package; no dataset is involved.

One step = one full assembly: upload of the space tables, pair classification, singular /
near-pair integrals, far-pair tiles with the gather write.  `value` is pair-interactions/s
(nt * nb / step time) of the MIXED kernel with the output in HBM; the plain FP64 kernel's rate
is reported beside it, and `e2e` is the same fill through the public API with the matrix
copied into a pinned host buffer (output blocks overlapped with the fill).  Errors of both
kernels against the FP64 CPU oracle are measured on 1000 seeded rows.

Other workloads print the same kind of line for their own configuration:
  --workload c3   MFIE on RWG and Helmholtz single layer on Lagrange over two jittered
                  96 x 96 coplanar plates 0.01 apart (36,864 triangles), k = 2 pi * 2; beside it the MFIE
                  on the same plates 0.003 apart with the second one turned up by 30 degrees (near pairs
                  across the fold with values)
  --workload c4   64 seeded ellipsoids (icosphere levels 1-4, axes U[0.5, 2], k U[1, 10]), EFIE,
                  one batched persistent launch replayed from a CUDA graph vs 64 sequential
                  plain FP64 assemblies
  --workload c5   EFIE on an icosphere of level 6 (81,920 triangles, 122,880 RWG), k = 2 pi * 8,
                  ComplexF32 output (121 GB) streamed to pinned host memory in output blocks
  --workload cube  the reference's own benchmark: Helmholtz3D single layer, k = 1, on lagrangec0d1 over
                  meshcuboid(1, 1, 1, 0.5/d) (--cube-d, default 40: 76,800 triangles, 38,402 functions;
                  data/graph_data.jl:2-4), mixed and plain FP64, into HBM and end to end into pinned host
                  memory, beside the reference's recorded full-assemble time for the same d
  --workload curve  Helmholtz2D hypersingular (the operator of the reference's 2-D prototype) on
                  hats over a jittered ellipse of 16,384 segments, k = 2 pi * 100, mixed and FP64

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c2|c3|c4|c5|cube|curve] [--impl reference]

`--impl reference` times the CPU restatement of the reference algorithm (the oracle, OpenMP
over all host cores) on a bounded row sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair-interactions/s: mixed FP32 vs plain FP64 on GB300 at rel err <=1e-5; CPU ref"
UNIT = "pair-interactions/s"
LEVEL, KWAVE = 5, 2 * np.pi * 4
ERR_ROWS, ERR_SEED = 1000, 0
# DRAM bytes (read + write) of one far-kernel launch per triangle pair, from the ncu capture of
# the level-4 case (0.462 GB for 5120^2 pairs); the traffic is the output written once, so it
# scales with the pairs.
FAR_DRAM_BYTES_PER_PAIR = 0.462e9 / (5120 * 5120)


def workload():
    import beastgpu_gb300 as bg
    mesh = bg.icosphere(LEVEL)
    X = bg.raviartthomas(mesh)
    op = bg.Maxwell3D.singlelayer(wavenumber=KWAVE)
    return bg, mesh, X, op, bg.QuadStrat()


def config_dict(mesh, X, extra=None):
    d = {"workload": f"EFIE Maxwell3D.singlelayer on RWG, icosphere level {LEVEL} ({mesh.nt} triangles, "
                     f"{X.nfun} RWG), k=2*pi*4, quadstrat far 3x4 / Sauter-Schwab n=4",
         "triangles": mesh.nt, "functions": X.nfun, "pairs_per_step": mesh.nt * mesh.nt,
         "output": "dense complex matrix, column-major",
         "l2": "output 7.5 GB > L2; a 256 MiB buffer is also written between timed steps"}
    if extra:
        d.update(extra)
    return d


def dist_init(ngpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            dist.init_process_group(backend=backend)
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, local):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = f"cuda:{local}" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index):
        import tempfile
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"bgb_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
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
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def flush_l2(buf):
    buf.add_(1)


def time_fill(bg, X, op, prec, steps, warmup, local, out="device", pinned=None, cfg=None, rows=None):
    """Per-step device time (CUDA events on the launching stream) of full assemblies, or of the row
    window rows = (row0, nrows)."""
    import torch
    cfg = cfg or bg.GPUConfiguration(precision=prec, device=local)
    scratch = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")
    dt = np.complex64 if prec == "mixed" else np.complex128
    nr = X.nfun if rows is None else int(rows[1])
    Zbuf = None
    if out == "device":
        tdt = torch.complex64 if prec == "mixed" else torch.complex128
        Zbuf = torch.empty((X.nfun, nr), dtype=tdt, device=f"cuda:{local}")
    stats = []

    def one():
        if out == "device":
            _, st = bg.assemble_gpu(op, X, X, cfg, out="device", out_buffer=Zbuf, rows=rows, return_stats=True)
        else:
            _, st = bg.assemble_gpu(op, X, X, cfg, out="host", out_buffer=pinned, dtype=dt, rows=rows,
                                    return_stats=True)
        return st

    for _ in range(warmup):
        one()
        flush_l2(scratch)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    wall0 = time.perf_counter()
    for i in range(steps):
        flush_l2(scratch)
        ev[i][0].record(stream)
        stats.append(one())
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    ms = [a.elapsed_time(b) for a, b in ev]
    return ms, stats, wall, Zbuf


def rows_error(Z_rows, ref):
    d = Z_rows - ref
    return {"rel_frobenius": float(np.linalg.norm(d) / np.linalg.norm(ref)),
            "max_entry_rel": float(np.abs(d).max() / np.abs(ref).max())}


CURVE_N, CURVE_K, CURVE_ROWS = 16384, 2 * np.pi * 100, 64
# FP64 flops (2 DFMA + DADD + DMUL thread instructions) per far point pair of the plain hypersingular
# far kernel, counted by ncu on the 4,096-segment case, and its DRAM bytes per segment pair (the 2x2
# complex double local matrix written once).
CURVE_FP64_FLOPS_PER_POINT_PAIR = 239.5
CURVE_DRAM_BYTES_PER_PAIR = 1.040e9 / (4096 * 4096)
# The same for the mixed far kernel: FP32 flops (2 FFMA + FADD + FMUL) per far point pair and DRAM
# bytes per segment pair (the local matrix as 2x2 complex float), ncu on the 4,096-segment case.
CURVE_MIXED_FP32_FLOPS_PER_POINT_PAIR = 97.2
CURVE_MIXED_DRAM_BYTES_PER_PAIR = 0.4755e9 / (4096 * 4096)


def curve_workload(n=CURVE_N):
    import beastgpu_gb300 as bg
    mesh = bg.ellipse(n, 1.0, 0.5, jitter=0.2, seed=11)
    return bg, mesh, bg.curve_lagrangec0d1(mesh), bg.Helmholtz2D.hypersingular(wavenumber=CURVE_K), bg.QuadStrat2D()


def curve_config(mesh, X, extra=None):
    d = {"workload": f"Helmholtz2D.hypersingular on lagrangec0d1 hats, jittered ellipse (1, 0.5) of {mesh.ns} "
                     f"segments, k=2*pi*100 (far 4x4 Gauss, near 12, singular order 10)",
         "segments": mesh.ns, "functions": X.nfun, "pairs_per_step": mesh.ns * mesh.ns,
         "l2": "outputs > L2; a 256 MiB buffer is written between timed steps"}
    d.update(extra or {})
    return d


def run_reference_curve(args):
    """CPU arm of the curve workload: the curve oracle on a row sample, all host cores."""
    import oracle
    bg, mesh, X, op, qs = curve_workload(args.curve_segments)
    rank, world, local = dist_init(args.gpus)
    if rank != 0:
        return 0
    threads = oracle.max_threads()
    rng = np.random.default_rng(1)
    pairs_per_row = 2 * mesh.ns
    vals = []
    for i in range(args.warmup + args.steps):
        rows = np.sort(rng.choice(X.nfun, CURVE_ROWS, replace=False)).astype(np.int32)
        t0 = time.perf_counter()
        oracle.assemble_rows_curve(op, X, X, qs, rows, nthreads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            vals.append(CURVE_ROWS * pairs_per_row / dt)
    v = float(np.mean(vals))
    sample = f"{CURVE_ROWS} random rows per step ({CURVE_ROWS * pairs_per_row} segment pairs)"
    print(json.dumps({"metric": "segment pair-interactions/s (2-D): mixed FP32 vs plain FP64", "value": v, "unit": UNIT,
                      "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": CURVE_ROWS * pairs_per_row / v * 1e3, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ellipse)",
                      "impl": "reference",
                      "config": curve_config(mesh, X, {"parallelism": f"OpenMP x{threads} host threads"}),
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def run_curve(args):
    """2-D path: Helmholtz2D hypersingular on an ellipse; mixed (value) and plain FP64, device output,
    and e2e of the mixed fill into pinned host memory."""
    import torch
    import oracle
    rank, world, local = dist_init(args.gpus)
    bg, mesh, X, op, qs = curve_workload(args.curve_segments)
    pairs = mesh.ns * mesh.ns
    # the caller's pinned output of the end-to-end leg, allocated once up front
    pinned = None if args.no_e2e else torch.empty((X.nfun, X.nfun), dtype=torch.complex64, pin_memory=True)
    fp32_peak, fp64_peak, _ = bg.measure_issue_peaks(local)
    barrier(world)
    with ClockSampler(local) as clocks:
        ms_m, st_m, _, Zm = time_fill(bg, X, op, "mixed", args.steps, args.warmup, local)
    barrier(world)
    m = max_over_ranks(float(np.mean(ms_m)), world, local)
    value = world * pairs / (m * 1e-3)
    ms_d, st_d, _, Zd = time_fill(bg, X, op, "fp64", args.fp64_steps, min(args.warmup, 3), local)
    md = max_over_ranks(float(np.mean(ms_d)), world, local)
    out = {}
    if rank == 0:
        rows = np.sort(np.random.default_rng(ERR_SEED).choice(X.nfun, CURVE_ROWS, replace=False)).astype(np.int32)
        threads = oracle.max_threads()
        t0 = time.perf_counter()
        ref = oracle.assemble_rows_curve(op, X, X, qs, rows, nthreads=threads)
        cpu_s = time.perf_counter() - t0
        ridx = torch.as_tensor(rows.astype(np.int64), device=Zm.device)
        out["error_vs_oracle"] = {"mixed": rows_error(Zm[:, ridx].T.cpu().numpy().astype(np.complex128), ref),
                                  "fp64": rows_error(Zd[:, ridx].T.cpu().numpy(), ref), "rows": CURVE_ROWS,
                                  "seed": ERR_SEED}
        cpu_pairs = CURVE_ROWS * 2 * mesh.ns
        out["cpu_baseline"] = {"value": cpu_pairs / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{CURVE_ROWS} seeded rows ({cpu_pairs} segment pairs, {cpu_s:.1f} s), "
                                         f"FP64 curve oracle with OpenMP"}
    del Zm, Zd
    torch.cuda.empty_cache()
    e2e = None
    if not args.no_e2e:
        ms_e2e, st_e2e, _, _ = time_fill(bg, X, op, "mixed", max(3, args.steps // 2), 1, local, out="host",
                                         pinned=pinned)
        e2e_ms = max_over_ranks(float(np.mean(ms_e2e)), world, local)
        h2d = X.mesh.vertices.nbytes + X.mesh.segments.nbytes + X.fn_index.nbytes + X.fn_coef.nbytes
        e2e = {"value": world * pairs / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(X.nfun) * int(X.nfun) * 8, "ms_per_step": e2e_ms,
               "ms_copy": float(np.mean([s["ms_copy"] for s in st_e2e]))}
        del pinned
    if rank != 0:
        return 0
    cls = st_m[0]["pairs_class"]
    point_pairs = cls[0] * qs.far_test * qs.far_trial

    def kernels(st):
        return {"far_and_gather": float(np.mean([s["ms_far"] for s in st])),
                "singular_and_near": float(np.mean([s["ms_singular"] for s in st])),
                "classify": float(np.mean([s["ms_classify"] for s in st]))}
    km, kd = kernels(st_m), kernels(st_d)
    tf = point_pairs * CURVE_MIXED_FP32_FLOPS_PER_POINT_PAIR / (km["far_and_gather"] * 1e-3) / 1e12
    roof = {"kernel": "curve::k_curve_far_mixed<HS> (+ gather)", "bound": "fp32", "achieved": tf, "peak": fp32_peak,
            "unit": "TFLOP/s", "frac": tf / fp32_peak, "traffic": CURVE_MIXED_DRAM_BYTES_PER_PAIR * pairs,
            "traffic_source": "ncu dram__bytes of the 4,096-segment launch scaled by pairs (x16)",
            "peak_source": "measured live by bgb_measure_issue_peaks (FFMA chains)",
            "flop_convention": f"{CURVE_MIXED_FP32_FLOPS_PER_POINT_PAIR} FP32 flops per far point pair (ncu count: "
                               "2 FFMA + FADD + FMUL, per-pair double-float setup included)",
            "note": "issue-bound: 89% of issue slots (FMA 46%, ALU 45%, MUFU 19% of peak), ncu on 4,096 segments"}
    tf64 = point_pairs * CURVE_FP64_FLOPS_PER_POINT_PAIR / (kd["far_and_gather"] * 1e-3) / 1e12
    roof64 = {"kernel": "curve::k_curve_far<HS> (+ gather)", "bound": "fp64", "achieved": tf64, "peak": fp64_peak,
              "unit": "TFLOP/s", "frac": tf64 / fp64_peak,
              "flop_convention": f"{CURVE_FP64_FLOPS_PER_POINT_PAIR} FP64 flops per far point pair (ncu count, "
                                 "CUDA's J0 and Y0 included)"}
    line = line_base(args, world, value, m, "f32 far pairs (FP32 Hankel approximations, double-float phase) + "
                     "double-float singular, FP64 near (mixed)", curve_config(mesh, X, {
                         "parallelism": f"{world} independent matrices, one per rank, no collective" if world > 1
                         else "single GPU"}),
                     metric="segment pair-interactions/s (2-D): mixed FP32 vs plain FP64",
                     fp64_value=world * pairs / (md * 1e-3), fp64_ms_per_step=md, mixed_over_fp64=md / m,
                     roofline=roof, fp64_roofline=roof64, kernels_ms={"mixed": km, "fp64": kd},
                     far_point_pairs_per_s=point_pairs / (km["far_and_gather"] * 1e-3), pairs_class=cls,
                     clocks=clocks.summary(),
                     gpu_launches=int(sum(s["kernel_launches"] for s in st_m)), e2e=e2e)
    line.update(out)
    print(json.dumps(line))
    return 0


def run_reference(args):
    """CPU arm: the oracle (restatement of the reference's algorithm) on host cores."""
    import oracle
    if args.workload == "curve":
        return run_reference_curve(args)
    if args.workload == "cube":
        bg, mesh, X, op, qs = cube_workload(args.cube_d)
        cfg = cube_config(mesh, X, args.cube_d)
    else:
        bg, mesh, X, op, qs = workload()
        cfg = config_dict(mesh, X)
    rank, world, local = dist_init(args.gpus)
    if rank != 0:
        return 0
    threads = oracle.max_threads()
    nrows = args.ref_rows
    rng = np.random.default_rng(1)
    sup = np.bincount(X.fn_index[X.fn_index >= 0], minlength=X.nfun)  # support triangles of each function
    vals, npairs = [], 0
    for i in range(args.warmup + args.steps):
        rows = np.sort(rng.choice(X.nfun, nrows, replace=False)).astype(np.int32)
        npairs = int(sup[rows].sum()) * mesh.nt  # triangle pairs the rows' local matrices cover
        t0 = time.perf_counter()
        oracle.assemble_rows(op, X, X, qs, rows, nthreads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            vals.append(npairs / dt)
    v = float(np.mean(vals))
    sample = f"{nrows} random rows per step ({npairs} triangle pairs, full local matrices)"
    cfg["parallelism"] = f"OpenMP x{threads} host threads"
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": npairs / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded meshes)",
            "impl": "reference",
            "config": cfg,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_profile_case(args):
    """Small cases for ncu captures, device output: EFIE on an icosphere of level --profile-level
    (mixed, then FP64); with --profile-cube D also the Helmholtz single layer on meshcuboid(1,1,1,0.5/D)
    (the Lagrange instances); with --profile-batch also one run of the 64-ellipsoid batch (mixed, no
    autotuning: its persistent far launch)."""
    import torch
    import beastgpu_gb300 as bg
    cases = []
    if args.profile_level > 0:
        mesh = bg.icosphere(args.profile_level)
        cases.append((f"icosphere level {args.profile_level}", bg.raviartthomas(mesh),
                      bg.Maxwell3D.singlelayer(wavenumber=KWAVE)))
    if args.profile_cube:
        mesh = bg.meshcuboid(1.0, 1.0, 1.0, 0.5 / args.profile_cube)
        cases.append((f"meshcuboid(1,1,1,0.5/{args.profile_cube})", bg.lagrangec0d1(mesh),
                      bg.Helmholtz3D.singlelayer(wavenumber=1.0)))
    for name, X, op in cases:
        for prec in ("mixed", "fp64"):
            ms, st, _, _ = time_fill(bg, X, op, prec, args.steps, args.warmup, 0)
            print(json.dumps({"profile_case": name, "precision": prec, "ms_per_step": float(np.mean(ms)),
                              "stats": st[-1]}))
    if args.profile_batch:
        probs = []
        for mesh, k in bg.ellipsoid_batch(64, seed=2):
            X = bg.raviartthomas(mesh)
            probs.append((bg.Maxwell3D.singlelayer(wavenumber=k), X, X))
        B = bg.Batch(probs, bg.GPUConfiguration(precision="mixed"), out="device", autotune=False)
        print(json.dumps({"profile_case": "64-ellipsoid batch", "precision": "mixed", "stats": B.create_stats}))
        B.close()
    torch.cuda.synchronize()
    return 0


def line_base(args, world, value, ms_step, dtype, config, **extra):
    d = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
         "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
         "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded meshes built in-process)",
         "config": config}
    d.update(extra)
    return d


def oracle_rows_error(op, X, Zrows, rows, qs=None):
    import oracle
    import beastgpu_gb300 as bg
    ref = oracle.assemble_rows(op, X, X, qs or bg.QuadStrat(), rows, nthreads=oracle.max_threads())
    return rows_error(np.asarray(Zrows, dtype=np.complex128), ref)


def run_c3(args, emit=True):
    """Near-singular stress: MFIE (RWG) and Helmholtz single layer (Lagrange) on two plates.  Returns
    the line (rank 0; None elsewhere) and prints it when `emit`."""
    import torch
    import beastgpu_gb300 as bg
    rank, world, local = dist_init(args.gpus)
    mesh = bg.two_plates(96, jitter=0.3, seed=1, gap=0.01)
    k = 2 * np.pi * 2
    R, L = bg.raviartthomas(mesh), bg.lagrangec0d1(mesh)
    # the Maxwell double layer vanishes on coplanar plates: two such plates 0.003 apart (0.3 h) with the
    # second one turned up by 30 degrees about its edge give it near pairs with values across the fold
    # (reported beside, not in `value`)
    fp = bg.two_plates(96, jitter=0.3, seed=1, gap=0.003)
    v = fp.vertices.copy()
    up = v[:, 0] > 1.0
    v[up, 2] = (v[up, 0] - 1.003) * np.sin(np.pi / 6)
    v[up, 0] = 1.003 + (v[up, 0] - 1.003) * np.cos(np.pi / 6)
    folded = bg.Mesh(v, fp.triangles)
    cases = [("mfie_rwg", bg.Maxwell3D.doublelayer(wavenumber=k), R),
             ("helmholtz_sl_lagrange", bg.Helmholtz3D.singlelayer(wavenumber=k), L),
             ("mfie_rwg_folded", bg.Maxwell3D.doublelayer(wavenumber=k), bg.raviartthomas(folded))]
    pairs = mesh.nt * mesh.nt
    res = {}
    tot_ms = {"mixed": 0.0, "fp64": 0.0}
    launches = 0
    with ClockSampler(local) as clocks:
        for name, op, X in cases:
            rows = np.sort(np.random.default_rng(3).choice(X.nfun, 200, replace=False)).astype(np.int32)
            r = {"functions": X.nfun}
            for prec in ("mixed", "fp64"):
                steps = args.steps if prec == "mixed" else args.fp64_steps
                ms, st, _, Z = time_fill(bg, X, op, prec, steps, args.warmup, local)
                m = max_over_ranks(float(np.mean(ms)), world, local)
                if name != "mfie_rwg_folded":
                    tot_ms[prec] += m
                launches += sum(x["kernel_launches"] for x in st) if prec == "mixed" else 0
                Zr = Z[:, torch.as_tensor(rows.astype(np.int64), device=Z.device)].T.cpu().numpy()
                r[prec] = {"ms_per_step": m, "pairs_per_s": pairs / (m * 1e-3), "stats": st[-1]}
                if rank == 0:
                    if name == "mfie_rwg":
                        r[prec]["max_abs_entry"] = float(np.abs(Zr).max())  # coplanar plates: exactly zero
                    else:
                        r[prec]["error_vs_oracle_200_rows"] = oracle_rows_error(op, X, Zr, rows)
                del Z
                torch.cuda.empty_cache()
            res[name] = r
    if rank != 0:
        return None
    value = world * 2 * pairs / (tot_ms["mixed"] * 1e-3)
    cfg = {"workload": "MFIE (RWG) + Helmholtz SL (Lagrange, interior vertices) on two jittered 96x96 plates, "
                       "gap 0.01, k=2*pi*2", "triangles": mesh.nt, "pairs_per_step": 2 * pairs,
           "l2": "outputs > L2; a 256 MiB buffer is written between timed steps"}
    line = line_base(args, world, value, tot_ms["mixed"], "f32 far pairs + double-float singular, FP64 near (mixed)",
                     cfg, fp64_value=world * 2 * pairs / (tot_ms["fp64"] * 1e-3), cases=res,
                     clocks=clocks.summary(), gpu_launches=launches)
    if emit:
        print(json.dumps(line))
    return line


def run_c4(args, emit=True):
    """64 uneven ellipsoids: one batched persistent launch (CUDA graph) vs 64 sequential assemblies.
    Returns the line (rank 0; None elsewhere) and prints it when `emit`."""
    import torch
    import beastgpu_gb300 as bg
    rank, world, local = dist_init(args.gpus)
    batch = bg.ellipsoid_batch(64, seed=2)
    probs = []
    for mesh, k in batch:
        X = bg.raviartthomas(mesh)
        probs.append((bg.Maxwell3D.singlelayer(wavenumber=k), X, X))
    pairs = sum(m.nt * m.nt for m, _ in batch)
    stream = torch.cuda.current_stream(local)
    out = {}
    with ClockSampler(local) as clocks:
        for prec in ("mixed", "fp64"):
            steps = args.steps if prec == "mixed" else args.fp64_steps
            B = bg.Batch(probs, bg.GPUConfiguration(precision=prec, device=local), out="device",
                         autotune=prec == "mixed" or not getattr(args, "c4_fp64_default_tiles", False))
            for _ in range(args.warmup):
                B.run()
            torch.cuda.synchronize()
            ms = [B.run()["ms_total"] for _ in range(steps)]
            graph_ms = max_over_ranks(float(np.mean(ms)), world, local)
            # 64 sequential single assemblies (one bgb_assemble each), device outputs
            bufs = [torch.empty((X.nfun, X.nfun), dtype=torch.complex64 if prec == "mixed" else torch.complex128,
                                device=f"cuda:{local}") for _, X, _ in probs]
            cfg = bg.GPUConfiguration(precision=prec, device=local)

            def seq():
                for (op, X, Y), b in zip(probs, bufs):
                    bg.assemble_gpu(op, X, Y, cfg, out="device", out_buffer=b)
            for _ in range(args.warmup):
                seq()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                seq()
            e1.record(stream)
            torch.cuda.synchronize()
            seq_ms = max_over_ranks(e0.elapsed_time(e1) / steps, world, local)
            same = all(bool(torch.equal(a.T, b)) for a, b in zip(bufs, B.outputs))
            errs = []
            if rank == 0:
                for i in (0, 21, 42, 63):
                    op, X, _ = probs[i]
                    rows = np.sort(np.random.default_rng(i).choice(X.nfun, min(20, X.nfun), replace=False)).astype(np.int32)
                    Zr = B.outputs[i][torch.as_tensor(rows.astype(np.int64), device=B.outputs[i].device)].cpu().numpy()
                    errs.append(oracle_rows_error(op, X, Zr, rows)["rel_frobenius"])
            out[prec] = {"graph_ms_per_step": graph_ms, "graph_pairs_per_s": pairs / (graph_ms * 1e-3),
                         "sequential_ms_per_step": seq_ms, "sequential_pairs_per_s": pairs / (seq_ms * 1e-3),
                         "batch_bit_identical_to_sequential": same, "tile_config": B.create_stats["tile_config"],
                         "schedule": B.create_stats["schedule"],
                         "max_rel_frobenius_vs_oracle_sampled": max(errs) if errs else None}
            B.close()
            del bufs
            torch.cuda.empty_cache()
    if rank != 0:
        return None
    value = world * pairs / (out["mixed"]["graph_ms_per_step"] * 1e-3)
    cfg = {"workload": "64 seeded ellipsoids (icosphere levels 1-4, axes U[0.5,2], k U[1,10]), EFIE on RWG, "
                       "one persistent CUDA-graph launch, autotuned tiles and schedule",
           "problems": 64, "triangles": sum(m.nt for m, _ in batch), "pairs_per_step": pairs}
    line = line_base(args, world, value, out["mixed"]["graph_ms_per_step"],
                     "f32 far pairs + double-float singular, FP64 near (mixed)", cfg,
                     vs_sequential_fp64=out["fp64"]["sequential_ms_per_step"] / out["mixed"]["graph_ms_per_step"],
                     results=out, clocks=clocks.summary(), gpu_launches=3 * (args.steps + args.warmup))
    if emit:
        print(json.dumps(line))
    return line


def run_c5(args):
    """Out of core: level-6 icosphere EFIE, ComplexF32 output streamed to pinned host memory."""
    import torch
    import beastgpu_gb300 as bg
    rank, world, local = dist_init(args.gpus)
    mesh = bg.icosphere(6)
    X = bg.raviartthomas(mesh)
    op = bg.Maxwell3D.singlelayer(wavenumber=2 * np.pi * 8)
    n = X.nfun
    nbytes = n * n * 8
    avail = 0
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                avail = int(line.split()[1]) * 1024
    except OSError:
        pass
    cfg_d = {"workload": f"EFIE on RWG, icosphere level 6 ({mesh.nt} triangles, {n} RWG), k=2*pi*8, ComplexF32 "
                         f"output ({nbytes / 1e9:.1f} GB) in pinned host memory",
             "triangles": mesh.nt, "functions": n, "pairs_per_step": mesh.nt * mesh.nt,
             "hbm_budget_bytes": args.hbm_budget}
    if avail and avail < nbytes + (24 << 30):
        print(json.dumps({"metric": METRIC, "skipped": f"host memory {avail / 1e9:.0f} GB < output + 24 GB",
                          "config": cfg_d}))
        return 0
    Z = np.empty((n, n), dtype=np.complex64, order="F")
    cfg = bg.GPUConfiguration(precision="mixed", device=local, total_GPU_budget=args.hbm_budget)
    # pageable destination first (the first call faults its pages in), then the same memory pinned
    ms_pg, st_pg, _, _ = time_fill(bg, X, op, "mixed", args.steps, 1, local, out="host", pinned=Z, cfg=cfg)
    cudart = torch.cuda.cudart()
    t0 = time.perf_counter()
    rc = cudart.cudaHostRegister(Z.ctypes.data, Z.nbytes, 0)
    reg_s = time.perf_counter() - t0
    if int(rc) != 0:
        raise RuntimeError(f"cudaHostRegister failed ({rc})")
    try:
        with ClockSampler(local) as clocks:
            ms_steps, stats, _, _ = time_fill(bg, X, op, "mixed", args.steps, args.warmup, local, out="host",
                                              pinned=Z, cfg=cfg)
        rows = np.sort(np.random.default_rng(5).choice(n, 100, replace=False)).astype(np.int32)
        err = oracle_rows_error(op, X, Z[rows, :], rows) if rank == 0 else None
    finally:
        cudart.cudaHostUnregister(Z.ctypes.data)
    ms = max_over_ranks(float(np.mean(ms_steps)), world, local)
    if rank != 0:
        return 0
    st = stats[-1]
    far, cp, pipe = st["ms_far"], st["ms_copy"], st["ms_pipeline"]
    pairs = mesh.nt * mesh.nt
    value = world * pairs / (ms * 1e-3)
    h2d = X.mesh.vertices.nbytes + X.mesh.triangles.nbytes + X.fn_index.nbytes + X.fn_coef.nbytes
    print(json.dumps(line_base(
        args, world, value, ms, "f32 far pairs + double-float (f32 pairs) singular/near (mixed)", cfg_d,
        e2e={"value": value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(nbytes)},
        pipeline={"out_blocks": st["out_blocks"], "ms_classify": st["ms_classify"], "ms_singular": st["ms_singular"],
                  "ms_far": far, "ms_copy": cp, "ms_pipeline": pipe, "ms_plan": st["ms_plan"],
                  "overlap_fraction": (far + cp - pipe) / min(far, cp) if min(far, cp) > 0 else None,
                  "copy_gbs": nbytes / (cp * 1e-3) / 1e9 if cp > 0 else None, "host_register_s": reg_s},
        pageable_destination={"ms_per_step": float(np.mean(ms_pg)), "pairs_per_s": pairs / (np.mean(ms_pg) * 1e-3),
                              "ms_copy": st_pg[-1]["ms_copy"], "ms_pipeline": st_pg[-1]["ms_pipeline"]},
        error_vs_oracle=dict(err, rows=100, seed=5), clocks=clocks.summary(),
        gpu_launches=int(sum(x["kernel_launches"] for x in stats)))))
    return 0


# The reference's recorded full GPU assemble of this workload (GPU write-back, FP64, ComplexF64 host
# matrix), median of its logs data/GPU_full/storeGPU/<d>/full_time.txt; its GPU is not named.
CUBE_REFERENCE_S = {24: 1.208, 40: 9.610}


def cube_workload(d):
    import beastgpu_gb300 as bg
    mesh = bg.meshcuboid(1.0, 1.0, 1.0, 0.5 / d)
    return bg, mesh, bg.lagrangec0d1(mesh), bg.Helmholtz3D.singlelayer(wavenumber=1.0), bg.QuadStrat()


def cube_config(mesh, X, d, extra=None):
    c = {"workload": f"Helmholtz3D.singlelayer k=1 on lagrangec0d1, meshcuboid(1,1,1,0.5/{d}) ({mesh.nt} triangles, "
                     f"{X.nfun} functions), quadstrat far 3x4 / Sauter-Schwab n=4 (the reference's benchmark)",
         "triangles": mesh.nt, "functions": X.nfun, "pairs_per_step": mesh.nt * mesh.nt,
         "l2": "outputs > L2; a 256 MiB buffer is written between timed steps"}
    c.update(extra or {})
    return c


def run_cube(args, emit=True):
    """The reference's benchmark workload (data/graph_data.jl:2-4): mixed (value) and plain FP64 into HBM,
    both end to end into pinned host memory (FP64 into ComplexF64 like the reference's storeGPU path).
    Returns the line (rank 0; None elsewhere) and prints it when `emit`."""
    import torch
    import oracle
    rank, world, local = dist_init(args.gpus)
    d = args.cube_d
    bg, mesh, X, op, qs = cube_workload(d)
    pairs = mesh.nt * mesh.nt
    n = X.nfun
    barrier(world)
    with ClockSampler(local) as clocks:
        ms_m, st_m, _, Zm = time_fill(bg, X, op, "mixed", args.steps, args.warmup, local)
    barrier(world)
    m = max_over_ranks(float(np.mean(ms_m)), world, local)
    value = world * pairs / (m * 1e-3)
    ms_d, st_d, _, Zd = time_fill(bg, X, op, "fp64", args.fp64_steps, 1, local)
    md = max_over_ranks(float(np.mean(ms_d)), world, local)
    out = {}
    if rank == 0:
        rows = np.sort(np.random.default_rng(ERR_SEED).choice(n, min(n, 200), replace=False)).astype(np.int32)
        threads = oracle.max_threads()
        t0 = time.perf_counter()
        ref = oracle.assemble_rows(op, X, X, qs, rows, nthreads=threads)
        cpu_s = time.perf_counter() - t0
        ridx = torch.as_tensor(rows.astype(np.int64), device=Zm.device)
        out["error_vs_oracle"] = {"mixed": rows_error(Zm[:, ridx].T.cpu().numpy().astype(np.complex128), ref),
                                  "fp64": rows_error(Zd[:, ridx].T.cpu().numpy(), ref), "rows": int(rows.size),
                                  "fp64_max_abs": float(np.abs(Zd[:, ridx].T.cpu().numpy() - ref).max()),
                                  "seed": ERR_SEED}
        sup = np.bincount(X.fn_index[X.fn_index >= 0], minlength=n)
        cpu_pairs = int(sup[rows].sum()) * mesh.nt
        out["cpu_baseline"] = {"value": cpu_pairs / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{rows.size} seeded rows ({cpu_pairs} triangle pairs, {cpu_s:.1f} s), FP64 "
                                         f"oracle with OpenMP"}
    del Zm, Zd
    torch.cuda.empty_cache()
    e2e, e2e64 = None, None
    h2d = X.mesh.vertices.nbytes + X.mesh.triangles.nbytes + X.fn_index.nbytes + X.fn_coef.nbytes
    if not args.no_e2e:
        pinned = torch.empty((n, n), dtype=torch.complex64, pin_memory=True)
        ms_e, st_e, _, _ = time_fill(bg, X, op, "mixed", max(2, args.steps // 2), 1, local, out="host", pinned=pinned)
        em = max_over_ranks(float(np.mean(ms_e)), world, local)
        e2e = {"value": world * pairs / (em * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": n * n * 8, "ms_per_step": em,
               "ms_copy": float(np.mean([s["ms_copy"] for s in st_e]))}
        del pinned
        if not getattr(args, "cube_no_fp64_e2e", False):
            pinned = torch.empty((n, n), dtype=torch.complex128, pin_memory=True)
            ms_e64, st_e64, _, _ = time_fill(bg, X, op, "fp64", 1, 0, local, out="host", pinned=pinned)
            e64 = max_over_ranks(float(np.mean(ms_e64)), world, local)
            e2e64 = {"value": world * pairs / (e64 * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                     "d2h_bytes_per_step": n * n * 16, "ms_per_step": e64,
                     "ms_copy": float(np.mean([s["ms_copy"] for s in st_e64]))}
            del pinned
    if rank != 0:
        return None

    def kernels(st):
        return {k: float(np.mean([s["ms_" + k] for s in st])) for k in ("far", "singular", "classify")}
    ref_s = CUBE_REFERENCE_S.get(d)
    line = line_base(args, world, value, m, "f32 far pairs + double-float (f32 pairs) singular (mixed)",
                     cube_config(mesh, X, d, {"parallelism": "single GPU" if world == 1 else
                                              f"{world} independent matrices, one per rank, no collective"}),
                     fp64_value=world * pairs / (md * 1e-3), fp64_ms_per_step=md, mixed_over_fp64=md / m,
                     kernels_ms={"mixed": kernels(st_m), "fp64": kernels(st_d)}, pairs_class=st_m[0]["pairs_class"],
                     halo_redundancy=st_m[0]["pairs_computed"] / pairs, clocks=clocks.summary(),
                     gpu_launches=int(sum(s["kernel_launches"] for s in st_m)), e2e=e2e, e2e_fp64=e2e64,
                     reference_recorded=None if ref_s is None else {
                         "full_assemble_s": ref_s, "pairs_per_s": pairs / ref_s,
                         "source": f"data/GPU_full/storeGPU/{d}/full_time.txt (median), FP64, GPU write-back, "
                                   "ComplexF64 host matrix; GPU model not recorded"})
    line.update(out)
    if emit:
        print(json.dumps(line))
    return line


def extra_workloads(args):
    """Short runs of the other workloads for the default line (one GPU): the two-plate near-singular
    stress, the 64-ellipsoid batch and the reference's cube benchmark at d = 40, each with its own
    error against the oracle.  Each is also a workload of its own (--workload c3 | c4 | cube)."""
    import copy
    import torch
    sub = copy.copy(args)
    sub.steps, sub.warmup, sub.fp64_steps = 3, 1, 1
    sub.cube_d, sub.no_e2e, sub.cube_no_fp64_e2e, sub.c4_fp64_default_tiles = 40, False, True, True
    out = {}
    for name, fn in (("c3", run_c3), ("c4", run_c4), ("cube_d40", run_cube)):
        t0 = time.perf_counter()
        line = fn(sub, emit=False)
        torch.cuda.empty_cache()
        if line is None:
            continue
        keep = ("value", "unit", "ms_per_step", "fp64_value", "fp64_ms_per_step", "mixed_over_fp64", "config",
                "error_vs_oracle", "cases", "results", "vs_sequential_fp64", "e2e", "reference_recorded",
                "kernels_ms", "halo_redundancy", "cpu_baseline", "clocks")
        out[name] = {k: line[k] for k in keep if k in line}
        out[name]["wall_s"] = time.perf_counter() - t0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--ref-rows", type=int, default=200)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="default workload: leave out the c3 / c4 / cube sub-results")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5", "cube", "curve"])
    ap.add_argument("--cube-d", type=int, default=40, help="cube: density d of meshcuboid(1, 1, 1, 0.5/d)")
    ap.add_argument("--hbm-budget", type=int, default=0, help="c5: HBM budget in bytes (0 = 90%% of free)")
    ap.add_argument("--curve-segments", type=int, default=CURVE_N, help="curve: segments of the ellipse")
    ap.add_argument("--profile-level", type=int, default=None,
                    help="profiling case: run W + K mixed and FP64 fills of an icosphere of this level and exit "
                         "(0: none, with --profile-cube / --profile-batch)")
    ap.add_argument("--profile-cube", type=int, default=0, help="profiling case: also the cube at this density d")
    ap.add_argument("--profile-batch", action="store_true", help="profiling case: also one 64-ellipsoid batch")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_level is not None:
        return run_profile_case(args)
    if args.workload != "c2":
        rc = {"c3": run_c3, "c4": run_c4, "c5": run_c5, "cube": run_cube, "curve": run_curve}[args.workload](args)
        return rc if isinstance(rc, int) else 0

    import torch
    rank, world, local = dist_init(args.gpus)
    bg, mesh, X, op, qs = workload()
    pairs = mesh.nt * mesh.nt
    # N ranks: one matrix, cut into N balanced row windows (each rank assembles its rows against all
    # trial functions; no data exchange); value = the whole matrix's pairs / the slowest rank's time
    win = None if world == 1 else bg.row_shard(X.nfun, rank, world)
    r0, nr = (0, X.nfun) if win is None else win
    # the caller's pinned output of the end-to-end leg, allocated once up front (as an application
    # holds its output buffer), before the CPU oracle's allocations
    pinned = None if args.no_e2e else torch.empty((X.nfun, nr), dtype=torch.complex64, pin_memory=True)

    # roofline denominators measured live (FP32 / FP64 FMA issue, MUFU)
    fp32_peak, fp64_peak, mufu_peak = bg.measure_issue_peaks(local)

    barrier(world)
    with ClockSampler(local) as clocks:
        ms_mixed, st_mixed, wall_mixed, Zm = time_fill(bg, X, op, "mixed", args.steps, args.warmup, local, rows=win)
    barrier(world)
    ms_step = max_over_ranks(float(np.mean(ms_mixed)), world, local)
    value = pairs / (ms_step * 1e-3)

    ms_fp64, st_fp64, _, Zd = time_fill(bg, X, op, "fp64", args.fp64_steps, min(args.warmup, 3), local, rows=win)
    fp64_ms = max_over_ranks(float(np.mean(ms_fp64)), world, local)
    fp64_value = pairs / (fp64_ms * 1e-3)

    out = {}
    if rank == 0:
        # accuracy on 1000 seeded rows (of rank 0's window) against the FP64 CPU oracle (also the CPU
        # baseline sample)
        import oracle
        rows = (r0 + np.sort(np.random.default_rng(ERR_SEED).choice(nr, min(nr, ERR_ROWS), replace=False))).astype(np.int32)
        threads = oracle.max_threads()
        t0 = time.perf_counter()
        ref = oracle.assemble_rows(op, X, X, qs, rows, nthreads=threads)
        cpu_s = time.perf_counter() - t0
        ridx = torch.as_tensor((rows - r0).astype(np.int64), device=Zm.device)
        # Zbuf is (cols, rows) storage of the column-major matrix: row r of Z is column r of Zbuf
        err_mixed = rows_error(Zm[:, ridx].T.cpu().numpy().astype(np.complex128), ref)
        err_fp64 = rows_error(Zd[:, ridx].T.cpu().numpy(), ref)
        cpu_pairs = ERR_ROWS * 2 * mesh.nt
        out["cpu_baseline"] = {"value": cpu_pairs / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{ERR_ROWS} seeded rows of the same matrix ({cpu_pairs} triangle pairs, "
                                         f"{cpu_s:.1f} s), FP64 oracle with OpenMP"}
        out["error_vs_oracle"] = {"mixed": err_mixed, "fp64": err_fp64, "rows": ERR_ROWS, "seed": ERR_SEED}
    del Zd

    e2e = None
    if not args.no_e2e:
        del Zm
        torch.cuda.empty_cache()
        ms_e2e, st_e2e, wall_e2e, _ = time_fill(bg, X, op, "mixed", max(3, args.steps // 2), 1, local, out="host",
                                                pinned=pinned, rows=win)
        e2e_ms = max_over_ranks(float(np.mean(ms_e2e)), world, local)
        h2d = X.mesh.vertices.nbytes + X.mesh.triangles.nbytes + X.fn_index.nbytes + X.fn_coef.nbytes
        e2e = {"value": pairs / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(X.nfun) * int(nr) * 8, "ms_per_step": e2e_ms,
               "ms_copy": float(np.mean([s["ms_copy"] for s in st_e2e]))}
        del pinned

    if rank != 0:
        return 0
    # roofline of the dominant kernel (far tiles or singular pairs) from the library's events
    far_ms = float(np.mean([s["ms_far"] for s in st_mixed]))
    sing_ms = float(np.mean([s["ms_singular"] for s in st_mixed]))
    cls = st_mixed[0]["pairs_class"]
    far_pairs = cls[0]
    flops_far = far_pairs * 3 * 4 * (15 + 108)              # per point pair: kernel 15 + EFIE accumulation 108
    n = qs.ss_cf
    sing_evals = n ** 4 * (6 * cls[3] + 5 * cls[2] + 2 * cls[1])
    flops_sing = sing_evals * (15 + 108)
    far_tf = flops_far / (far_ms * 1e-3) / 1e12
    sing_tf = flops_sing / (sing_ms * 1e-3) / 1e12
    if far_ms >= sing_ms:
        roof = {"kernel": "k_far_tiles<PMixed, EFIE, 3, 4>", "bound": "fp32", "achieved": far_tf, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": far_tf / fp32_peak}
    else:
        roof = {"kernel": "k_singular (FP64 Sauter-Schwab)", "bound": "fp64", "achieved": sing_tf, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": sing_tf / fp64_peak}
    hbm_peak = None
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
    except (OSError, ValueError):
        pass
    out_gb = X.nfun * X.nfun * 8 / 1e9
    roof.update({"traffic": FAR_DRAM_BYTES_PER_PAIR * pairs if far_ms >= sing_ms else None,
                 "traffic_source": "ncu dram__bytes of the level-4 launch scaled by pairs (x16)",
                 "hbm_gbs_far": out_gb / (far_ms * 1e-3), "hbm_frac_far_of_measured": (out_gb / (far_ms * 1e-3)) / hbm_peak
                 if hbm_peak else None,
                 "peak_source": "measured live by bgb_measure_issue_peaks (FMA chains)",
                 "flop_convention": "per point pair: 15 (kernel) + 108 (EFIE 9-entry accumulation), FMA = 2",
                 "kernels_ms": {"far": far_ms, "singular": sing_ms,
                                "classify": float(np.mean([s["ms_classify"] for s in st_mixed]))},
                 "far_tflops": far_tf, "singular_tflops": sing_tf,
                 "fp64_peak_tflops": fp64_peak, "mufu_peak_tops": mufu_peak,
                 "halo_redundancy": st_mixed[0]["pairs_computed"] / st_mixed[0]["pairs_total"]})
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak",
            "vs_baseline": None, "dtype": "f32 far pairs + double-float (f32 pairs) singular/near (mixed)",
            "data": "synthetic (seeded icosphere, built in-process)",
            "config": config_dict(mesh, X, {"parallelism": f"one matrix in {world} row windows, one per rank, no "
                                            "collective on the data path" if world > 1 else "single GPU"}),
            "fp64_value": fp64_value, "fp64_ms_per_step": fp64_ms, "mixed_over_fp64": value / fp64_value,
            "roofline": roof, "clocks": clocks.summary(),
            "gpu_launches": int(sum(s["kernel_launches"] for s in st_mixed)),
            "e2e": e2e}
    line.update(out)
    if world == 1 and not args.no_extra:
        line["workloads"] = extra_workloads(args)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
