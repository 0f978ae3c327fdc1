"""Benchmark of the dense Galerkin matrix fill on one GB300 (or N, one rank per GPU).

Workload (default): Maxwell3D single layer (EFIE, alpha = -ik, beta = 1/(-ik)) on RWG over an
icosphere of level 5 (20,480 triangles, 30,720 RWG functions), k = 2 pi * 4, default quadrature
strategy (3 x 4-point far rule, Sauter-Schwab n = 4 for common face/edge/vertex).  Synthetic,
seeded mesh built by the package; no dataset is involved.

One step = one full assembly: upload of the space tables, pair classification, FP64
singular / near-pair integrals, far-pair tiles with the gather write.  `value` is
pair-interactions/s (nt * nb / step time) of the MIXED kernel with the output in HBM; the plain
FP64 kernel's rate is reported beside it, and `e2e` is the same fill through the C ABI with
the matrix copied into a pinned host buffer.  Errors of both kernels against the FP64 CPU
oracle are measured on 1000 seeded rows.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

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
        self.index = index
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

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


def time_fill(bg, X, op, prec, steps, warmup, local, out="device", pinned=None):
    """Per-step device time (CUDA events on the launching stream) of full assemblies."""
    import torch
    cfg = bg.GPUConfiguration(precision=prec, device=local)
    scratch = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")
    dt = np.complex64 if prec == "mixed" else np.complex128
    Zbuf = None
    if out == "device":
        tdt = torch.complex64 if prec == "mixed" else torch.complex128
        Zbuf = torch.empty((X.nfun, X.nfun), dtype=tdt, device=f"cuda:{local}")
    stats = []

    def one():
        if out == "device":
            _, st = bg.assemble_gpu(op, X, X, cfg, out="device", out_buffer=Zbuf, return_stats=True)
        else:
            _, st = bg.assemble_gpu(op, X, X, cfg, out="host", out_buffer=pinned, dtype=dt, return_stats=True)
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


def run_reference(args):
    """CPU arm: the oracle (restatement of the reference's algorithm) on host cores."""
    import oracle
    bg, mesh, X, op, qs = workload()
    rank, world, local = dist_init(args.gpus)
    if rank != 0:
        return 0
    threads = oracle.max_threads()
    nrows = args.ref_rows
    rng = np.random.default_rng(1)
    pairs_per_row = 2 * mesh.nt
    vals = []
    for i in range(args.warmup + args.steps):
        rows = np.sort(rng.choice(X.nfun, nrows, replace=False)).astype(np.int32)
        t0 = time.perf_counter()
        oracle.assemble_rows(op, X, X, qs, rows, nthreads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            vals.append(nrows * pairs_per_row / dt)
    v = float(np.mean(vals))
    sample = f"{nrows} random rows per step ({nrows * pairs_per_row} triangle pairs, full local matrices)"
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": nrows * pairs_per_row / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded icosphere)",
            "impl": "reference",
            "config": config_dict(mesh, X, {"parallelism": f"OpenMP x{threads} host threads"}),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_profile_case(args):
    """Small case for ncu captures: EFIE on an icosphere of the given level, device output."""
    import torch
    import beastgpu_gb300 as bg
    mesh = bg.icosphere(args.profile_level)
    X = bg.raviartthomas(mesh)
    op = bg.Maxwell3D.singlelayer(wavenumber=KWAVE)
    for prec in ("mixed", "fp64"):
        ms, st, _, _ = time_fill(bg, X, op, prec, args.steps, args.warmup, 0)
        print(json.dumps({"profile_case": f"icosphere level {args.profile_level}", "precision": prec,
                          "ms_per_step": float(np.mean(ms)), "stats": st[-1]}))
    torch.cuda.synchronize()
    return 0


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
    ap.add_argument("--profile-level", type=int, default=None,
                    help="profiling case: run W + K mixed and FP64 fills of an icosphere of this level and exit")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_level is not None:
        return run_profile_case(args)

    import torch
    rank, world, local = dist_init(args.gpus)
    bg, mesh, X, op, qs = workload()
    pairs = mesh.nt * mesh.nt

    # roofline denominators measured live (FP32 / FP64 FMA issue, MUFU)
    fp32_peak, fp64_peak, mufu_peak = bg.measure_issue_peaks(local)

    barrier(world)
    with ClockSampler(local) as clocks:
        ms_mixed, st_mixed, wall_mixed, Zm = time_fill(bg, X, op, "mixed", args.steps, args.warmup, local)
    barrier(world)
    ms_step = max_over_ranks(float(np.mean(ms_mixed)), world, local)
    value = world * pairs / (ms_step * 1e-3)

    ms_fp64, st_fp64, _, Zd = time_fill(bg, X, op, "fp64", args.fp64_steps, min(args.warmup, 3), local)
    fp64_ms = max_over_ranks(float(np.mean(ms_fp64)), world, local)
    fp64_value = world * pairs / (fp64_ms * 1e-3)

    out = {}
    if rank == 0:
        # accuracy on 1000 seeded rows against the FP64 CPU oracle (also the CPU baseline sample)
        import oracle
        rows = np.sort(np.random.default_rng(ERR_SEED).choice(X.nfun, ERR_ROWS, replace=False)).astype(np.int32)
        threads = oracle.max_threads()
        t0 = time.perf_counter()
        ref = oracle.assemble_rows(op, X, X, qs, rows, nthreads=threads)
        cpu_s = time.perf_counter() - t0
        ridx = torch.as_tensor(rows.astype(np.int64), device=Zm.device)
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
        pinned = torch.empty((X.nfun, X.nfun), dtype=torch.complex64, pin_memory=True)
        ms_e2e, st_e2e, wall_e2e, _ = time_fill(bg, X, op, "mixed", max(3, args.steps // 2), 1, local, out="host",
                                                pinned=pinned)
        e2e_ms = max_over_ranks(float(np.mean(ms_e2e)), world, local)
        h2d = X.mesh.vertices.nbytes + X.mesh.triangles.nbytes + X.fn_index.nbytes + X.fn_coef.nbytes
        e2e = {"value": world * pairs / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(X.nfun) * int(X.nfun) * 8, "ms_per_step": e2e_ms,
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
    roof.update({"traffic": None, "peak_source": "measured live by bgb_measure_issue_peaks (FMA chains)",
                 "flop_convention": "per point pair: 15 (kernel) + 108 (EFIE 9-entry accumulation), FMA = 2",
                 "kernels_ms": {"far": far_ms, "singular": sing_ms,
                                "classify": float(np.mean([s["ms_classify"] for s in st_mixed]))},
                 "far_tflops": far_tf, "singular_tflops": sing_tf,
                 "fp64_peak_tflops": fp64_peak, "mufu_peak_tops": mufu_peak,
                 "halo_redundancy": st_mixed[0]["pairs_computed"] / pairs})
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 far pairs + f64 singular/near (mixed)",
            "data": "synthetic (seeded icosphere, built in-process)",
            "config": config_dict(mesh, X, {"parallelism": f"replicas x{world}" if world > 1 else "single GPU"}),
            "fp64_value": fp64_value, "fp64_ms_per_step": fp64_ms, "mixed_over_fp64": value / fp64_value,
            "roofline": roof, "clocks": clocks.summary(),
            "gpu_launches": int(sum(s["kernel_launches"] for s in st_mixed)),
            "e2e": e2e}
    line.update(out)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
