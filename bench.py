"""Benchmark: triangle-soup fast winding number (igl::fast_winding_number soup
overloads), the configuration the headline metric is quoted on:

  mesh    icosphere subdivided 8 times (1,310,720 triangles), radial
          spherical-harmonic displacement (degree <= 8, N(0, 0.05/l)), 1% of
          the triangles deleted at random (1,297,489 left);
  queries 10M: 90% uniform in the 1.2x bounding box, 10% along random face
          normals at 10^U(-4,-1); float64 (float32 with --qdtype f32);
  order 2, accuracy_scale (beta) 2.

A step is one evaluation of all queries on the device (mixed precision:
FP32 bulk, FP64 near-field terms and threshold re-evaluation) over the
reference's own 4-wide tree (--tree reference, the default) or the binned
binary tree.  Reported: value = queries/s of the device-resident call; e2e =
the same call through the C ABI with host (pinned) buffers, copies
included; accuracy of the mixed result against the plain FP64 walk of the
same tree and (vs_reference) against the reference's own FP32 values on the
first 200k queries; the plain FP64 walk's own throughput; the dominant
kernel's live CUDA-event duration and roofline; a CPU baseline on this
host's cores.  Unless --no-extras, the line also carries the other
configurations as sub-results, each with its own CPU baseline: exact_c1,
cloud_c3, precision_c4, served_c5 (2 s Poisson trace, 120 GB budget) and
served_c5_pressure (a budget below the resident set).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gwn|reference]

Under torchrun (N > 1) every rank evaluates its own 10M-query batch against a
replica of the tree (queries shard with no data-path collective; weak
scaling); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "soup_fwn_icosphere8_sh_1pct_holes_10Mq"
METRIC = "winding queries/s at |dW|<=1e-4 vs FP64 (mixed vs plain FP64 GPU)"
UNIT = "queries/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gwn", "reference"], default="gwn")
    ap.add_argument("--nq", type=int, default=10_000_000)
    ap.add_argument("--qdtype", choices=["f64", "f32"], default="f64")
    ap.add_argument("--subdiv", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU work for the CPU baseline sample")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--workload", choices=["soup", "exact", "cloud", "precision", "served",
                                           "signed_distance", "knn", "eytzinger2d", "swept",
                                           "point_areas"],
                    default="soup",
                    help="soup = the headline line; the others are extra measurement lines")
    ap.add_argument("--served-seconds", type=float, default=4.0,
                    help="served: length of the Poisson arrival trace")
    ap.add_argument("--tree", choices=["reference", "binned"], default="reference",
                    help="soup tree: the reference's own 4-wide tree (default) or the "
                         "binned binary tree")
    ap.add_argument("--no-extras", action="store_true",
                    help="default line only: skip the C1/C3/C4/C5 sub-results")
    ap.add_argument("--extras-served-seconds", type=float, default=2.0,
                    help="trace length of the C5 sub-results of the default line")
    ap.add_argument("--pressure-budget-gb", type=float, default=40.0,
                    help="HBM budget of the C5 run under memory pressure")
    ap.add_argument("--served-meshes", type=int, default=256)
    ap.add_argument("--fp64-sample", type=int, default=5000,
                    help="precision study: FP64 reference queries per (decade, side)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic(name: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/<name>.md, line 'dram_bytes_per_launch: N'), else None."""
    path = os.path.join(ROOT, "profiles", name + ".md")
    try:
        for line in open(path):
            if line.strip().startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except OSError:
        pass
    return None


# FP32 operations of the mixed walk (a fused multiply-add counts 2): the
# reference's open test |q - P|^2 <= maxP2 beta^2 (3 sub, 4 mul, 2 add), the
# packed order-2 far field (soup.cuh pack_far32: rsqrt, 27 mul/add, 13 fma,
# the sum), one FP32 exact triangle term (corner vectors, normalisation,
# triple product, denominator, atan2f).
FLOPS_OPEN_TEST = 9
FLOPS_FAR_FIELD = 54
FLOPS_EXACT_TRI = 100


def walk_compute(bvh, dQ, nq, walk_ms, clocks, peaks):
    """Compute side of the walk's roofline: FP32 FLOPs per query from the
    instrumented walk's counters over the same queries, achieved FLOP/s in
    the timed launches, against the nominal FP32 rate at the sampled clock
    (152 SMs x 128 lanes x 2 x MHz; no measured FP32 peak exists)."""
    c = bvh.walk_stats(dQ, 2.0)
    per_q = {k: c[k] / nq for k in ("node_visits", "far_field", "exact_fp32", "exact_fp64_near")}
    flops_q = (per_q["node_visits"] * FLOPS_OPEN_TEST + per_q["far_field"] * FLOPS_FAR_FIELD
               + per_q["exact_fp32"] * FLOPS_EXACT_TRI)
    mhz = (clocks or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
    achieved = flops_q * nq / (walk_ms / 1e3) / 1e12
    warps = (nq + 31) // 32
    return {"unit": "TFLOP/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "peak_source": f"nominal FP32 at the sampled {mhz:.0f} MHz",
            "flops_per_query": flops_q, "per_query": per_q,
            "warp_steps_per_warp": c["warp_steps"] / warps,
            "lane_utilisation": c["node_visits"] / max(1, c["warp_steps"] * 32)}


def make_workload(args, rank):
    from libigl_gb300 import synth
    V, F = synth.soup_mesh(seed=1, subdiv=args.subdiv)
    Q = synth.soup_queries(V, F, seed=2 + rank, nq=args.nq)
    if args.qdtype == "f32":
        Q = Q.astype(np.float32)
    return V, F, Q


def soup_config(args, triangles, world):
    """The headline line's config, identical in both arms."""
    return {"workload": WORKLOAD, "triangles": int(triangles), "queries_per_gpu": int(args.nq),
            "qdtype": args.qdtype, "order": 2, "beta": 2.0, "tree": args.tree,
            "l2": "inputs larger than L2 (queries+results > 126 MB per step)",
            "parallelism": f"query shards x{world}, tree replicated"}


def cpu_baseline(V, F, Q, seconds: float, probe_n: int = 200_000):
    """CPU soup FWN (oracle restatement of the reference algorithm, equal to
    the reference's own outputs bit for bit) on this host's cores, on a
    bounded sample of the same queries.  Also returns its values on the
    first probe_n queries (the reference's W there)."""
    from oracle import oracle as O
    nthreads = O.num_threads(0)
    t0 = time.perf_counter()
    port = O.SoupPort(V, F, order=2)
    build_s = time.perf_counter() - t0
    probe = Q[: min(len(Q), probe_n)]
    t0 = time.perf_counter()
    Wprobe = port.eval(probe, 2.0, nthreads)
    dt = time.perf_counter() - t0
    rate = len(probe) / max(dt, 1e-9)
    n = int(min(len(Q), max(len(probe), rate * seconds)))
    sample = Q[:n]
    t0 = time.perf_counter()
    port.eval(sample, 2.0, nthreads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"first {n} of the workload's queries (same mesh), "
                      f"precompute {build_s:.3f} s not included",
            "precompute_s": build_s}, Wprobe


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm on the host cores."""
    if rank != 0:
        return
    V, F, Q = make_workload(args, 0)
    from oracle import oracle as O
    nthreads = O.num_threads(0)
    port = O.SoupPort(V, F, order=2)
    # size one step to a bounded sample (~3 s of CPU work)
    probe = Q[:100_000]
    t0 = time.perf_counter()
    port.eval(probe, 2.0, nthreads)
    rate = len(probe) / max(time.perf_counter() - t0, 1e-9)
    n = int(min(len(Q), max(100_000, rate * 3.0)))
    sample = Q[:n]
    for _ in range(args.warmup):
        port.eval(sample[: min(n, 100_000)], 2.0, nthreads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        port.eval(sample, 2.0, nthreads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n * args.steps / total
    ntri = int(F.shape[0])
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": soup_config(args, ntri, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{n} queries per step of the {args.nq}-query workload "
                                   "(the reference's own algorithm and tree, FP32)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def timed_steps(fn, steps, warmup, stream):
    """Run fn() warmup times, then time `steps` calls with CUDA events."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    ev[0].record(stream)
    for k in range(steps):
        fn()
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    per = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
    return ev[0].elapsed_time(ev[-1]), per


def _line(value, ms_per_step, steps, warmup, config, **extra):
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps,
            "warmup": warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config, **extra}


def exact_c1(steps, warmup):
    """Configuration C1: exact winding number, icosphere subdiv 4 (5120
    triangles, radial noise), 100k float64 queries in [-1.5,1.5]^3; mixed
    and plain FP64 (both through the cap hierarchy), against the CPU
    restatement of the reference's hierarchy on all queries."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    V, F, Q = synth.exact_workload(seed=0, subdiv=4, nq=100_000)
    dV, dF, dQ = (torch.from_numpy(x).cuda() for x in (V, F, Q))
    stream = torch.cuda.current_stream()
    out = {}
    for prec in ("mixed", "fp64"):
        W = None

        def step():
            nonlocal W
            W = G.winding_number(dV, dF, dQ, precision=prec)
        total, per = timed_steps(step, steps, warmup, stream)
        out[prec] = (Q.shape[0] * steps / (total / 1e3), total / steps, W.cpu().numpy())
    Wm, W64 = out["mixed"][2], out["fp64"][2]
    t0 = time.perf_counter()
    Wref = O.winding_number_hier(V, F, Q)
    cpu_s = time.perf_counter() - t0
    err = np.abs(Wm - Wref)
    return {"config": {"workload": "exact_icosphere4_noise_100kq", "triangles": int(F.shape[0]),
                       "queries": int(Q.shape[0])},
            "mixed_qps": out["mixed"][0], "mixed_ms": out["mixed"][1],
            "fp64_qps": out["fp64"][0], "fp64_ms": out["fp64"][1],
            "mixed_over_fp64": out["mixed"][0] / out["fp64"][0],
            "accuracy": {"max_abs_dW_vs_cpu_fp64": float(err.max()),
                         "p99_abs_dW": float(np.quantile(err, 0.99)),
                         "labels_identical": bool(np.array_equal(Wm > 0.5, Wref > 0.5)),
                         "fp64_gpu_vs_cpu_max": float(np.abs(W64 - Wref).max())},
            "cpu_baseline": {"value": Q.shape[0] / cpu_s, "unit": UNIT,
                             "cores": O.num_threads(0), "kind": "port",
                             "sample": "all 100k queries, hierarchical exact restatement "
                                       "(oracle/wn_hier.cpp), build included"}}


def run_exact_line(args):
    r = exact_c1(args.steps, args.warmup)
    print(json.dumps(_line(r["mixed_qps"], r["mixed_ms"], args.steps, args.warmup, r["config"],
                           accuracy=r["accuracy"],
                           plain_fp64={"value": r["fp64_qps"], "ms_per_step": r["fp64_ms"],
                                       "mixed_speedup": r["mixed_over_fp64"]},
                           cpu_baseline=r["cpu_baseline"])), flush=True)


def cloud_c3(steps, warmup):
    """Configuration C3: point-cloud FWN, 2M torus samples, 8M queries,
    order 2, beta 2; octree and precompute timed, mixed and FP64 walks,
    the CPU restatement of the reference on a 200k-query sample."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    P, Nn, A = synth.torus_cloud(seed=3, n=2_000_000)
    Q = synth.cloud_queries(seed=4, nq=8_000_000)
    dP, dN, dA = (torch.from_numpy(x).cuda() for x in (P, Nn, A))
    torch.cuda.synchronize()
    # the first build in the process also grows the device memory pool: it
    # is timed apart from a second, warm build
    t0 = time.perf_counter()
    tree0 = G.Octree(dP)
    torch.cuda.synchronize()
    octree_first_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ce0 = G.CloudExpansion(dP, dN, dA, order=2, tree=tree0)
    torch.cuda.synchronize()
    pre_first_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    tree = G.Octree(dP)
    torch.cuda.synchronize()
    octree_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ce = G.CloudExpansion(dP, dN, dA, order=2, tree=tree)
    torch.cuda.synchronize()
    pre_s = time.perf_counter() - t0
    del ce0, tree0
    dQ = torch.from_numpy(Q).cuda()
    stream = torch.cuda.current_stream()
    res = {}
    for prec, st in (("mixed", steps), ("fp64", max(1, steps // 5))):
        W = None

        def step():
            nonlocal W
            W = ce.eval(dQ, 2.0, precision=prec)
        total, per = timed_steps(step, st, min(warmup, 3), stream)
        res[prec] = (Q.shape[0] * st / (total / 1e3), total / st, W.cpu().numpy())
    Wm, W64 = res["mixed"][2], res["fp64"][2]
    err = np.abs(Wm - W64)
    out_band = np.abs(W64 - 0.5) > 1e-3
    nc = O.num_threads(0)
    t0 = time.perf_counter()
    ot = O.octree(P)
    CM, R, EC = O.cloud_precompute(P, Nn, A, ot, 2)
    cpu_pre = time.perf_counter() - t0
    sample = Q[:200_000]
    t0 = time.perf_counter()
    Wc = O.cloud_eval(P, Nn, A, ot, CM, R, EC, sample, 2.0)
    cpu_s = time.perf_counter() - t0
    return {"config": {"workload": "cloud_torus_2Mpts_8Mq", "points": int(P.shape[0]),
                       "queries": int(Q.shape[0]), "order": 2, "beta": 2.0,
                       "cells": int(tree.sizes()[0])},
            "mixed_qps": res["mixed"][0], "mixed_ms": res["mixed"][1],
            "fp64_qps": res["fp64"][0], "fp64_ms": res["fp64"][1],
            "mixed_over_fp64": res["mixed"][0] / res["fp64"][0],
            "octree_ms": octree_s * 1e3, "precompute_ms": pre_s * 1e3,
            "octree_first_call_ms": octree_first_s * 1e3,
            "precompute_first_call_ms": pre_first_s * 1e3,
            "accuracy": {"max_abs_dW": float(err.max()), "p99_abs_dW": float(np.quantile(err, 0.99)),
                         "label_mismatch_outside_band":
                             int(((Wm > 0.5) != (W64 > 0.5))[out_band].sum()),
                         "fp64_vs_cpu_oracle_max": float(np.abs(W64[:len(sample)] - Wc).max()),
                         "queries_compared": int(Q.shape[0])},
            "cpu_baseline": {"value": len(sample) / cpu_s, "unit": UNIT, "cores": nc,
                             "kind": "port", "precompute_s": cpu_pre,
                             "sample": f"first {len(sample)} queries (oracle restatement of "
                                       "fast_winding_number.cpp), octree+precompute timed apart"}}


def run_cloud_line(args):
    r = cloud_c3(args.steps, args.warmup)
    print(json.dumps(_line(r["mixed_qps"], r["mixed_ms"], args.steps, args.warmup, r["config"],
                           accuracy=r["accuracy"],
                           plain_fp64={"value": r["fp64_qps"], "ms_per_step": r["fp64_ms"],
                                       "mixed_speedup": r["mixed_over_fp64"]},
                           octree_s=r["octree_ms"] / 1e3, precompute_s=r["precompute_ms"] / 1e3,
                           cpu_baseline=r["cpu_baseline"])), flush=True)


def precision_c4(fp64_sample):
    """Configuration C4: 500k-triangle deformed geodesic sphere (nu = 158)
    with one 2000-triangle hole; 1M queries at 10^-k (k = 1..7) along vertex
    normals, inside and outside.  Mixed vs plain FP64, exact and soup paths,
    per decade: max / p99 |dW| and label mismatches outside 0.5 +- 1e-3; the
    CPU restatement of the reference's hierarchy timed on the FP64 sample."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    V, F, Q, dec, side = synth.precision_workload(seed=5)
    dV, dF, dQ = (torch.from_numpy(x).cuda() for x in (V, F, Q))
    rng = np.random.default_rng(0)
    # FP64 reference sample: fp64_sample queries per (decade, side)
    idx = []
    for k in range(1, 8):
        for sd in (-1.0, 1.0):
            cand = np.nonzero((dec == k) & (side == sd))[0]
            idx.append(rng.choice(cand, size=min(fp64_sample, cand.size), replace=False))
    idx = np.sort(np.concatenate(idx))
    report = {"triangles": int(F.shape[0]), "queries": int(Q.shape[0]),
              "fp64_reference_queries": int(idx.size)}
    G.winding_number(dV, dF, dQ[:4096], precision="mixed")  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    We_m = G.winding_number(dV, dF, dQ, precision="mixed").cpu().numpy()
    report["exact_mixed_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    We_64 = G.winding_number(dV, dF, dQ[idx], precision="fp64").cpu().numpy()
    report["exact_fp64_s_sample"] = time.perf_counter() - t0
    bvh = G.FastWindingNumberBVH(dV, dF, 2)
    Ws_m = bvh.eval(dQ, 2.0, "mixed").cpu().numpy()
    Ws_64 = bvh.eval(dQ, 2.0, "fp64").cpu().numpy()

    def stats(a, b, mask):
        e = np.abs(a - b)[mask]
        out = np.abs(b - 0.5)[mask] > 1e-3
        return {"n": int(mask.sum()), "max": float(e.max()), "p99": float(np.quantile(e, 0.99)),
                "label_mismatch_outside_band": int(((a > 0.5) != (b > 0.5))[mask][out].sum())}
    per = []
    for k in range(1, 8):
        m_all = dec == k
        m_s = dec[idx] == k
        per.append({"distance": 10.0 ** -k,
                    "exact_mixed_vs_fp64": stats(We_m[idx], We_64, m_s),
                    "soup_mixed_vs_fp64": stats(Ws_m, Ws_64, m_all),
                    "soup_fp64_vs_exact_fp64": stats(Ws_64[idx], We_64, m_s)})
    report["per_decade"] = per
    report["worst"] = {
        "exact_mixed_vs_fp64_max": max(d["exact_mixed_vs_fp64"]["max"] for d in per),
        "soup_mixed_vs_fp64_max": max(d["soup_mixed_vs_fp64"]["max"] for d in per),
        "label_mismatches": sum(d["exact_mixed_vs_fp64"]["label_mismatch_outside_band"] +
                                d["soup_mixed_vs_fp64"]["label_mismatch_outside_band"]
                                for d in per)}
    sub = idx[: min(idx.size, 20_000)]
    t0 = time.perf_counter()
    O.winding_number_hier(V, F, Q[sub])
    cpu_s = time.perf_counter() - t0
    report["exact_mixed_qps"] = Q.shape[0] / report["exact_mixed_s"]
    report["cpu_baseline"] = {"value": sub.size / cpu_s, "unit": UNIT, "cores": O.num_threads(0),
                              "kind": "port",
                              "sample": f"{sub.size} of the FP64 sample's queries, hierarchical "
                                        "exact restatement (oracle/wn_hier.cpp), build included"}
    return report


def run_precision_study(args):
    r = precision_c4(args.fp64_sample)
    print(json.dumps({"workload": "precision_study_geodesic158_hole2000_1Mq", **r}), flush=True)


def _served_mesh(spec):
    from libigl_gb300 import synth
    V, F = synth.served_mesh(spec)
    return np.ascontiguousarray(V), np.ascontiguousarray(F, np.int32)


def served_meshes(count):
    """The served workload's meshes (256 by default), generated in parallel."""
    import multiprocessing as mp
    from libigl_gb300 import synth
    specs = synth.served_meshes(seed=6, count=count)
    order = sorted(range(len(specs)), key=lambda i: -specs[i]["nu"])
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        gen = pool.map(_served_mesh, [specs[i] for i in order], chunksize=1)
    meshes = [None] * len(specs)
    for i, m in zip(order, gen):
        meshes[i] = m
    return meshes


def served_c5(meshes, trace_s, budget_bytes, nsat=1000, nsat_fp64=1000, cpu=True, seed=7):
    """Configuration C5 through gwn_server: the meshes resident under an HBM
    budget (LRU eviction, trees built on the server's builder thread);
    Poisson arrivals at 2000 requests/s, each a uniform mesh with n_q
    log-uniform in [1e3, 1e6] float32 queries uniform in that mesh's box.
    Served throughput, p50/p99 submit-to-result latency, builds and
    evictions during the trace, then the saturated throughput of the first
    nsat requests in mixed precision and in plain FP64 through the same
    server, and the CPU soup FWN (the reference's algorithm) on a sample of
    the trace's requests."""
    import threading
    import torch
    import libigl_gb300 as G
    from oracle import oracle as O
    torch.cuda.set_device(0)
    S = G.Server(hbm_budget_bytes=budget_bytes, max_batch_queries=1 << 22, slots=3)
    ids = [S.add_mesh(V, F) for V, F in meshes]
    ntri = np.array([F.shape[0] for _, F in meshes])
    rng = np.random.default_rng(seed)
    pool_n = 1_000_000
    pools = []
    for V, _ in meshes:
        lo, hi = V.min(0), V.max(0)
        pools.append((lo + rng.random((pool_n, 3)) * (hi - lo)).astype(np.float32))
    # warm-up: one small request per mesh builds every tree (admission; under
    # a budget below the resident set this already evicts)
    t0 = time.perf_counter()
    reqs = [S.submit(ids[k], pools[k][:256]) for k in range(len(ids))]
    for r in reqs:
        r.wait()
    warm_s = time.perf_counter() - t0
    st0 = S.stats()
    rate = 2000.0
    nreq = int(rate * trace_s)
    arr = np.cumsum(rng.exponential(1.0 / rate, nreq))
    mesh_of = rng.integers(len(ids), size=nreq)
    nq_of = np.exp(rng.uniform(np.log(1e3), np.log(1e6), nreq)).astype(np.int64)
    off_of = (rng.random(nreq) * (pool_n - nq_of)).astype(np.int64)
    lat = np.zeros(nreq)
    done_t = np.zeros(nreq)
    handles = [None] * nreq
    ready = threading.Semaphore(0)

    def waiter():
        for i in range(nreq):
            ready.acquire()
            _, lat[i] = handles[i].wait()
            done_t[i] = time.perf_counter()
    wt = threading.Thread(target=waiter)
    wt.start()
    launches0 = G.launch_count()
    t_start = time.perf_counter()
    for i in range(nreq):
        delay = t_start + arr[i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        k = int(mesh_of[i])
        handles[i] = S.submit(ids[k], pools[k][off_of[i]:off_of[i] + nq_of[i]])
        ready.release()
    wt.join()
    span = done_t.max() - t_start
    st1 = S.stats()
    launches = G.launch_count() - launches0
    served_q = int(nq_of.sum())

    def saturated(precision, n):
        a = S.stats()
        t = time.perf_counter()
        hs = [S.submit(ids[int(mesh_of[i])],
                       pools[int(mesh_of[i])][off_of[i]:off_of[i] + nq_of[i]], 2.0, precision)
              for i in range(n)]
        for h in hs:
            h.wait()
        wall = time.perf_counter() - t
        b = S.stats()
        return {"requests": n, "qps": int(nq_of[:n].sum()) / wall, "wall_s": wall,
                "walk_gpu_ms": b["walk_gpu_ms"] - a["walk_gpu_ms"],
                "batch_gpu_ms": b["batch_gpu_ms"] - a["batch_gpu_ms"],
                "batches": b["batches"] - a["batches"], "builds": b["builds"] - a["builds"]}
    sat_m = saturated("mixed", min(nsat, nreq))
    sat_d = saturated("fp64", min(nsat_fp64, nreq))
    S.close()
    out = {"config": {"workload": "served_256_meshes_poisson_2000rps", "meshes": len(ids),
                      "triangles_total": int(ntri.sum()), "requests": nreq,
                      "queries": served_q, "offered_qps": served_q / arr[-1],
                      "trace_s": trace_s, "qdtype": "f32",
                      "hbm_budget_gb": budget_bytes / 2**30, "slots": 3,
                      "max_batch_queries": 1 << 22},
           "qps": served_q / span, "span_s": span,
           "p50_ms": float(np.percentile(lat, 50) * 1e3),
           "p99_ms": float(np.percentile(lat, 99) * 1e3),
           "mean_ms": float(lat.mean() * 1e3),
           "batches": st1["batches"] - st0["batches"],
           "walk_gpu_ms": st1["walk_gpu_ms"] - st0["walk_gpu_ms"],
           "batch_gpu_ms": st1["batch_gpu_ms"] - st0["batch_gpu_ms"],
           "refined": st1["refined"] - st0["refined"],
           "builds_during_trace": st1["builds"] - st0["builds"],
           "evictions_during_trace": st1["evictions"] - st0["evictions"],
           "resident": {"meshes": st1["resident_meshes"], "bytes": st1["resident_bytes"],
                        "peak_bytes": st1["peak_resident_bytes"], "builds": st1["builds"],
                        "evictions": st1["evictions"], "admission_s": warm_s},
           "saturated": {"mixed_qps": sat_m["qps"], "fp64_qps": sat_d["qps"],
                         "mixed_over_fp64": sat_m["qps"] / sat_d["qps"],
                         "mixed": sat_m, "fp64": sat_d},
           "gpu_launches": launches, "kernels_per_batch": st1["kernels_per_batch"]}
    if cpu:
        # the reference's soup FWN on the host cores: the first 6 requests of
        # the trace whose mesh has at most 500k triangles (precompute apart)
        nthreads = O.num_threads(0)
        picked = [i for i in range(nreq) if ntri[mesh_of[i]] <= 500_000][:6]
        q_tot, t_eval, t_pre = 0, 0.0, 0.0
        for i in picked:
            V, F = meshes[int(mesh_of[i])]
            t0 = time.perf_counter()
            port = O.SoupPort(V, F, order=2)
            t_pre += time.perf_counter() - t0
            Qi = pools[int(mesh_of[i])][off_of[i]:off_of[i] + nq_of[i]].astype(np.float64)
            t0 = time.perf_counter()
            port.eval(Qi, 2.0, nthreads)
            t_eval += time.perf_counter() - t0
            q_tot += Qi.shape[0]
        out["cpu_baseline"] = {"value": q_tot / max(t_eval, 1e-9), "unit": UNIT,
                               "cores": nthreads, "kind": "port", "precompute_s": t_pre,
                               "sample": f"{len(picked)} requests of the trace ({q_tot} queries, "
                                         "meshes <= 500k triangles), oracle/soup_hdk.cpp, "
                                         "precompute timed apart"}
    return out


def run_served_line(args):
    t0 = time.perf_counter()
    meshes = served_meshes(args.served_meshes)
    gen_s = time.perf_counter() - t0
    r = served_c5(meshes, args.served_seconds, 120 << 30)
    print(json.dumps(_line(r["qps"], r["span_s"] * 1e3, 1, 1, r["config"],
                           **{k: v for k, v in r.items() if k not in ("config", "qps")},
                           mesh_generation_s=gen_s)), flush=True)


def run_point_areas_line(args):
    """Per-point areas (igl::copyleft::cgal::point_areas) of the C3 torus
    cloud (2M points) from its 21 nearest points, as
    copyleft/cgal/fast_winding_number.cpp:36-38 computes them; then the
    whole points-only winding number (octree, knn, areas, expansions, 8M
    queries).  CPU baseline: the oracle restatement (brute-force Delaunay,
    not CGAL: CGAL is not in the image) on a sample of points."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    P, Nn, _ = synth.torus_cloud(seed=3, n=2_000_000)
    dP, dN = torch.from_numpy(P).cuda(), torch.from_numpy(Nn).cuda()
    stream = torch.cuda.current_stream()
    I = None

    def knn_step():
        nonlocal I
        I = G.knn(dP, dP, 21)
    knn_total, _ = timed_steps(knn_step, max(1, args.steps // 2), 2, stream)
    A = None

    def step():
        nonlocal A
        A = G.point_areas(dP, I, dN)
    total, per = timed_steps(step, args.steps, args.warmup, stream)
    n = P.shape[0]
    Ah, Ih = A.cpu().numpy(), I.cpu().numpy()
    sample = 20_000
    t0 = time.perf_counter()
    Ao, _ = O.point_areas(P, Ih[:sample], Nn)
    cpu_s = time.perf_counter() - t0
    rel = np.abs(Ah[:sample] - Ao) / np.maximum(np.abs(Ao), 1e-300)
    Q = synth.cloud_queries(seed=4, nq=8_000_000)
    dQ = torch.from_numpy(Q).cuda()
    W = None

    def full():
        nonlocal W
        W = G.fast_winding_number_cloud_points(dP, dN, dQ, 2, 2.0, precision="mixed")
    full_total, _ = timed_steps(full, 2, 1, stream)
    line = _line(n * args.steps / (total / 1e3), total / args.steps, args.steps, args.warmup,
                 {"workload": "point_areas_torus_2Mpts_k21", "points": n, "k": 21},
                 metric_note="points/s of gwn_point_areas (unit below is per point)",
                 knn_ms=knn_total / max(1, args.steps // 2),
                 accuracy={"vs_cpu_restatement_rel_max": float(rel.max()),
                           "vs_cpu_restatement_rel_p999": float(np.quantile(rel, 0.999)),
                           "points_compared": sample,
                           "area_sum_over_torus_area":
                               float(Ah.sum() / (4 * np.pi ** 2 * 1.0 * 0.35))},
                 points_only_fwn={"queries": int(Q.shape[0]), "ms_per_call": full_total / 2,
                                  "qps_including_precompute": Q.shape[0] / (full_total / 2e3)},
                 cpu_baseline={"value": sample / cpu_s, "unit": "points/s",
                               "cores": O.num_threads(0), "kind": "port",
                               "sample": f"first {sample} points, oracle/point_areas.cpp "
                                         "(brute-force Delaunay, not CGAL)"})
    line["unit"] = "points/s"
    print(json.dumps(line), flush=True)


def run_signed_distance_line(args):
    """igl::signed_distance with the fast-winding-number sign on the C2 mesh
    (1,297,489 triangles), 1M float64 queries of the C2 distribution.
    value = queries/s of the whole call on device-resident arrays (the tree
    is built inside every call, as the reference builds its AABB and soup
    tree); e2e = the same call from host arrays; closest_only_qps = closest
    triangles on a built tree; CPU baseline = the AABB restatement
    (oracle/aabb.cpp) + the reference's soup winding number on the host
    cores, on a 200k-query sample, trees built apart."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    V, F = synth.soup_mesh(seed=1, subdiv=8)
    Q = synth.soup_queries(V, F, seed=2, nq=1_000_000)
    dQ, dV, dF = (torch.from_numpy(x).cuda() for x in (Q, V, F))
    stream = torch.cuda.current_stream()
    out = {}
    FWN = G.SIGNED_DISTANCE_TYPE_FAST_WINDING_NUMBER

    def step():
        out["S"], out["I"], out["C"] = G.signed_distance(dQ, dV, dF, FWN)
    total, per = timed_steps(step, args.steps, args.warmup, stream)
    launches = G.launch_count_of(step)
    bvh = G.FastWindingNumberBVH(dV, dF, 2)
    walk = {}

    def closest_only():
        walk["D"] = bvh.squared_distance(dQ)
    tc, _ = timed_steps(closest_only, args.steps, args.warmup, stream)
    t0 = time.perf_counter()
    S1, I1, C1 = G.signed_distance(Q, V, F, FWN)
    one_shot = time.perf_counter() - t0
    # CPU: AABB restatement + reference soup winding number, on a sample
    ns = 200_000
    sample = Q[:ns]
    t0 = time.perf_counter()
    tree = O.AABB(V, F)
    port = O.SoupPort(V.astype(np.float32).astype(np.float64), F, order=2)
    cpu_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    Dc, Ic, Cc = tree.squared_distance(sample)
    wc = port.eval(sample, 2.0)
    cpu_s = time.perf_counter() - t0
    D = walk["D"][0].cpu().numpy()[:ns]
    Sg = out["S"].cpu().numpy()[:ns]
    Sc = (1.0 - 2.0 * np.abs(wc)) * np.sqrt(Dc)
    d_err = np.abs(D - Dc) / np.maximum(Dc, 1e-300)
    line = {"metric": "signed distance queries/s (closest triangle FP64 + winding-number sign)",
            "value": Q.shape[0] * args.steps / (total / 1e3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "signed_distance_fwn_icosphere8_sh_1pct_holes_1Mq",
                       "triangles": int(F.shape[0]), "queries": int(Q.shape[0]),
                       "sign": "FAST_WINDING_NUMBER (order 2, accuracy 2, mixed)"},
            "closest_only_qps": Q.shape[0] * args.steps / (tc / 1e3),
            "e2e": {"value": Q.shape[0] / one_shot, "unit": UNIT,
                    "h2d_bytes_per_step": int(Q.nbytes + V.nbytes + F.nbytes),
                    "d2h_bytes_per_step": int(Q.shape[0] * (8 + 4 + 24))},
            "accuracy": {"sqrD_max_rel_vs_cpu_aabb": float(d_err.max()),
                         "S_max_abs_vs_cpu": float(np.abs(Sg - Sc).max()),
                         "sign_mismatch": int(((Sg < 0) != (Sc < 0))[np.abs(wc - 0.5) > 0.05].sum()),
                         "queries_compared": ns},
            "gpu_launches": launches,
            "cpu_baseline": {"value": ns / cpu_s, "unit": UNIT, "cores": O.num_threads(0),
                             "kind": "port", "build_s": cpu_build,
                             "sample": f"first {ns} queries: igl::AABB restatement "
                                       "(oracle/aabb.cpp) + reference soup winding number "
                                       "(oracle/soup_hdk.cpp), trees built apart"}}
    print(json.dumps(line), flush=True)


def run_knn_line(args):
    """igl::knn on the C3 cloud: the 16 nearest of the 2M torus points for
    1M of the points themselves (the use of knn before point areas).
    value = queries/s on a built octree (device arrays); one-shot = octree
    build + search from host arrays; CPU baseline = the restated reference
    best-first search (oracle/knn.cpp) on the host cores, 20k-query sample."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    P, _, _ = synth.torus_cloud(seed=3, n=2_000_000)
    Q = P[::2][:1_000_000]
    k = 16
    dP, dQ = torch.from_numpy(P).cuda(), torch.from_numpy(Q).cuda()
    tree = G.Octree(dP)
    stream = torch.cuda.current_stream()
    out = {}

    def step():
        out["I"] = tree.knn(dQ, k)
    total, _ = timed_steps(step, args.steps, args.warmup, stream)
    launches = G.launch_count_of(step)
    t0 = time.perf_counter()
    I1 = G.knn(Q, P, k)
    one_shot = time.perf_counter() - t0
    ns = 20_000
    t0 = time.perf_counter()
    ot = O.octree(P)
    cpu_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    Ir = O.knn(Q[:ns], P, k, ot)
    cpu_s = time.perf_counter() - t0
    Ig = out["I"].cpu().numpy()
    line = {"metric": "knn queries/s (k = 16, exact FP64 distances)",
            "value": Q.shape[0] * args.steps / (total / 1e3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "knn_torus_2Mpts_1Mq_k16", "points": int(P.shape[0]),
                       "queries": int(Q.shape[0]), "k": k},
            "e2e": {"value": Q.shape[0] / one_shot, "unit": UNIT,
                    "h2d_bytes_per_step": int(P.nbytes + Q.nbytes),
                    "d2h_bytes_per_step": int(Q.shape[0] * k * 4)},
            "accuracy": {"identical_to_cpu_reference_search": bool(np.array_equal(Ig[:ns], Ir)),
                         "one_shot_identical": bool(np.array_equal(I1, Ig)),
                         "queries_compared": ns},
            "gpu_launches": launches,
            "cpu_baseline": {"value": ns / cpu_s, "unit": UNIT, "cores": O.num_threads(0),
                             "kind": "port", "build_s": cpu_build,
                             "sample": f"first {ns} queries, the reference's best-first search "
                                       "restated (oracle/knn.cpp), octree built apart"}}
    print(json.dumps(line), flush=True)


def run_eytzinger_line(args):
    """igl::eytzinger_aabb_winding_number (2-D segments): 16 x 16 cells of
    wavy closed loops, 1M segments, 10M uniform float64 query points.  value =
    queries/s of the mixed-precision evaluation on device-resident arrays
    (tree and pairs built once); e2e = the same call from pinned host arrays
    (points, mesh and tree copied in, W out, every step); plain FP64 and the
    build (tree + pairs) timed beside it; CPU baseline = the restated
    reference walk (oracle/eytzinger.cpp) on all host cores, 2M-query sample."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    V, E = synth.loops2d(seed=7, n_segments=1_000_000, n_cells=16)
    P = synth.loops2d_queries(16, seed=8, nq=10_000_000)
    PB1, PB2 = O.segment_boxes(V, E)
    stream = torch.cuda.current_stream()
    dV, dE, dP, dPB1, dPB2 = (torch.from_numpy(x).cuda() for x in (V, E, P, PB1, PB2))
    tree = {}

    def build():
        tree["B1"], tree["B2"], tree["leaf"] = G.eytzinger_aabb(dPB1, dPB2)
        tree["I"], tree["C"] = G.eytzinger_aabb_winding_number_tree(dE, tree["leaf"])
    build_ms, _ = timed_steps(build, 3, 2, stream)
    build_ms /= 3
    out = {}

    def run(prec):
        def step():
            out[prec] = G.eytzinger_aabb_winding_number(dP, dV, dE, tree["B1"], tree["B2"],
                                                        tree["leaf"], tree["I"], tree["C"],
                                                        precision=prec)
        return step
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    for _ in range(max(args.warmup, 3)):
        run("mixed")()
    torch.cuda.synchronize()
    G.profile_enable(True, accumulate=True)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for k in range(args.steps):
        run("mixed")()
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    total = ev[0].elapsed_time(ev[-1])
    clocks = sampler.stop()
    phases = {k: v / args.steps for k, v in G.profile_read().items()}
    walk_ms = [phases.get("walk", float("nan"))]
    G.profile_enable(False)
    launches = G.launch_count_of(run("mixed"))
    fp64_ms, _ = timed_steps(run("fp64"), 2, 1, stream)
    fp64_ms /= 2
    Wm, W64 = out["mixed"].cpu().numpy(), out["fp64"].cpu().numpy()
    err = np.abs(Wm - W64)
    away = np.abs(W64 - 0.5) > 1e-3
    nq = P.shape[0]
    # e2e through the C ABI from pinned host arrays
    h = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in
         (("P", P), ("V", V), ("E", E), ("B1", tree["B1"].cpu().numpy()),
          ("B2", tree["B2"].cpu().numpy()), ("leaf", tree["leaf"].cpu().numpy()),
          ("I", tree["I"].cpu().numpy()), ("C", tree["C"].cpu().numpy()))}
    hn = {k: v.numpy() for k, v in h.items()}

    def host_step():
        out["host"] = G.eytzinger_aabb_winding_number(hn["P"], hn["V"], hn["E"], hn["B1"],
                                                      hn["B2"], hn["leaf"], hn["I"], hn["C"],
                                                      precision="mixed")
    host_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        host_step()
    e2e_s = (time.perf_counter() - t0) / args.steps
    h2d = sum(int(v.nbytes) for v in hn.values())
    # CPU baseline: the reference's build and walk restated, all host cores
    t0 = time.perf_counter()
    rB1, rB2, rleaf = O.eytzinger_aabb(PB1, PB2, median_mode=0)
    rI, rC = O.eytzinger_wn_tree(E, rleaf, canonical=False)
    cpu_build_s = time.perf_counter() - t0
    ns = 2_000_000
    t0 = time.perf_counter()
    Wr = O.eytzinger_winding_number(P[:ns], V, E, rB1, rB2, rleaf, rI, rC)
    cpu_s = time.perf_counter() - t0
    nodes = int(tree["leaf"].shape[0])
    npairs = int(tree["I"].shape[0]) // 2
    walk = float(np.nanmean(walk_ms))
    alg_bytes = nq * (16 + 4 + 8) + nodes * 48 + npairs * 24
    peaks, peak_kind = load_peaks()
    achieved = alg_bytes / (walk / 1e3) / 1e9
    line = {"metric": "2-D winding queries/s (Eytzinger AABB, |dW| <= 1e-4 vs FP64)",
            "value": nq * args.steps / (total / 1e3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic",
            "config": {"workload": "eytzinger2d_loops_1Mseg_10Mq", "segments": int(E.shape[0]),
                       "queries": nq, "tree_slots": nodes, "pairs": npairs,
                       "l2": "inputs larger than L2 (160 MB of queries)"},
            "e2e": {"value": nq / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": int(nq * 8), "ms_per_step": 1e3 * e2e_s},
            "plain_fp64": {"value": nq / (fp64_ms / 1e3), "unit": UNIT,
                           "ratio_mixed_over_fp64": (nq * args.steps / (total / 1e3))
                           / (nq / (fp64_ms / 1e3))},
            "build_ms": build_ms, "phases_ms_per_step": phases,
            "accuracy": {"max_abs_dW": float(err.max()), "p99_abs_dW": float(np.quantile(err, .99)),
                         "label_mismatch_outside_band":
                             int((np.round(Wm) != np.round(W64))[away].sum()),
                         "fp64_vs_cpu_reference_max": float(np.abs(W64[:ns] - Wr).max()),
                         "host_call_identical": bool(np.array_equal(out["host"], Wm))},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                         "traffic": ncu_traffic("eytzinger_walk_2d"), "peak_source": peak_kind,
                         "kernel": "eval_mixed_kernel", "kernel_ms": walk,
                         "algorithmic_bytes": alg_bytes},
            "clocks": clocks, "gpu_launches": launches,
            "cpu_baseline": {"value": ns / cpu_s, "unit": UNIT, "cores": O.num_threads(0),
                             "kind": "port", "build_s": cpu_build_s,
                             "sample": f"first {ns} queries, the reference's walk restated "
                                       "(oracle/eytzinger.cpp) over its own tree"}}
    print(json.dumps(line), flush=True)


def run_swept_line(args):
    """igl::swept_volume_signed_distance: a 20,480-triangle deformed ellipsoid
    under 64 rigid motions of a screw, a 128 x 69 x 60 grid (529,920 points)
    around the sweep, isolevel 0, sign SIGNED_DISTANCE_TYPE_DEFAULT (exact
    winding number).  value = grid-point evaluations per second (#GV x
    #transforms / s) of the device call on device arrays (tree built inside,
    as the reference does; the sign's exact winding number in mixed
    precision, plain FP64 timed beside it); e2e = the same call from host
    arrays; CPU
    baseline = the restated reference loop (oracle.swept_volume_signed_
    distance: AABB, exact winding number, flood fill) on the first 4
    transforms, all host cores; accuracy = GPU vs that restatement on the
    same 4 transforms."""
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import synth
    from oracle import oracle as O
    V, F, T, GV, res, h = synth.swept_workload()
    sign = G.SIGNED_DISTANCE_TYPE_DEFAULT
    dV, dF, dGV = (torch.from_numpy(x).cuda() for x in (V, F, GV))
    stream = torch.cuda.current_stream()
    out = {}

    def step():
        out["S"] = G.swept_volume_signed_distance(dV, dF, T, sign, dGV, res, h, 0.0)
    steps = min(args.steps, 5)
    G.profile_enable(True)
    total, per = timed_steps(step, steps, max(args.warmup, 1), stream)
    phases = G.profile_read()  # the last sweep's phases
    G.profile_enable(False)
    launches = G.launch_count_of(step)
    nG, nT = GV.shape[0], T.shape[0]
    t0 = time.perf_counter()
    Sh = G.swept_volume_signed_distance(V, F, T, sign, GV, res, h, 0.0)
    e2e_s = time.perf_counter() - t0
    k = 4
    S4 = G.swept_volume_signed_distance(V, F, T[:k], sign, GV, res, h, 0.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    S4_64 = G.swept_volume_signed_distance(dV, dF, T[:k], sign, dGV, res, h, 0.0,
                                           precision="fp64").cpu().numpy()
    fp64_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    Sr = O.swept_volume_signed_distance(V, F, T[:k], sign, GV, res, h, 0.0)
    cpu_s = time.perf_counter() - t0
    rel = np.abs(S4 - Sr) / np.maximum(np.abs(Sr), 1e-12)
    rel64 = np.abs(S4_64 - Sr) / np.maximum(np.abs(Sr), 1e-12)
    line = {"metric": "swept-volume grid-point evaluations/s (#GV x #transforms / s)",
            "value": nG * nT * steps / (total / 1e3), "unit": "evaluations/s", "n_gpus": 1,
            "steps": steps, "warmup": max(args.warmup, 1), "ms_per_step": total / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "swept_ellipsoid20k_64T_grid128", "triangles": int(F.shape[0]),
                       "transforms": int(nT), "grid": [int(x) for x in res],
                       "grid_points": int(nG), "h": h, "isolevel": 0.0,
                       "sign_type": "DEFAULT (exact winding number)"},
            "e2e": {"value": nG * nT / e2e_s, "unit": "evaluations/s",
                    "h2d_bytes_per_step": int(V.nbytes + F.nbytes + GV.nbytes + T.nbytes),
                    "d2h_bytes_per_step": int(nG * 8), "ms_per_step": 1e3 * e2e_s},
            "phases_ms_last_sweep": phases,
            "plain_fp64": {"value": nG * k / fp64_s, "unit": "evaluations/s",
                           "sample": f"first {k} transforms, device arrays"},
            "accuracy": {"nan_pattern_identical": bool(np.array_equal(np.isnan(S4), np.isnan(Sr))),
                         "max_rel_dS_mixed": float(np.nanmax(rel)),
                         "max_rel_dS_fp64": float(np.nanmax(rel64)),
                         "host_call_identical": bool(np.array_equal(Sh, out["S"].cpu().numpy(),
                                                                    equal_nan=True)),
                         "transforms_compared": k},
            "gpu_launches": launches,
            "cpu_baseline": {"value": nG * k / cpu_s, "unit": "evaluations/s",
                             "cores": O.num_threads(0), "kind": "port",
                             "sample": f"first {k} of {nT} transforms, the reference's loop "
                                       "restated over the oracle AABB / exact winding number"}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload != "soup":
        import torch
        if args.workload != "served":  # served starts its generator pool first
            torch.cuda.set_device(local)
        {"exact": run_exact_line, "cloud": run_cloud_line, "precision": run_precision_study,
         "served": run_served_line,
         "signed_distance": run_signed_distance_line, "knn": run_knn_line,
         "eytzinger2d": run_eytzinger_line, "swept": run_swept_line,
         "point_areas": run_point_areas_line}[args.workload](args)
        return
    import torch
    import libigl_gb300 as G
    from libigl_gb300 import _native as NV

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    V, F, Q = make_workload(args, rank)
    nq = Q.shape[0]
    qcode = NV.GWN_F64 if Q.dtype == np.float64 else NV.GWN_F32
    qbytes = Q.dtype.itemsize

    # precompute (tree + moments), timed on the device
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bvh = G.FastWindingNumberBVH(V, F, order=2, tree=args.tree)
    torch.cuda.synchronize()
    build_s_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    bvh2 = G.FastWindingNumberBVH(V, F, order=2, tree=args.tree)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    bvh2.close()
    stats = bvh.stats

    dQ = torch.from_numpy(Q).to(dev)
    dW = torch.empty(nq, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(prec="mixed"):
        bvh.eval_ptr(dQ.data_ptr(), qcode, nq, dW.data_ptr(), NV.GWN_F64, 2.0, prec,
                     stream.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    # timed region: per-step CUDA events on the launch stream + live phase
    # events (recorded by the library on its stream, read after the loop)
    G.profile_enable(True, accumulate=True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for k in range(args.steps):
        step()
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ph = G.profile_read()
    walk_ms = [ph.get("walk", float("nan")) / args.steps]
    G.profile_enable(False)
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * nq * args.steps / (total_ms / 1e3)
    ms_per_step = total_ms / args.steps

    # accuracy of the mixed result against the plain FP64 walk (untimed)
    step("mixed")
    Wm = dW.cpu().numpy().copy()
    torch.cuda.synchronize()
    e64 = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    e64[0].record(stream)
    step("fp64")
    e64[1].record(stream)
    torch.cuda.synchronize()
    fp64_ms = e64[0].elapsed_time(e64[1])
    W64 = dW.cpu().numpy()
    err = np.abs(Wm - W64)
    out = np.abs(W64 - 0.5) > 1e-3
    accuracy = {"max_abs_dW": float(err.max()), "p99_abs_dW": float(np.quantile(err, 0.99)),
                "label_mismatch_outside_band": int(((Wm > 0.5) != (W64 > 0.5))[out].sum()),
                "queries_compared": int(nq)}
    plain_fp64_qps = nq / (fp64_ms / 1e3)

    # e2e through the C ABI with pinned host buffers (copies inside the timing)
    e2e = None
    if not args.skip_e2e:
        hQ = torch.from_numpy(Q).pin_memory()
        hW = torch.empty(nq, dtype=torch.float64).pin_memory()
        L = NV.load()

        def host_step():
            NV.check(L.gwn_soup_eval(bvh._h, C.c_float(2.0), C.c_void_p(hQ.data_ptr()), qcode, nq,
                                     C.c_void_p(hW.data_ptr()), NV.GWN_F64, NV.GWN_MIXED,
                                     NV.GWN_HOST, None))

        host_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            host_step()
        e2e_s = time.perf_counter() - t0
        if dist:
            t = torch.tensor([e2e_s], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        assert np.array_equal(hW.numpy(), Wm), "host-buffer call differs from the device call"
        e2e = {"value": world * nq * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(nq * 3 * qbytes), "d2h_bytes_per_step": int(nq * 8),
               "ms_per_step": 1e3 * e2e_s / args.steps}

    # roofline of the dominant kernel (the mixed walk): HBM-level algorithmic
    # bytes per launch = queries in + order permutation in + results out + every
    # FP32 node record and leaf triangle once.
    peaks, peak_kind = load_peaks()
    walk = float(np.nanmean(walk_ms))
    nn, nt = stats["num_nodes"], stats["num_triangles"]
    alg_bytes = nq * (3 * qbytes + 4 + 8) + nn * 96 + nt * 48
    achieved = alg_bytes / (walk / 1e3) / 1e9
    traffic = ncu_traffic("soup_walk_c2")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "peak_source": peak_kind, "kernel": "soup_eval_mixed_kernel",
                "kernel_ms": walk, "kernel_share_of_step": walk / ms_per_step,
                "compute": walk_compute(bvh, dQ, nq, walk, clocks, peaks)}

    cpu = None
    vs_reference = None
    if rank == 0 and not args.skip_cpu:
        cpu, Wref = cpu_baseline(V, F, Q, args.cpu_seconds)
        # against the reference's own W (its algorithm and tree, FP32, as
        # restated bit for bit by the oracle) on the first queries
        n = Wref.shape[0]
        e = np.abs(Wm[:n] - Wref)
        out_ref = np.abs(Wref - 0.5) > 1e-3
        vs_reference = {"max_abs_dW": float(e.max()), "p99_abs_dW": float(np.quantile(e, 0.99)),
                        "p999_abs_dW": float(np.quantile(e, 0.999)),
                        "label_mismatch_outside_band":
                            int(((Wm[:n] > 0.5) != (Wref > 0.5))[out_ref].sum()),
                        "queries_compared": int(n),
                        "note": "mixed GPU result vs the reference's FP32 soup algorithm "
                                "(oracle/soup_hdk.cpp, bit-exact restatement) on the first "
                                f"{n} queries; tree={args.tree}"}

    # kernels launched per step by the library (counted in the library's launch sites)
    launches_per_step = G.launch_count_of(lambda: step())
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step,
        "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": soup_config(args, nt, world),
        "precision": "mixed",
        "accuracy": dict(accuracy, vs_reference=vs_reference),
        "plain_fp64": {"value": plain_fp64_qps, "unit": UNIT, "ms_per_step": fp64_ms,
                       "mixed_speedup": value / world / plain_fp64_qps},
        "precompute_s": build_s, "precompute_first_call_s": build_s_first,
        "tree": stats,
        "roofline": roofline, "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu,
        "gpu_launches": int(launches_per_step * args.steps),
    }
    if rank == 0 and world == 1 and not args.no_extras:
        line.update(run_extras(args))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_extras(args):
    """The other configurations as sub-results of the default line, each
    with its own CPU baseline: exact_c1, cloud_c3, precision_c4, served_c5
    (120 GB budget, every tree resident) and served_c5_pressure (a budget
    below the resident set: builds and evictions during the trace).  A
    failing sub-result records its error instead of ending the run."""
    import torch
    out = {}
    t_all = time.perf_counter()

    def guard(name, fn):
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as e:  # recorded in the line, the headline stands
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = time.perf_counter() - t0
        torch.cuda.empty_cache()
    guard("exact_c1", lambda: exact_c1(5, 3))
    guard("cloud_c3", lambda: cloud_c3(3, 2))
    guard("precision_c4", lambda: precision_c4(2000))
    meshes = []

    def gen():
        meshes.extend(served_meshes(256))
        return {"meshes": len(meshes)}
    guard("served_meshes", gen)
    if meshes:
        guard("served_c5", lambda: served_c5(meshes, args.extras_served_seconds, 120 << 30,
                                              nsat=500, nsat_fp64=150))
        guard("served_c5_pressure",
              lambda: served_c5(meshes, args.extras_served_seconds,
                                int(args.pressure_budget_gb * 2**30), nsat=200,
                                nsat_fp64=50, cpu=False, seed=8))
    out["extras_wall_s"] = time.perf_counter() - t_all
    return out


if __name__ == "__main__":
    main()
