"""Benchmark: triangle-soup fast winding number (igl::fast_winding_number soup
overloads), the configuration the headline metric is quoted on:

  mesh    icosphere subdivided 8 times (1,310,720 triangles), radial
          spherical-harmonic displacement (degree <= 8, N(0, 0.05/l)), 1% of
          the triangles deleted at random (1,297,489 left);
  queries 10M: 90% uniform in the 1.2x bounding box, 10% along random face
          normals at 10^U(-4,-1); float64 (float32 with --qdtype f32);
  order 2, accuracy_scale (beta) 2.

A step is one evaluation of all queries on the device (mixed precision:
FP32 bulk, FP64 near-field / decision guard band / threshold re-evaluation).
Reported: value = queries/s of the device-resident call; e2e = the same call
through the C ABI with host (pinned) buffers, copies included; accuracy of
the mixed result against the plain FP64 walk of the same tree; the plain FP64
walk's own throughput; the dominant kernel's live CUDA-event duration and
roofline; a CPU baseline on this host's cores.

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


def make_workload(args, rank):
    from libigl_gb300 import synth
    V, F = synth.soup_mesh(seed=1, subdiv=args.subdiv)
    Q = synth.soup_queries(V, F, seed=2 + rank, nq=args.nq)
    if args.qdtype == "f32":
        Q = Q.astype(np.float32)
    return V, F, Q


def cpu_baseline(V, F, Q, seconds: float, mesh_handle=None):
    """CPU soup FWN (oracle restatement of the reference algorithm) on this
    host's cores, on a bounded sample of the same queries."""
    from oracle import oracle as O
    nthreads = O.num_threads(0)
    t0 = time.perf_counter()
    port = O.SoupPort(V, F, order=2)
    build_s = time.perf_counter() - t0
    probe = Q[: min(len(Q), 200_000)]
    t0 = time.perf_counter()
    port.eval(probe, 2.0, nthreads)
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
            "precompute_s": build_s}


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
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "queries_per_step": n,
                                        "order": 2, "beta": 2.0, "qdtype": args.qdtype},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{n} queries per step of the {args.nq}-query workload"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
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
    bvh = G.FastWindingNumberBVH(V, F, order=2)
    torch.cuda.synchronize()
    build_s_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    bvh2 = G.FastWindingNumberBVH(V, F, order=2)
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

    # timed region: per-step CUDA events on the launch stream + live phase events
    G.profile_enable(True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    walk_ms = []
    evs[0].record(stream)
    for k in range(args.steps):
        step()
        evs[k + 1].record(stream)
        ph = G.profile_read()  # waits for this step's phase events
        walk_ms.append(ph.get("walk", float("nan")))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = sampler.stop()
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
                "kernel_ms": walk, "kernel_share_of_step": walk / ms_per_step}

    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu = cpu_baseline(V, F, Q, args.cpu_seconds)

    # kernels launched per step by the library (counted in the library's launch sites)
    launches_per_step = G.launch_count_of(lambda: step())
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step,
        "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "triangles": int(nt), "queries_per_gpu": int(nq),
                   "qdtype": args.qdtype, "order": 2, "beta": 2.0, "precision": "mixed",
                   "l2": "inputs larger than L2 (queries+results > 126 MB per step)",
                   "parallelism": f"query shards x{world}, tree replicated"},
        "accuracy": accuracy,
        "plain_fp64": {"value": plain_fp64_qps, "unit": UNIT, "ms_per_step": fp64_ms,
                       "mixed_speedup": value / world / plain_fp64_qps},
        "precompute_s": build_s, "precompute_first_call_s": build_s_first,
        "tree": stats,
        "roofline": roofline, "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu,
        "gpu_launches": int(launches_per_step * args.steps),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
