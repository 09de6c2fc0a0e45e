"""Benchmark: complex64 ijkl,klmn->ijmn with all extents 64 (M = N = K = 4096).

Default arm: one step = one t1m_contract over device-resident operands with
the tensor-core split-precision method (3xTF32) when available; the plain FP32
GPU form is timed beside it.  ``value`` is whole-job complex TFLOP/s
(8*M*N*K per step), ``e2e`` the same metric through the public API with pinned
HOST buffers (host->device copy of A and B and device->host copy of C inside
every timed step).

``--impl reference`` times the reference's own algorithm on the host cores (the
oracle's C++ restatement of it, bit-identical to the reference built against
the same BLIS stand-in) on a bounded column slab of the same workload.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
(N > 1 under torchrun: independent replicas, one per GPU, weak scaling.)
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

EXT = 64
LA, LB, LC = "ijkl", "klmn", "ijmn"
M = N = K = EXT * EXT
FLOPS = 8.0 * M * N * K
WORKLOAD = "complex64 ijkl,klmn->ijmn, all extents 64 (M=N=K=4096), col-major"


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        d["_source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "sm_max_mhz": 2070.0, "_source": "fallback"}


def _profiled_traffic():
    """DRAM bytes (read + write) per launch of the tensor-core kernel on this
    workload, from the committed ncu summary (None if absent)."""
    p = ROOT / "profiles" / "tc3xtf32_ijkl_klmn_64.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch"):
            return int(line.split("=")[1])
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(
            ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
             "--format=csv,noheader,nounits", "-lms", "100"],
            stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        time.sleep(0.3)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait(timeout=5)
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append({"sm": float(parts[1]), "max": float(parts[2]),
                             "power": float(parts[3]), "hw": parts[5], "hwt": parts[6],
                             "swt": parts[7], "cap": parts[8]})
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [r for r in rows if r["power"] > 300.0] or rows
        reasons = set()
        for r in load:
            for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                              ("swt", "sw_thermal_slowdown"), ("cap", "sw_power_cap")):
                if r[key].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in load),
                "sm_max_mhz": max(r["max"] for r in rows), "reasons": sorted(reasons),
                "samples_under_load": len(load), "samples": len(rows)}


# ----------------------------------------------------------- reference arm ---
def _port_slab_run(fa, fb, fc, n_cols: int, nthreads: int) -> float:
    """Time the reference algorithm (oracle port) on C columns [0, n_cols)."""
    from oracle import libs
    from oracle import numpy_oracle as no
    dims = [EXT] * 4
    # klmn col-major: (m, n) -> columns m + 64 n; a slab of whole n values.
    n_ext = n_cols // EXT
    db = [EXT, EXT, EXT, n_ext]
    dc = [EXT, EXT, EXT, n_ext]
    t0 = time.perf_counter()
    libs.port_contract(fa, dims, no.col_major_strides(dims), LA, fb, db, no.col_major_strides(db),
                       LB, fc, dc, no.col_major_strides(dc), LC, nthreads=nthreads)
    return time.perf_counter() - t0


def _cpu_inputs(n_cols: int, seed: int = 1):
    rng = np.random.default_rng(seed)
    fa = (rng.uniform(-1, 1, M * K) + 1j * rng.uniform(-1, 1, M * K)).astype(np.complex64)
    fb = (rng.uniform(-1, 1, K * n_cols) + 1j * rng.uniform(-1, 1, K * n_cols)).astype(np.complex64)
    fc = np.zeros(M * n_cols, np.complex64)
    return fa, fb, fc


def cpu_baseline(target_s: float = 12.0, nthreads: int = 1) -> dict:
    """Reference algorithm on the host: 1 thread (the reference is single-
    threaded by construction), bounded column slab sized to ~target_s."""
    from oracle import build as obuild
    obuild.build_port()
    width = 64
    fa, fb, fc = _cpu_inputs(width)
    t = _port_slab_run(fa, fb, fc, width, nthreads)
    # Grow the slab to about target_s of work.
    want = int(min(N, max(64, width * target_s / max(t, 1e-3))))
    want = max(64, (want // 64) * 64)
    if want > width:
        fa, fb, fc = _cpu_inputs(want)
        t = _port_slab_run(fa, fb, fc, want, nthreads)
        width = want
    flops = 8.0 * M * width * K
    return {"value": flops / t / 1e12, "unit": "TFLOP/s", "cores": nthreads, "kind": "port",
            "sample": f"C columns [0,{width}) of {N} (mn slab of the same contraction), "
                      f"{flops:.3e} flop in {t:.2f} s; host nproc={os.cpu_count()}"}


def run_reference(args) -> None:
    world, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import build as obuild
    obuild.build_port()
    nthreads = os.cpu_count() or 1
    # Size each step to a few seconds of all-core work.
    width = 64 * nthreads
    fa, fb, fc = _cpu_inputs(width)
    t = _port_slab_run(fa, fb, fc, width, nthreads)
    budget = 150.0 / max(1, args.steps + args.warmup)
    width = int(min(N, max(64 * nthreads, width * min(budget, 8.0) / max(t, 1e-3))))
    width = max(64, (width // 64) * 64)
    fa, fb, fc = _cpu_inputs(width)
    for _ in range(args.warmup):
        fc[:] = 0
        _port_slab_run(fa, fb, fc, width, nthreads)
    times = []
    for _ in range(args.steps):
        fc[:] = 0
        times.append(_port_slab_run(fa, fb, fc, width, nthreads))
    flops = 8.0 * M * width * K
    total = sum(times)
    value = flops * len(times) / total / 1e12
    line = {
        "impl": "reference", "metric": "complex TFLOP/s (8MNK/t)", "value": value,
        "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "complex64", "data": "synthetic (U[-1,1] re/im, seed 1)",
        "config": {"workload": WORKLOAD, "sample_columns": width},
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": nthreads, "kind": "port",
                         "sample": f"C columns [0,{width}) of {N} per step, "
                                   f"{nthreads} threads on disjoint column slabs"},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU arm ---
def _sampled_error(torch, ga, gb, gc, samples=2048, seed=5):
    """Normwise (max, Frobenius) relative error of sampled C entries against
    FP64 dot products (col-major 4096x4096 matricisation of this workload)."""
    rng = np.random.default_rng(seed)
    rows = torch.from_numpy(rng.integers(0, M, samples)).to(ga.device)
    cols = torch.from_numpy(rng.integers(0, N, samples)).to(ga.device)
    Am = ga.view(K, M).t()            # A[m, k] = a[m + M k]
    Bm = gb.view(N, K).t()            # B[k, n] = b[k + K n]
    Cm = gc.view(N, M).t()
    ref = (Am[rows].to(torch.complex128) * Bm[:, cols].t().to(torch.complex128)).sum(1)
    got = Cm[rows, cols].to(torch.complex128)
    d = (got - ref).abs()
    return (float(d.max() / ref.abs().max()),
            float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref)))


def run_gpu(args) -> None:
    import torch
    import torch.distributed as dist

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import t1m_gb300 as t1m

    ctx = t1m.Context(local)
    dev = torch.device("cuda", local)
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    ga = torch.complex(torch.rand(M * K, device=dev, generator=g) * 2 - 1,
                       torch.rand(M * K, device=dev, generator=g) * 2 - 1)
    gb = torch.complex(torch.rand(K * N, device=dev, generator=g) * 2 - 1,
                       torch.rand(K * N, device=dev, generator=g) * 2 - 1)
    gc = torch.zeros(M * N, dtype=torch.complex64, device=dev)
    dims = [EXT] * 4
    ta, tb, tc = t1m.tensor(dims, ga), t1m.tensor(dims, gb), t1m.tensor(dims, gc)

    def one(method_name):
        ctx.set_method(method_name)
        return t1m.contract_scaled(1.0, ta, LA, tb, LB, 0.0, tc, LC, ctx=ctx)

    # Method of the tensor-core arm: 3xTF32 if this build has it.
    tc_method = args.method
    if tc_method == "auto":
        try:
            one("tc_3xtf32")
            tc_method = "tc_3xtf32"
        except t1m.T1MError:
            tc_method = "plain"
    torch.cuda.synchronize()
    err_tc = _sampled_error(torch, ga, gb, gc)

    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    sampler = ClockSampler(local)
    sampler.start()

    def timed(method_name, steps, warmup):
        ctx.set_method(method_name)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                t1m.contract_scaled(1.0, ta, LA, tb, LB, 0.0, tc, LC, ctx=ctx)
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            stream.synchronize()
            if world > 1:
                dist.barrier()
            start.record(stream)
            kernels = 0
            for _ in range(steps):
                rep = t1m.contract_raw(1.0, ta, LA, tb, LB, 0.0, tc, LC,
                                       t1m.FLAG_NO_TIMING, ctx)
                kernels += rep.kernels
            end.record(stream)
            end.synchronize()
        ms = start.elapsed_time(end)
        return ms, kernels

    ms_tc, launches = timed(tc_method, args.steps, args.warmup)
    clocks = sampler.stop()
    # The plain FP32 form, same workload (fewer steps: it is slower).
    plain_steps = max(1, min(args.steps, 5))
    one("plain")
    torch.cuda.synchronize()
    err_plain = _sampled_error(torch, ga, gb, gc)
    ms_plain, _ = timed("plain", plain_steps, 1)
    # Per-launch kernel time of the dominant kernel, events around the launch
    # on the launching stream.
    ctx.set_method(tc_method)
    reps = [t1m.contract_raw(1.0, ta, LA, tb, LB, 0.0, tc, LC, 0, ctx) for _ in range(3)]
    kernel_ms = min(r.kernel_ms for r in reps)

    # e2e: pinned host buffers through the public API; H2D of A and B and D2H
    # of C inside each timed step.
    ha = torch.empty(M * K, dtype=torch.complex64, pin_memory=True)
    hb = torch.empty(K * N, dtype=torch.complex64, pin_memory=True)
    hc = torch.empty(M * N, dtype=torch.complex64, pin_memory=True)
    ha.copy_(ga)
    hb.copy_(gb)
    hta, htb, htc = t1m.tensor(dims, ha), t1m.tensor(dims, hb), t1m.tensor(dims, hc)
    ctx.set_method(tc_method)
    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(max(1, args.warmup)):
        t1m.contract_scaled(1.0, hta, LA, htb, LB, 0.0, htc, LC, ctx=ctx)
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    h2d = d2h = 0
    for _ in range(e2e_steps):
        rep = t1m.contract_raw(1.0, hta, LA, htb, LB, 0.0, htc, LC, t1m.FLAG_NO_TIMING, ctx)
        h2d, d2h = rep.h2d_bytes, rep.d2h_bytes
    e2e_s = (time.perf_counter() - t0) / e2e_steps

    # Max over ranks.
    vals = torch.tensor([ms_tc, ms_plain, e2e_s], dtype=torch.float64, device=dev)
    if world > 1:
        dist.all_reduce(vals, op=dist.ReduceOp.MAX)
    ms_tc, ms_plain, e2e_s = vals.tolist()
    if rank == 0:
        peaks = _peaks()
        step_ms = ms_tc / args.steps
        value = world * FLOPS / (step_ms * 1e-3) / 1e12
        plain_tflops = FLOPS / (ms_plain / plain_steps * 1e-3) / 1e12
        per_gpu = FLOPS / (step_ms * 1e-3) / 1e12
        kernel_tflops = FLOPS / (kernel_ms * 1e-3) / 1e12
        if tc_method == "tc_3xtf32":
            peak = peaks["bf16_tflops"] / 2.0 / 3.0
            peak_note = ("TF32 dense = measured bf16 burst / 2, divided by the 3 TF32 "
                         f"products per algorithmic flop ({peaks['_source']})")
        else:
            peak = 152 * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
            peak_note = "FP32 SIMT nominal 152 SM x 128 lanes x 2 x max SM clock"
        line = {
            "metric": "complex TFLOP/s (8MNK/t) tensor-core vs plain GPU form @ rel err <=1e-6 vs FP64",
            "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "complex64",
            "data": "synthetic (re/im U[-1,1], torch seed 1234+rank)",
            "config": {"workload": WORKLOAD, "method": tc_method,
                       "l2": "inputs larger than L2 (A, B, C 134 MB each)",
                       "parallelism": f"replicas x{world}"},
            "plain_fp32": {"value": plain_tflops, "unit": "TFLOP/s", "steps": plain_steps,
                           "rel_err_max": err_plain[0], "rel_err_fro": err_plain[1]},
            "speedup_vs_plain": per_gpu / plain_tflops,
            "rel_err": {"max": err_tc[0], "fro": err_tc[1],
                        "oracle": "2048 sampled entries, FP64 dot products"},
            "roofline": {"bound": "tensor" if tc_method != "plain" else "fp32-simt",
                         "achieved": kernel_tflops, "peak": peak, "unit": "TFLOP/s",
                         "frac": kernel_tflops / peak,
                         "traffic": _profiled_traffic() if tc_method == "tc_3xtf32" else None,
                         "traffic_source": "profiles/tc3xtf32_ijkl_klmn_64.md (ncu dram bytes "
                                           "read+write per launch)",
                         "peak_note": peak_note},
            "e2e": {"value": world * FLOPS / e2e_s / 1e12, "unit": "TFLOP/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if world == 1 and not args.no_cpu_baseline:
            try:
                line["cpu_baseline"] = cpu_baseline()
            except Exception as e:  # reported, not fatal
                line["cpu_baseline"] = {"value": None, "error": str(e)}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--method", default="auto")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
