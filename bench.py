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
# One metric string for both arms, so their lines compare directly.
METRIC = "complex TFLOP/s (8MNK/t) tensor-core vs plain GPU form @ rel err <=1e-6 vs FP64"


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


# ncu summaries of the dominant kernel per method (the automatic tile form of
# this workload: CTA pairs over operand pieces for BF16x6, CTA pairs with
# in-kernel splitting for 3xTF32).
PROFILE_OF = {"tc_3xtf32": "tc1m_contract_pair_3xtf32_ijkl_klmn_64.md",
              "tc_bf16x6": "tc1m_pieces_bf16x6_ijkl_klmn_64.md"}


def _profiled_traffic(method):
    """DRAM bytes (read + write) per launch of the tensor-core kernel of
    `method` on this workload, from the committed ncu summary (None if absent)."""
    name = PROFILE_OF.get(method)
    p = ROOT / "profiles" / name if name else None
    if p is None or not p.exists():
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
        "impl": "reference", "metric": METRIC, "value": value,
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
    ctx.set_tile_form(args.tile_form)
    ctx.set_autotune(args.autotune)
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

    # Method of the tensor-core arm: the library's automatic choice (BF16x6
    # or 3xTF32 for this layout), reported by the method that ran.
    tc_method = args.method
    rep0 = one(tc_method)
    ran = t1m.method(rep0.method).name
    if tc_method == "auto":
        tc_method = ran
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
    # The other tensor-core split forms on the same workload.
    other = {}
    if tc_method != "plain":
        for m in ("tc_3xtf32", "tc_bf16x3", "tc_bf16x6"):
            if m == tc_method:
                continue
            one(m)
            torch.cuda.synchronize()
            e = _sampled_error(torch, ga, gb, gc)
            ms_m, _ = timed(m, max(1, min(args.steps, 10)), 1)
            other[m] = {"value": FLOPS / (ms_m / max(1, min(args.steps, 10)) * 1e-3) / 1e12,
                        "unit": "TFLOP/s", "rel_err_max": e[0], "rel_err_fro": e[1],
                        "meets_1e-6": e[0] <= 1e-6}
    # Per-launch kernel time of the dominant kernel, events around the launch
    # on the launching stream.
    ctx.set_method(tc_method)
    reps = [t1m.contract_raw(1.0, ta, LA, tb, LB, 0.0, tc, LC, 0, ctx) for _ in range(3)]
    kernel_ms = min(r.main_ms if r.main_ms > 0 else r.kernel_ms for r in reps)
    product_ms = min(r.kernel_ms for r in reps)

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
    # The same with pageable host buffers (what a C++ caller holding
    # std::vector data passes): the copies go through the driver's staging
    # and overlap the kernels less.
    pa, pb = ha.numpy().copy(), hb.numpy().copy()
    pc = np.empty(M * N, dtype=np.complex64)
    pta, ptb, ptc = t1m.tensor(dims, pa), t1m.tensor(dims, pb), t1m.tensor(dims, pc)
    t1m.contract_raw(1.0, pta, LA, ptb, LB, 0.0, ptc, LC, t1m.FLAG_NO_TIMING, ctx)
    page_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(page_steps):
        t1m.contract_raw(1.0, pta, LA, ptb, LB, 0.0, ptc, LC, t1m.FLAG_NO_TIMING, ctx)
    e2e_page_s = (time.perf_counter() - t0) / page_steps

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
        # FP32 SIMT nominal: 152 SMs x 128 FMA lanes x 2 flop x max SM clock
        # (no measured FP32 peak exists).
        fp32_nominal = 152 * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
        per_gpu = FLOPS / (step_ms * 1e-3) / 1e12
        kernel_tflops = FLOPS / (kernel_ms * 1e-3) / 1e12
        if tc_method == "tc_3xtf32":
            peak = peaks["bf16_tflops"] / 2.0 / 3.0
            peak_note = ("TF32 dense = measured bf16 burst / 2, divided by the 3 TF32 "
                         f"products per algorithmic flop ({peaks['_source']})")
        elif tc_method in ("tc_bf16x6", "tc_bf16x3"):
            nprod = 6.0 if tc_method == "tc_bf16x6" else 3.0
            peak = peaks["bf16_tflops"] / nprod
            peak_note = (f"measured bf16 burst divided by the {int(nprod)} bf16 products per "
                         f"algorithmic flop ({peaks['_source']})")
        else:
            peak = 152 * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
            peak_note = "FP32 SIMT nominal 152 SM x 128 lanes x 2 x max SM clock"
        line = {
            "metric": METRIC,
            "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "complex64",
            "data": "synthetic (re/im U[-1,1], torch seed 1234+rank)",
            "config": {"workload": WORKLOAD, "method": tc_method, "tile_form": args.tile_form,
                       "autotune": bool(args.autotune), "split_k": rep0.split_k,
                       "tile_path": rep0.fetch,
                       "l2": "inputs larger than L2 (A, B, C 134 MB each)",
                       "parallelism": f"replicas x{world}"},
            "plain_fp32": {"value": plain_tflops, "unit": "TFLOP/s", "steps": plain_steps,
                           "rel_err_max": err_plain[0], "rel_err_fro": err_plain[1],
                           "frac_of_fp32_simt_nominal": plain_tflops / fp32_nominal,
                           "fp32_simt_nominal_tflops": fp32_nominal},
            "speedup_vs_plain": per_gpu / plain_tflops,
            "other_tc_methods": other,
            "rel_err": {"max": err_tc[0], "fro": err_tc[1],
                        "oracle": "2048 sampled entries, FP64 dot products"},
            "roofline": {"bound": "tensor" if tc_method != "plain" else "fp32-simt",
                         "achieved": kernel_tflops, "peak": peak, "unit": "TFLOP/s",
                         "frac": kernel_tflops / peak,
                         "kernel": "main kernel alone (CUDA events around its launch)",
                         "product_tflops": FLOPS / (product_ms * 1e-3) / 1e12,
                         "product_note": "whole product: operand split pass + main kernel",
                         "traffic": _profiled_traffic(tc_method),
                         "traffic_source": f"profiles/{PROFILE_OF.get(tc_method)} (ncu dram bytes "
                                           "read+write per launch)",
                         "peak_note": peak_note},
            "e2e": {"value": world * FLOPS / e2e_s / 1e12, "unit": "TFLOP/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "host_buffers": "pinned",
                    "pageable": {"value": FLOPS / e2e_page_s / 1e12, "unit": "TFLOP/s",
                                 "steps": page_steps, "rank": rank}},
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


# --------------------------------------------------------- other workloads ---
def _events_ms(torch, fn, steps, warmup):
    """Mean ms of fn() over `steps`, CUDA events on torch's current stream
    (callers run their context on that stream)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(steps):
        fn()
    e.record()
    e.synchronize()
    return s.elapsed_time(e) / steps


def _sampled_err(la, lb, lc, dims, ga, gb, gc, alpha=1.0, beta=0.0, gc0=None, samples=1024):
    """Normwise errors at sampled C entries vs FP64 dot products (host numpy)."""
    import numpy as np
    da, db, dc = dims
    cm = lambda d: [int(np.prod(d[:i])) for i in range(len(d))]  # noqa: E731 col-major
    bd = _bundles(la, lb, lc)
    scat = [_scatter(bd[k], d, cm(d)) for k, d in (("AX", da), ("AY", da), ("BX", db),
                                                   ("BY", db), ("CX", dc), ("CY", dc))]
    fa, fb, fc = ga.cpu().numpy(), gb.cpu().numpy(), gc.cpu().numpy()
    rng = np.random.default_rng(3)
    rows = rng.integers(0, len(scat[0]), samples)
    cols = rng.integers(0, len(scat[3]), samples)
    ab = np.einsum("sk,sk->s", fa[scat[0][rows][:, None] + scat[1][None, :]].astype(np.complex128),
                   fb[scat[2][None, :] + scat[3][cols][:, None]].astype(np.complex128))
    off = scat[4][rows] + scat[5][cols]
    ref = alpha * ab
    if gc0 is not None and beta != 0:
        ref = ref + beta * gc0.cpu().numpy()[off].astype(np.complex128)
    d = np.abs(fc[off].astype(np.complex128) - ref)
    return float(d.max() / np.abs(ref).max()), float(np.linalg.norm(d) / np.linalg.norm(ref))


def _bundles(la, lb, lc):
    sa, sb = set(la), set(lb)
    con, fa, fb = sorted(sa & sb), sorted(sa - sb), sorted(sb - sa)
    return {"AX": [la.find(c) for c in fa], "AY": [la.find(c) for c in con],
            "BX": [lb.find(c) for c in con], "BY": [lb.find(c) for c in fb],
            "CX": [lc.find(c) for c in fa], "CY": [lc.find(c) for c in fb]}


def _scatter(idx, dims, strides):
    import numpy as np
    out = np.zeros(1, dtype=np.int64)
    for i in reversed(idx):
        out = (out[:, None] + np.arange(dims[i], dtype=np.int64)[None, :] * strides[i]).reshape(-1)
    return out


def workload_config2(args):
    """Plain GPU drop-in: abcd,efcd->abef (48^4) and abcd,dbea->ec, c64/c128,
    col/row-major, alpha = 1+0.5i, beta = 0.25, every method."""
    import torch
    import t1m_gb300 as t1m
    ctx = t1m.Context()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    dev = torch.device("cuda")
    cases = []
    shapes = [("abcd", "efcd", "abef", dict(a=48, b=48, c=48, d=48, e=48, f=48)),
              ("abcd", "dbea", "ec", dict(a=24, b=32, c=96, d=48, e=64))]
    for la, lb, lc, ext in shapes:
        dims = [[ext[ch] for ch in s] for s in (la, lb, lc)]
        for dt in (torch.complex64, torch.complex128):
            g = torch.Generator(device=dev)
            g.manual_seed(7)
            rdt = torch.float32 if dt == torch.complex64 else torch.float64
            mk = lambda n: torch.complex(torch.rand(n, device=dev, generator=g, dtype=rdt) * 2 - 1,  # noqa: E731
                                         torch.rand(n, device=dev, generator=g, dtype=rdt) * 2 - 1)
            ga, gb = mk(int(np.prod(dims[0]))), mk(int(np.prod(dims[1])))
            gc0 = mk(int(np.prod(dims[2])))
            methods = ["plain", "tc_3xtf32"] if dt == torch.complex64 else ["plain", "dmma"]
            for layout in ("col", "row"):
                L = t1m.col_major if layout == "col" else t1m.row_major
                for m in methods:
                    ctx.set_method(m)
                    gc = gc0.clone()
                    ta, tb, tc = (t1m.tensor(d, x, L) for d, x in zip(dims, (ga, gb, gc)))
                    rep = t1m.contract_raw(1 + 0.5j, ta, la, tb, lb, 0.25, tc, lc, 0, ctx)
                    if layout == "col":
                        err = _sampled_err(la, lb, lc, dims, ga, gb, gc, 1 + 0.5j, 0.25, gc0)
                    else:
                        err = (None, None)
                    ms = _events_ms(torch, lambda: t1m.contract_raw(
                        1 + 0.5j, ta, la, tb, lb, 0.25, tc, lc, t1m.FLAG_NO_TIMING, ctx),
                        args.steps, args.warmup)
                    cases.append({"labels": f"{la},{lb}->{lc}", "dtype": str(dt).split(".")[1],
                                  "layout": layout, "method": m, "split_k": rep.split_k,
                                  "ms": ms, "tflops": rep.flops / ms / 1e9,
                                  "rel_err_max": err[0], "rel_err_fro": err[1]})
    ctx.close()
    print(json.dumps({"workload": "config2 plain GPU drop-in", "cases": cases}), flush=True)


def workload_logmag(args):
    """Precision form, input set 2: |z| log-uniform over [1e-3, 1e3], uniform
    phase, complex64 ijkl,klmn->ijmn extents 64; every method's error."""
    import torch
    import t1m_gb300 as t1m
    ctx = t1m.Context()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    dev = torch.device("cuda")
    g = torch.Generator(device=dev)
    g.manual_seed(11)

    def mk(n):
        mag = torch.pow(10.0, torch.rand(n, device=dev, generator=g) * 6 - 3)
        ph = torch.rand(n, device=dev, generator=g) * 2 * np.pi
        return torch.polar(mag, ph)

    ga, gb = mk(M * K), mk(K * N)
    gc = torch.zeros(M * N, dtype=torch.complex64, device=dev)
    dims = [[EXT] * 4] * 3
    ta, tb, tc = (t1m.tensor(d, x) for d, x in zip(dims, (ga, gb, gc)))
    out = []
    for m in ("plain", "tc_3xtf32", "tc_bf16x3", "tc_bf16x6"):
        ctx.set_method(m)
        rep = min((t1m.contract_raw(1.0, ta, LA, tb, LB, 0.0, tc, LC, 0, ctx) for _ in range(3)),
                  key=lambda r: r.kernel_ms)
        err = _sampled_err(LA, LB, LC, dims, ga, gb, gc)
        out.append({"method": m, "ms": rep.kernel_ms, "tflops": FLOPS / rep.kernel_ms / 1e9,
                    "rel_err_max": err[0], "rel_err_fro": err[1]})
    ctx.close()
    print(json.dumps({"workload": "config3 set 2 (log-uniform magnitudes)", "cases": out}),
          flush=True)


def workload_c128(args):
    """Precision form, complex128 companion: ijkl,klmn->ijmn extents 64
    (M = N = K = 4096) in FP64, on the FP64 tensor cores (DMMA) and on the
    plain FP64 kernel (the automatic choice), with sampled FP64 errors and
    the fraction of the nominal FP64 peak (no measured FP64 peak exists)."""
    import torch
    import t1m_gb300 as t1m
    ctx = t1m.Context()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    dev = torch.device("cuda")
    g = torch.Generator(device=dev)
    g.manual_seed(1234)
    mk = lambda n: torch.complex(  # noqa: E731
        torch.rand(n, device=dev, generator=g, dtype=torch.float64) * 2 - 1,
        torch.rand(n, device=dev, generator=g, dtype=torch.float64) * 2 - 1)
    ga, gb = mk(M * K), mk(K * N)
    gc = torch.zeros(M * N, dtype=torch.complex128, device=dev)
    dims = [[EXT] * 4] * 3
    ta, tb, tc = (t1m.tensor(d, x) for d, x in zip(dims, (ga, gb, gc)))
    # GB300's nominal dense FP64 rate (its FP64 units are a small fraction
    # of the FP32 ones; no measured FP64 peak exists).
    peak = 1.25
    out = []
    for m in ("dmma", "auto"):
        ctx.set_method(m)
        rep = t1m.contract_raw(1.0, ta, LA, tb, LB, 0.0, tc, LC, 0, ctx)
        err = _sampled_err(LA, LB, LC, dims, ga, gb, gc, samples=256)
        ms = _events_ms(torch, lambda: t1m.contract_raw(1.0, ta, LA, tb, LB, 0.0, tc, LC,
                                                        t1m.FLAG_NO_TIMING, ctx),
                        max(1, min(args.steps, 3)), 1)
        out.append({"method": m, "ran": t1m.method(rep.method).name, "split_k": rep.split_k,
                    "ms": ms, "tflops": FLOPS / ms / 1e9, "frac_of_fp64_nominal": FLOPS / ms / 1e9 / peak,
                    "rel_err_max": err[0], "rel_err_fro": err[1]})
    ctx.close()
    print(json.dumps({"workload": "config3 complex128 companion, ijkl,klmn->ijmn extents 64 "
                                  "(M=N=K=4096), col-major", "fp64_peak_nominal_tflops": peak,
                      "cases": out}), flush=True)


def workload_plain(args):
    """The plain FP32 form alone on the headline workload (complex64
    ijkl,klmn->ijmn, extents --extent, col-major): TFLOP/s and its fraction
    of the nominal FP32 SIMT peak (the command the plain kernel's profile is
    taken with)."""
    import torch
    import t1m_gb300 as t1m
    E = args.extent
    ctx = t1m.Context()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    n = E ** 4
    mk = lambda: torch.complex(torch.rand(n, device="cuda", generator=g) * 2 - 1,  # noqa: E731
                               torch.rand(n, device="cuda", generator=g) * 2 - 1)
    ga, gb = mk(), mk()
    gc = torch.zeros(n, dtype=torch.complex64, device="cuda")
    ta, tb, tc = (t1m.tensor([E] * 4, x) for x in (ga, gb, gc))
    ctx.set_method("plain")
    ms = _events_ms(torch, lambda: t1m.contract_raw(1.0, ta, LA, tb, LB, 0.0, tc, LC,
                                                   t1m.FLAG_NO_TIMING, ctx),
                    args.steps, args.warmup)
    flops = 8.0 * float(E ** 2) ** 3
    nominal = 152 * 128 * 2 * 2.07e9 / 1e12
    ctx.close()
    print(json.dumps({"workload": f"plain FP32 form, complex64 ijkl,klmn->ijmn extents {E}, col-major",
                      "ms": ms, "tflops": flops / ms / 1e9,
                      "frac_of_fp32_simt_nominal": flops / ms / 1e9 / nominal,
                      "fp32_simt_nominal_tflops": nominal}), flush=True)


def workload_batch(args):
    """Batching form: 1024 updates xay,asb->xsyb then xsyb,ytb->xst with
    x, y, a, b ~ U{16..256 step 16}, s, t ~ U{2, 4}, components N(0, 1/sqrt(bond));
    one grouped batch under a CUDA graph vs the same contractions one call at a time."""
    import torch
    import t1m_gb300 as t1m
    n_items = args.items
    ctx = t1m.Context()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    dev = torch.device("cuda")
    rng = np.random.default_rng(2024)
    bonds = np.arange(16, 257, 16)
    items, flops, keep = [], 0.0, []
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    for _ in range(n_items):
        x, y, a, b = (int(w) for w in rng.choice(bonds, 4))
        s, t = (int(w) for w in rng.choice([2, 4], 2))

        def mk(shape, bond):
            sc = 1.0 / np.sqrt(np.sqrt(bond))
            return torch.complex(torch.randn(shape, device=dev, generator=g) * sc,
                                 torch.randn(shape, device=dev, generator=g) * sc)

        X1, X2, X3 = mk((x, a, y), a), mk((a, s, b), a), mk((y, t, b), b)
        R = torch.empty((x, s, y, b), dtype=torch.complex64, device=dev)
        O = torch.empty((x, s, t), dtype=torch.complex64, device=dev)
        i1 = len(items)
        items.append((1.0, v(X1), "xay", v(X2), "asb", 0.0, v(R), "xsyb", -1))
        items.append((1.0, v(R), "xsyb", v(X3), "ytb", 0.0, v(O), "xst", i1))
        keep.append((X1, X2, X3, R, O))
        flops += 8.0 * x * y * s * b * a + 8.0 * x * s * t * y * b
    grp = t1m.Group(items, ctx=ctx, graph=True, autotune=not args.no_autotune)
    grouped_ms = _events_ms(torch, lambda: grp.launch(timed=False), args.steps, args.warmup)
    grouped_kernels = grp.launch().kernels
    # The same batch as ONE persistent launch (SIMT tiles for the second
    # steps, split-K reduced in the kernel), for comparison.
    one = t1m.Group(items, ctx=ctx, graph=True, autotune=not args.no_autotune,
                    options=t1m.GROUP_ONE_LAUNCH)
    one_ms = _events_ms(torch, lambda: one.launch(timed=False), args.steps, args.warmup)
    one_kernels = one.launch().kernels
    one.close()
    grp.launch(timed=False)  # outputs of the one-launch form for the check below
    torch.cuda.synchronize()
    # Sampled check of a few items against FP64.
    errs = []
    for X1, X2, X3, R, O in keep[:4]:
        Rr = torch.einsum("xay,asb->xsyb", X1.to(torch.complex128), X2.to(torch.complex128))
        Or = torch.einsum("xsyb,ytb->xst", Rr, X3.to(torch.complex128))
        errs.append(float((O.to(torch.complex128) - Or).abs().max() / Or.abs().max()))

    def one_by_one():
        for (alpha, a_, la, b_, lb, beta, c_, lc, _d) in items:
            t1m.contract_raw(alpha, a_, la, b_, lb, beta, c_, lc, t1m.FLAG_NO_TIMING, ctx)

    single_ms = _events_ms(torch, one_by_one, max(1, args.steps // 2), 1)
    grp.close()
    ctx.close()
    print(json.dumps({"workload": f"config4 batch of {n_items} sweep updates (2 contractions each)",
                      "flops_per_batch": flops, "grouped_graph_ms": grouped_ms,
                      "grouped_tflops": flops / grouped_ms / 1e9,
                      "grouped_kernels": grouped_kernels,
                      "one_launch_graph_ms": one_ms, "one_launch_kernels": one_kernels,
                      "one_launch_tflops": flops / one_ms / 1e9,
                      "one_call_at_a_time_ms": single_ms,
                      "one_call_tflops": flops / single_ms / 1e9,
                      "speedup_grouped": single_ms / grouped_ms, "rel_err_max_sampled": max(errs)}),
          flush=True)


def workload_vjp(args):
    """Differentiation form: abcd,ebfd->aecf extents 32 (complex64, tensor
    cores), forward + adjoint (dA, dB) vs FP64, and the ring chain."""
    import torch
    import t1m_gb300 as t1m
    from t1m_gb300.chain import ContractionChain
    ctx = t1m.Context()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    dev = torch.device("cuda")
    g = torch.Generator(device=dev)
    g.manual_seed(9)
    mk = lambda *s: torch.complex(torch.rand(s, device=dev, generator=g) * 2 - 1,  # noqa: E731
                                  torch.rand(s, device=dev, generator=g) * 2 - 1)
    A, B, dC = mk(32, 32, 32, 32), mk(32, 32, 32, 32), mk(32, 32, 32, 32)
    C = torch.empty_like(dC)
    dA, dB = torch.empty_like(A), torch.empty_like(B)
    v = lambda z: t1m.tensor(list(z.shape), z, t1m.row_major)  # noqa: E731
    ctx.set_method("tc_3xtf32")
    fwd_ms = _events_ms(torch, lambda: t1m.contract_raw(1.0, v(A), "abcd", v(B), "ebfd", 0.0,
                                                        v(C), "aecf", t1m.FLAG_NO_TIMING, ctx),
                        args.steps, args.warmup)
    vjp_ms = _events_ms(torch, lambda: t1m.contract_vjp(v(dC), "aecf", v(A), "abcd", v(B),
                                                        "ebfd", v(dA), v(dB), ctx=ctx,
                                                        timed=False),
                        args.steps, args.warmup)
    vrep = t1m.contract_vjp(v(dC), "aecf", v(A), "abcd", v(B), "ebfd", v(dA), v(dB), ctx=ctx)
    A64, B64, G64 = (z.to(torch.complex128) for z in (A, B, dC))
    rA = torch.einsum("aecf,ebfd->abcd", G64, B64.conj())
    rB = torch.einsum("abcd,aecf->ebfd", A64.conj(), G64)
    eA = float((dA.to(torch.complex128) - rA).abs().max() / rA.abs().max())
    eB = float((dB.to(torch.complex128) - rB).abs().max() / rB.abs().max())
    flops = 8.0 * 32 ** 6
    # Ring chain: four order-3 tensors, bond 64, physical 8, to a scalar.
    ext = dict(a=64, b=64, c=64, d=64, p=8, q=8)
    labels, outs = ["apb", "bpc", "cqd", "dqa"], ["ac", "aqd", ""]
    xs = [mk(*[ext[c] for c in lab]) / 8.0 for lab in labels]
    chain = ContractionChain(labels, outs)
    one = torch.ones((), dtype=torch.complex64, device=dev)
    chain_ms = _events_ms(torch, lambda: chain.backward(xs, one, ctx=ctx), 5, 2)
    # The same chain as one grouped launch per pass (forward + adjoint).
    gchain = ContractionChain(labels, outs, mode="grouped")
    gchain_ms = _events_ms(torch, lambda: gchain.backward(xs, one, ctx=ctx), 5, 2)
    gchain.close()
    ctx.close()
    print(json.dumps({"workload": "config5 abcd,ebfd->aecf extents 32 + VJP; ring chain",
                      "forward_ms": fwd_ms, "forward_tflops": flops / fwd_ms / 1e9,
                      "vjp_ms": vjp_ms, "vjp_tflops": 2 * flops / vjp_ms / 1e9,
                      "vjp_kernel_ms_reported": vrep.kernel_ms, "vjp_kernels": vrep.kernels,
                      "rel_err_dA": eA, "rel_err_dB": eB,
                      "ring_chain_backward_ms": chain_ms,
                      "ring_chain_backward_grouped_ms": gchain_ms}), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--method", default="auto")
    ap.add_argument("--tile-form", default="auto", choices=["auto", "one", "pair", "pieces"],
                    help="tensor-core tile form (one tile per CTA, CTA pairs, or CTA pairs "
                         "over operands split into bf16 pieces beforehand)")
    ap.add_argument("--autotune", action="store_true",
                    help="tune tile form and split count per shape class (first call)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="headline",
                    choices=["headline", "config2", "logmag", "c128", "batch", "vjp", "plain"])
    ap.add_argument("--items", type=int, default=1024)
    ap.add_argument("--extent", type=int, default=64,
                    help="plain workload: every extent of ijkl,klmn->ijmn")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batch workload: heuristic kernel families instead of the autotuner")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "headline":
        # The workloads run their contexts on torch's current stream and time
        # with torch events; a created stream (not the legacy stream 0, which
        # t1m_set_stream reads as "the context's own") keeps both on one.
        import torch
        fn = {"config2": workload_config2, "logmag": workload_logmag, "c128": workload_c128,
              "batch": workload_batch, "vjp": workload_vjp, "plain": workload_plain}[args.workload]
        with torch.cuda.stream(torch.cuda.Stream()):
            fn(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
