#!/usr/bin/env python
"""NTT benchmark on GB300 -- the headline line is a single Goldilocks NTT.

Default workload: one step = forward + inverse Goldilocks NTT of n = 2^24
elements (128 MiB), in place, inputs resident in HBM, L2 flushed between
steps (a 256 MiB write outside the timed events). Metric: Gelem/s =
2 * n / step time (both transforms count).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
    python bench.py --impl reference ...   # the reference's own code paths

Multi-GPU: replicas only (the transform does not shard); every rank runs the
same workload, value = all ranks' elements / max-over-ranks time.

JSON keys beyond the base contract:
  e2e           the same metric through the C ABI with host buffers: per step a
                pinned copy in, forward + inverse on the caller's stream, a copy
                out, all inside the timed region; steps go round 4 streams with
                their own buffers (copies of one step overlap another's), and
                `serial` times them one at a time
  roofline      the dominant kernel (the tile kernel): algorithmic bytes of a
                transform, B_alg = P_min * 2 * n * w (P_min = 1 when the
                transform fits one tile, else 2), over the transform time,
                against MEASURED_PEAKS.json hbm_gbs; `per_launch` keeps the
                bytes each launch moves (2 n w) over the mean launch time
  secondary     (default run, one GPU) the rest of the configurations, each
                timed the same way: Goldilocks 2^20, 32-bit 2^16 / 2^20 / 2^26,
                the uneven batched mix (persistent launch against one launch
                sequence per transform, compared bit for bit), and the serving
                loop (p50 / p99 latency and throughput on a shortened trace)
  cpu_baseline  the CPU path on a bounded sample, with the host CPU model
  clocks        nvidia-smi samples taken during the timed region

--impl reference runs the reference's own code: the 32-bit CPU transform is
the unmodified reference nttStockham (compiled from its sources into
oracle/_ref), Goldilocks the oracle's restatement of the same loop (the
reference has no Goldilocks CPU code), on all host threads; its line also
carries `reference_gpu`, the reference's own CUDA autoNtt<n> (rebuilt for
sm_100 from its sources) timed on this GPU at 32-bit 2^16, 2^20 and 2^26.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    # name: (field, log_n); "batch" = the uneven mix below, "serve" = the serving trace
    "gl64_batch_mix": ("gl64", "batch"),
    "serve_mix": ("mixed", "serve"),
    "gl64_2^24_fwd+inv": ("gl64", 24),
    "gl64_2^20_fwd+inv": ("gl64", 20),
    "u32_2^26_fwd+inv": ("u32", 26),
    "u32_2^20_fwd+inv": ("u32", 20),
    "u32_2^16_fwd+inv": ("u32", 16),
}
DEFAULT_WORKLOAD = "gl64_2^24_fwd+inv"
METRIC = "NTT Gelem/s (Goldilocks 2^24 forward+inverse, per element transformed)"
L2_BYTES = 129 * 1024 * 1024
E2E_SLOTS = 4  # streams (with their own buffers) the end-to-end steps go round (2: 31.4, 3: 38.3, 4: 39.6 Gelem/s)
# largest transform one tile (one HBM pass) holds: 2^12 eight-byte or 2^13 four-byte points
SINGLE_TILE_LOG = {"gl64": 12, "u32": 13}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the other configurations in the default run")
    ap.add_argument("--mix-jobs", type=int, default=4096, help="jobs in the batched mix (4096 for the headline)")
    ap.add_argument("--streams", type=int, default=32, help="serving: request slots")
    ap.add_argument("--serve-requests", type=int, default=0,
                    help="serving: requests in the trace (default: steps * 1000, at least 1000)")
    ap.add_argument("--serve-rate", type=float, default=20000.0, help="serving: mean arrival rate, requests/s")
    ap.add_argument("--tma", choices=["auto", "on", "off"], default="auto",
                    help="TMA-staged passes: built-in choice per pass, everywhere allowed, or never")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def ncu_traffic(workload: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    try:
        return json.loads((ROOT / "profiles" / "ncu_traffic.json").read_text())[workload]
    except (OSError, KeyError, ValueError):
        return None


def max_over_ranks(value: float, world: int, device=None) -> float:
    """The largest `value` over all ranks (timings: the slowest rank counts)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            d = json.loads(f.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def b_alg(field: str, lg: int) -> int:
    """Algorithmic HBM bytes of one transform: P_min * 2 * n * w."""
    w = 8 if field == "gl64" else 4
    pmin = 1 if lg <= SINGLE_TILE_LOG[field] else 2
    return pmin * 2 * (1 << lg) * w


class ClockSampler:
    """nvidia-smi samples (100 ms) while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
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
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_index(local: int) -> int:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0]
    return int(vis) if vis.isdigit() else local


# --------------------------------------------------------------------------- reference arm
def _ref_u32_transforms(R, x: np.ndarray, n: int, root: int, mod: int, threads: int) -> None:
    """The unmodified reference nttStockham (ntt_cpu.cpp:46-85) on `threads`
    independent transforms at once (one per Python thread; ctypes releases the
    GIL): the forward transform, then the same loop with root^-1 (the
    reference's inverse transform step; its n^-1 scaling is one O(n) pass)."""
    rinv = pow(root, mod - 2, mod)

    def one(t):
        seg = x[t * n:(t + 1) * n]
        R.ref_ntt_stockham(seg, n, root, mod, -1)
        R.ref_ntt_stockham(seg, n, rinv, mod, -1)

    ths = [threading.Thread(target=one, args=(t,)) for t in range(threads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()


def reference_gpu(reps: int = 3):
    """The reference's own CUDA NTT (cuda::ntt::autoNtt<n>, ntt_kernel.cuh:153-200),
    rebuilt for sm_100 from its unmodified sources (oracle/ref_gpu_bench.cu),
    timed on this GPU: kernel milliseconds from its own CUDA events, per block
    size of its sweep, for the 32-bit field at n = 2^16, 2^20, 2^26 (forward
    transforms; the reference has no GPU inverse and no working Goldilocks
    kernel)."""
    import oracle as O

    exe = O.ref_gpu_bench()
    if exe is None:
        return {"unavailable": "the reference CUDA benchmark was not built (no copy of the reference sources: "
                               "make -C oracle ref-stage REF=<checkout>)"}
    try:
        r = subprocess.run([str(exe), "16,20,26", str(reps)], capture_output=True, text=True, timeout=300)
    except subprocess.TimeoutExpired:
        return {"unavailable": "the reference CUDA benchmark did not finish within 300 s"}
    if r.returncode != 0:
        return {"unavailable": f"the reference CUDA benchmark failed (rc {r.returncode}): {r.stderr.strip()[-200:]}"}
    rows = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    out = {"api": "cuda::ntt::autoNtt<n>(NttArgs(vec, n, 1, root, mod, 2, block)), forward, batch 1, "
                  "findParams(n, 11); kernel time = its own CUDA events",
           "build": "nvcc -O3 -gencode arch=compute_100,code=sm_100 (unmodified reference headers)",
           "reps": reps, "sizes": {}}
    for lg in (16, 20, 26):
        mine = [x for x in rows if x["log_n"] == lg]
        if not mine:
            continue
        best = min(mine, key=lambda x: x["kernel_ms_mean"])
        at1024 = next((x for x in mine if x["block_size"] == 1024), best)
        out["sizes"][f"u32_2^{lg}"] = {
            "kernel_ms_best": best["kernel_ms_mean"], "best_block_size": best["block_size"],
            "kernel_ms_block1024": at1024["kernel_ms_mean"], "wall_ms_block1024": at1024["wall_ms_mean"],
            "gelem_per_s_best": (1 << lg) / (best["kernel_ms_mean"] / 1e3) / 1e9,
            "by_block_size": {str(x["block_size"]): x["kernel_ms_mean"] for x in mine},
        }
    return out


def run_reference(args):
    """The reference's CPU NTT on all host threads (each thread one
    independent transform), and its CUDA NTT on this GPU (reference_gpu)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle as O

    field, lg = WORKLOADS[args.workload]
    if lg in ("batch", "serve"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched or serving path; "
                          "its arm covers the single-transform workloads"}), flush=True)
        return
    n = 1 << lg
    threads = max(1, min(O.cpu_count(), 16))
    if field == "gl64":
        kind = "port"
        x = O.uniform_u64(7, n * threads)
        what = ("the oracle's restatement of the reference Stockham loop (src/ntt/ntt_cpu.cpp:46-85) with "
                "Goldilocks arithmetic: the reference has no Goldilocks CPU code")

        def step():
            y = O.ntt_gl64(x, batch=threads, threads=threads)
            O.ntt_gl64(y, inverse=True, batch=threads, threads=threads)
    else:
        root, p = O.find_params(n, 11)
        R = O.ref()
        if R is not None:
            kind = "reference"
            x0 = O.uniform_u32(7, p, n * threads).view(np.int32)
            what = ("the unmodified reference nttStockham (src/ntt/ntt_cpu.cpp:46-85, compiled from its sources), "
                    "forward then the same loop with root^-1")

            def step():
                _ref_u32_transforms(R, x0.copy(), n, root, p, threads)
        else:
            kind = "port"
            x = O.uniform_u32(7, p, n * threads)
            what = "the oracle's restatement of the reference Stockham loop (the reference build is absent)"

            def step():
                y = O.ntt_u32(x, root, p, batch=threads, threads=threads)
                O.ntt_u32(y, root, p, inverse=True, batch=threads, threads=threads)
    steps = max(1, min(args.steps, 3))
    warm = min(args.warmup, 1)
    for _ in range(warm):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = (time.perf_counter() - t0) / steps
    val = 2 * n * threads / dt / 1e9
    sample = (f"{threads} independent {field} 2^{lg} forward+inverse transforms per step, one per host thread, "
              f"{what}; {steps} timed steps after {warm} warm-up (steps capped so the CPU run stays within minutes)")
    line = {
        "impl": "reference", "metric": METRIC if args.workload == DEFAULT_WORKLOAD else f"NTT Gelem/s ({args.workload})",
        "value": val, "unit": "Gelem/s", "n_gpus": world, "steps": steps, "warmup": warm,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64" if field == "gl64" else "u32", "data": "synthetic (splitmix64 uniform residues)",
        "config": {"workload": args.workload, "n": n, "field": field, "host_threads": threads},
        "cpu_baseline": {"value": val, "unit": "Gelem/s", "cores": threads, "kind": kind, "sample": sample,
                         "cpu_model": cpu_model()},
        "e2e": {"value": val, "unit": "Gelem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    line["reference_gpu"] = reference_gpu() if has_gpu else {"unavailable": "no CUDA device"}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- CPU baseline of our arm
def cpu_baseline(field: str, lg: int):
    """One forward+inverse of the same size on one host core: the unmodified
    reference for the 32-bit field where it is built, else the oracle port."""
    import oracle as O

    n = 1 << lg
    kind = "port"
    if field == "gl64":
        x = O.uniform_u64(3, n)
        t0 = time.perf_counter()
        y = O.ntt_gl64(x)
        O.ntt_gl64(y, inverse=True)
        what = "oracle restatement of the reference Stockham loop (src/ntt/ntt_cpu.cpp:46-85), Goldilocks arithmetic"
    else:
        root, p = O.find_params(n, 11)
        x = O.uniform_u32(3, p, n)
        R = O.ref()
        t0 = time.perf_counter()
        if R is not None:
            _ref_u32_transforms(R, x.view(np.int32).copy(), n, root, p, 1)
            kind = "reference"
            what = "the unmodified reference nttStockham (src/ntt/ntt_cpu.cpp:46-85), forward then root^-1"
        else:
            y = O.ntt_u32(x, root, p)
            O.ntt_u32(y, root, p, inverse=True)
            what = "oracle restatement of the reference Stockham loop"
    dt = time.perf_counter() - t0
    return {"value": 2 * n / dt / 1e9, "unit": "Gelem/s", "cores": 1, "kind": kind, "cpu_model": cpu_model(),
            "sample": f"one {field} 2^{lg} forward+inverse on one host core ({dt:.1f} s), {what}"}


# --------------------------------------------------------------------------- single transforms
def measure_single(ctx, st, torch, field: str, lg: int, steps: int, warmup: int, dev, rank: int = 0,
                   check: bool = True):
    """Time `steps` forward+inverse steps of one transform of 2^lg points,
    inputs resident in HBM, L2 flushed between steps outside the events.
    Returns the per-direction event times and what a call launches."""
    n = 1 << lg
    stream = torch.cuda.Stream(device=dev)
    sp = stream.cuda_stream
    if field == "gl64":
        data = torch.empty(n, dtype=torch.int64, device=dev)
        st.fill_uniform_gl64(data, 1234 + rank, stream=sp)
        fwd = lambda: ctx.ntt_gl64(data, lg, 1, inverse=False, stream=sp)  # noqa: E731
        inv = lambda: ctx.ntt_gl64(data, lg, 1, inverse=True, stream=sp)  # noqa: E731
        fid, p, root = st.FIELD_GL64, 0, 0
    else:
        p, root = st.params_u32(lg)
        data = torch.empty(n, dtype=torch.int32, device=dev)
        st.fill_uniform_u32(data, 1234 + rank, p, stream=sp)
        fwd = lambda: ctx.ntt_u32(data, lg, 1, p, root, inverse=False, stream=sp)  # noqa: E731
        inv = lambda: ctx.ntt_u32(data, lg, 1, p, root, inverse=True, stream=sp)  # noqa: E731
        fid = st.FIELD_U32
    passes, pass_logs = ctx.call_info(fid, lg, 1, p, root)  # kernel launches one call of this shape makes
    stream.synchronize()
    ref_copy = data.clone() if check else None
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device=dev)
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            fwd()
            inv()
        stream.synchronize()
        ok = bool(torch.equal(data, ref_copy)) if check else None  # forward+inverse is the identity
        # Up to 2^22 elements a transform's kernels are shorter than one host
        # call (ctypes + the C ABI + the launch), so the events would time the
        # host. There each transform is captured once as a CUDA graph (same
        # calls, same kernels, same stream) and replayed.
        graph = lg <= 22
        if graph:
            g_f, g_i = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
            with torch.cuda.graph(g_f, stream=stream, capture_error_mode="relaxed"):
                fwd()
            with torch.cuda.graph(g_i, stream=stream, capture_error_mode="relaxed"):
                inv()
            run_fwd, run_inv = g_f.replay, g_i.replay
            for _ in range(3):
                run_fwd()
                run_inv()
            stream.synchronize()
            if check:
                ok = ok and bool(torch.equal(data, ref_copy))
        else:
            run_fwd, run_inv = fwd, inv
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize()
        for i in range(steps):
            flush.zero_()  # L2 flush, outside the events
            a, b, c = ev[i]
            a.record(stream)
            run_fwd()
            b.record(stream)
            run_inv()
            c.record(stream)
        torch.cuda.synchronize()
    t_fwd = [ev[i][0].elapsed_time(ev[i][1]) for i in range(steps)]
    t_inv = [ev[i][1].elapsed_time(ev[i][2]) for i in range(steps)]
    if check:
        ok = ok and bool(torch.equal(data, ref_copy))
    return {"t_fwd": t_fwd, "t_inv": t_inv, "step_ms": float(np.sum(t_fwd) + np.sum(t_inv)) / steps,
            "passes": passes, "pass_logs": pass_logs, "graph": graph, "ok": ok, "data": data, "ref": ref_copy,
            "fwd": fwd, "inv": inv, "stream": stream}


def roofline_of(field: str, lg: int, step_ms: float, t_fwd, t_inv, passes: int, workload: str | None = None):
    hbm, hbm_kind = peaks()
    n = 1 << lg
    w = 8 if field == "gl64" else 4
    ba = b_alg(field, lg)
    achieved = 2 * ba / (step_ms / 1e3) / 1e9  # two transforms per step
    launch_ms = (float(np.mean(t_fwd)) + float(np.mean(t_inv))) / 2 / passes
    per_launch = 2 * n * w
    r = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
         "peak_kind": hbm_kind, "b_alg_per_transform": ba, "p_min": ba // (2 * n * w),
         "one_pass_floor_bytes": 2 * n * w, "launches_per_transform": passes,
         "per_launch": {"bytes": per_launch, "mean_launch_us": launch_ms * 1e3,
                        "achieved": per_launch / (launch_ms / 1e3) / 1e9,
                        "frac": per_launch / (launch_ms / 1e3) / 1e9 / hbm}}
    if workload is not None:
        tr = ncu_traffic(workload)
        r["traffic"] = tr["bytes_per_launch"] if tr else None
        r["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, "
                               f"profiles/{tr['source']}" if tr else None)
    return r


def secondary_single(ctx, st, torch, field, lg, dev, steps=20, warmup=3):
    m = measure_single(ctx, st, torch, field, lg, steps, warmup, dev)
    n = 1 << lg
    r = roofline_of(field, lg, m["step_ms"], m["t_fwd"], m["t_inv"], m["passes"])
    out = {"value": 2 * n / (m["step_ms"] / 1e3) / 1e9, "unit": "Gelem/s", "ms_per_step": m["step_ms"],
           "fwd_ms": float(np.mean(m["t_fwd"])), "inv_ms": float(np.mean(m["t_inv"])), "steps": steps,
           "launches_per_transform": m["passes"], "pass_log_lengths": m["pass_logs"],
           "launch": "CUDA graph per transform, replayed" if m["graph"] else "direct C-ABI calls",
           "hbm_frac": r["frac"], "hbm_achieved_gbs": r["achieved"], "b_alg_per_transform": r["b_alg_per_transform"],
           "round_trip_ok": m["ok"]}
    del m
    return out


# --------------------------------------------------------------------------- batched mix
MIX_JOBS, MIX_LO, MIX_HI, MIX_SEED = 4096, 10, 18, 0x57170001 + 3


def mix_sizes(jobs: int = MIX_JOBS):
    """log2 n of each job: uniform in [10, 18] from a fixed seed; job i is
    forward for even i and inverse for odd i."""
    rng = np.random.default_rng(MIX_SEED)
    return [int(v) for v in rng.integers(MIX_LO, MIX_HI + 1, jobs)]


def measure_batch_mix(st, torch, dev, jobs_n: int, steps: int, warmup: int, rank: int = 0, world: int = 1):
    """The uneven batch: one persistent launch replayed from a CUDA graph,
    against one launch sequence per transform on the same inputs, compared
    bit for bit."""
    sizes = mix_sizes(jobs_n)
    total = sum(1 << s for s in sizes)
    data = torch.empty(total, dtype=torch.int64, device=dev)
    st.fill_uniform_gl64(data, 77 + rank)
    torch.cuda.synchronize()
    ref = data.clone()
    jobs, jobs_ref, off = [], [], 0
    for i, s in enumerate(sizes):
        jobs.append(st.Job(st.FIELD_GL64, s, i % 2, 0, 0, 0, data.data_ptr() + 8 * off))
        jobs_ref.append(st.Job(st.FIELD_GL64, s, i % 2, 0, 0, 0, ref.data_ptr() + 8 * off))
        off += 1 << s
    ctx = st.Context(dev.index)
    b = ctx.batch_create(jobs)
    info = b.info()
    stream = torch.cuda.Stream(device=dev)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        b.launch(stream=stream)
    # bit-exactness: one replay and one per-call sequence on the same inputs
    g.replay()
    ctx.ntt_batch(jobs_ref, per_call=True, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    bit_exact = bool(torch.equal(data, ref)) and b.status() == 0
    del ref
    for _ in range(warmup):
        g.replay()
    torch.cuda.synchronize()
    ok = b.status() == 0
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ok = ok and b.status() == 0
    ms = e0.elapsed_time(e1) / steps
    # one launch sequence per transform (the comparison), plain launches
    s2 = torch.cuda.current_stream()
    k = max(1, min(steps, 5))
    e0.record()
    for _ in range(k):
        ctx.ntt_batch(jobs, per_call=True, stream=s2)
    e1.record()
    torch.cuda.synchronize()
    per_ms = e0.elapsed_time(e1) / k
    b.close()
    ctx.close()
    del data
    bal = sum(b_alg("gl64", s) for s in sizes)
    return {"sizes": sizes, "total": total, "ms": ms, "per_ms": per_ms, "bit_exact": bit_exact, "ok": ok,
            "info": info, "b_alg": bal}


def run_batch_mix(args):
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    import stntt_gb300 as st

    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    time.sleep(0.25)
    m = measure_batch_mix(st, torch, dev, args.mix_jobs, args.steps, args.warmup, rank, world)
    clocks = sampler.stop()
    ms = max_over_ranks(m["ms"], world, dev) if world > 1 else m["ms"]
    value = world * m["total"] / (ms / 1e3) / 1e9
    hbm, hbm_kind = peaks()
    achieved = m["b_alg"] / (ms / 1e3) / 1e9
    if rank == 0:
        print(json.dumps({
            "metric": "NTT Gelem/s (uneven batch: 4096 Goldilocks transforms, log2 n in [10,18])",
            "value": value, "unit": "Gelem/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (splitmix64 uniform residues)",
            "config": {"workload": "gl64_batch_mix", "jobs": len(m["sizes"]), "log_n_range": [MIX_LO, MIX_HI],
                       "seed": MIX_SEED, "elements": m["total"], "directions": "alternating forward / inverse",
                       "launch": "one persistent launch replayed from a CUDA graph",
                       "l2": "inputs (1.9 GB) larger than L2", **m["info"]},
            "per_call": {"value": world * m["total"] / (m["per_ms"] / 1e3) / 1e9, "ms_per_step": m["per_ms"],
                         "launch": "one launch sequence per transform (stntt_ntt_batch_per_call)"},
            "speedup_vs_per_call": m["per_ms"] / ms, "bit_exact_vs_per_call": m["bit_exact"],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": hbm_kind, "b_alg_per_step": m["b_alg"]},
            "clocks": clocks, "gpu_launches": args.steps, "status_ok": m["ok"]}), flush=True)


# --------------------------------------------------------------------------- serving loop
SERVE_RATE, SERVE_LO, SERVE_HI, SERVE_SEED = 20000.0, 12, 22, 0x57170001 + 4


def device_stalls(torch, seconds: float = 1.5, threshold_ms: float = 2.0):
    """How often this GPU stops for a while on its own: back-to-back tiny
    kernels (no library code) on one stream for `seconds`, a CUDA event after
    each; every gap between consecutive completions above threshold_ms is a
    stall that any request in flight at that moment waits out. Reported beside
    the serving latencies, whose tail such stalls set."""
    s = torch.cuda.Stream()
    x = torch.zeros(1024, dtype=torch.int32, device="cuda")
    start = torch.cuda.Event(enable_timing=True)
    evs = []
    with torch.cuda.stream(s):
        start.record(s)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds and len(evs) < 400000:
            for _ in range(32):
                x.add_(1)
                e = torch.cuda.Event(enable_timing=True)
                e.record(s)
                evs.append(e)
            if len(evs) % 1024 == 0:
                evs[-1].synchronize()  # keep the device queue short: completions follow submissions
    s.synchronize()
    t = [start.elapsed_time(e) for e in evs]
    gaps = [{"at_ms": round(t[i - 1], 2), "gap_ms": round(t[i] - t[i - 1], 2)}
            for i in range(1, len(t)) if t[i] - t[i - 1] > threshold_ms]
    return {"span_ms": round(t[-1], 1) if t else 0.0, "kernels": len(t), "threshold_ms": threshold_ms,
            "stalls": gaps}


def measure_serve(st, torch, local: int, count: int, streams: int, rate: float = SERVE_RATE):
    """Seeded Poisson stream (mean 20k requests/s): 70% single NTTs, 30%
    cyclic polynomial products of two polynomials of degree < n/2, n = 2^k with
    k uniform in [12, 22], 50/50 32-bit prime / Goldilocks."""
    rng = np.random.default_rng(SERVE_SEED)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    kinds = rng.random(count) < 0.3
    logs = rng.integers(SERVE_LO, SERVE_HI + 1, count)
    gls = rng.integers(0, 2, count).astype(bool)
    dirs = rng.integers(0, 2, count)
    # operand pool: one pinned (a, b, out) triple per (field, size); inputs read-only
    pool = {}
    for lg in range(SERVE_LO, SERVE_HI + 1):
        n = 1 << lg
        for gl in (False, True):
            dt = torch.int64 if gl else torch.int32
            a, b, o = (torch.zeros(n, dtype=dt, pin_memory=True) for _ in range(3))
            if gl:
                a.numpy().view(np.uint64)[:] = st.uniform_gl64_host(lg, n)
                b.numpy().view(np.uint64)[: n // 2] = st.uniform_gl64_host(100 + lg, n // 2)
            else:
                p, _ = st.params_u32(lg)
                a.numpy().view(np.uint32)[:] = st.uniform_u32_host(lg, p, n)
                b.numpy().view(np.uint32)[: n // 2] = st.uniform_u32_host(100 + lg, p, n // 2)
            a2 = a.clone().pin_memory()
            a2.numpy()[n // 2:] = 0
            pool[(gl, lg)] = (a, a2, b, o)
    ctx = st.Context(local)
    sv = st.Server(ctx, streams=streams, max_log_n=SERVE_HI, prewarm=(SERVE_LO, SERVE_HI))
    reqs = []
    for i in range(count):
        lg, gl = int(logs[i]), bool(gls[i])
        a, a2, b, o = pool[(gl, lg)]
        p, root = (0, 0) if gl else st.params_u32(lg)
        if kinds[i]:
            reqs.append(st.Request(st.REQ_POLYMUL, st.FIELD_GL64 if gl else st.FIELD_U32, lg, 0, p, root, i,
                                   a2.data_ptr(), b.data_ptr(), o.data_ptr()))
        else:
            reqs.append(st.Request(st.REQ_NTT, st.FIELD_GL64 if gl else st.FIELD_U32, lg, int(dirs[i]), p, root, i,
                                   a.data_ptr(), 0, o.data_ptr()))
    # warm-up: the first few requests, run to completion
    sv.run_trace(reqs[: min(200, count)], [0.0] * min(200, count))
    stalls = device_stalls(torch)
    t0 = time.perf_counter()
    comps = sv.run_trace(reqs, list(arrivals))
    wall = time.perf_counter() - t0
    ok = all(c.status == 0 for c in comps)
    lat = np.array([c.done_s - c.submit_s for c in comps]) * 1e3
    qwait = np.array([c.start_s - c.submit_s for c in comps]) * 1e3
    span = max(c.done_s for c in comps) - min(c.submit_s for c in comps)
    elems = float(sum((3 if kinds[i] else 1) * (1 << int(logs[i])) for i in range(count)))
    stats = sv.stats()
    sv.close()
    ctx.close()
    return {
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p90": float(np.percentile(lat, 90)),
                       "p99": float(np.percentile(lat, 99)), "max": float(lat.max()),
                       "queue_p50": float(np.percentile(qwait, 50)), "queue_p99": float(np.percentile(qwait, 99))},
        "throughput": {"requests_per_s": count / span, "offered_per_s": rate,
                       "transform_gelem_per_s": elems / span / 1e9, "span_s": span, "wall_s": wall},
        "requests": count, "server": stats, "status_ok": ok, "device_stalls_before_trace": stalls}


def run_serve_mix(args):
    import torch
    import stntt_gb300 as st

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    count = args.serve_requests or max(1000, args.steps * 1000)
    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    time.sleep(0.25)
    m = measure_serve(st, torch, local, count, args.streams, args.serve_rate)
    clocks = sampler.stop()
    if rank == 0:
        print(json.dumps({
            "metric": "serving: p50/p99 request latency (ms) and throughput at 20k requests/s offered",
            "value": m["latency_ms"]["p99"], "unit": "ms (p99 latency)", "higher_is_better": False,
            "n_gpus": world, "steps": args.steps, "warmup": 200, "ms_per_step": None, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32+u64", "data": "synthetic (splitmix64 residues, seeded Poisson trace)",
            "config": {"workload": "serve_mix", "requests": count, "rate_per_s": args.serve_rate,
                       "log_n_range": [SERVE_LO, SERVE_HI], "polymul_fraction": 0.3, "fields": "50/50",
                       "streams": args.streams, "seed": SERVE_SEED},
            "latency_ms": m["latency_ms"], "throughput": m["throughput"], "server": m["server"], "clocks": clocks,
            "status_ok": m["status_ok"], "device_stalls_before_trace": m["device_stalls_before_trace"]}), flush=True)


# --------------------------------------------------------------------------- our arm, single transforms
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if WORKLOADS[args.workload][1] == "serve":
        run_serve_mix(args)
        return
    if WORKLOADS[args.workload][1] == "batch":
        run_batch_mix(args)
        return
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    import stntt_gb300 as st

    field, lg = WORKLOADS[args.workload]
    n = 1 << lg
    esz = 8 if field == "gl64" else 4
    ctx = st.Context(local)
    ctx.set_tma({"auto": -1, "on": 1, "off": 0}[args.tma])

    sampler = ClockSampler(gpu_index(local))
    sampler.start()
    time.sleep(0.25)
    if world > 1:
        torch.distributed.barrier()
    m = measure_single(ctx, st, torch, field, lg, args.steps, args.warmup, dev, rank)
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    step_ms = m["step_ms"]
    total_ms = step_ms * args.steps
    if world > 1:
        total_ms = max_over_ranks(total_ms, world, dev)
        step_ms = total_ms / args.steps
    value = world * 2 * n * args.steps / (total_ms / 1e3) / 1e9
    ok = m["ok"]
    passes = m["passes"]
    roofline = roofline_of(field, lg, step_ms, m["t_fwd"], m["t_inv"], passes, args.workload)
    roofline["pass_log_lengths"] = m["pass_logs"]

    int_roofline = None
    if field == "gl64":
        rate = st.gl64_butterfly_rate(local)  # measured now, same arithmetic on registers
        bfly = (n // 2) * lg  # butterflies per transform
        got = bfly / (step_ms / 2 / 1e3)
        int_roofline = {"bound": "int", "unit": "Gbutterfly/s", "achieved": got / 1e9, "peak": rate / 1e9,
                        "frac": got / rate, "peak_kind": "measured (stntt_measure_gl64_butterfly_rate)",
                        "butterflies_per_transform": bfly}

    # End to end through the C ABI: each step copies its input in from pinned
    # host memory, runs forward + inverse (stntt_ntt_gl64 / stntt_ntt_u32 on the
    # caller's stream) and reads the result back, all inside the timed region.
    # Steps go round E2E_SLOTS streams, each with its own device buffer and
    # pinned input / output buffers, so one step's copy in overlaps another's
    # copy out and transform (what a caller streaming data through the GPU
    # does); `serial` is the same with each step finished before the next.
    e2e = None
    data, ref_copy, fwd, inv, stream = m["data"], m["ref"], m["fwd"], m["inv"], m["stream"]
    if not args.no_e2e:
        dt_host = torch.int64 if field == "gl64" else torch.int32
        ref_host = ref_copy.cpu()
        k = max(3, min(args.steps, 50))
        slots = []
        for _ in range(E2E_SLOTS):
            h_in = torch.empty(n, dtype=dt_host, pin_memory=True)
            h_in.copy_(ref_host)
            slots.append({"in": h_in, "out": torch.empty(n, dtype=dt_host, pin_memory=True),
                          "dev": torch.empty(n, dtype=dt_host, device=dev), "stream": torch.cuda.Stream(device=dev)})

        def e2e_step(sl):
            sp = sl["stream"].cuda_stream
            with torch.cuda.stream(sl["stream"]):
                sl["dev"].copy_(sl["in"], non_blocking=True)
                if field == "gl64":
                    ctx.ntt_gl64(sl["dev"], lg, 1, inverse=False, stream=sp)
                    ctx.ntt_gl64(sl["dev"], lg, 1, inverse=True, stream=sp)
                else:
                    ctx.ntt_u32(sl["dev"], lg, 1, p_u32, root_u32, inverse=False, stream=sp)
                    ctx.ntt_u32(sl["dev"], lg, 1, p_u32, root_u32, inverse=True, stream=sp)
                sl["out"].copy_(sl["dev"], non_blocking=True)

        p_u32, root_u32 = (0, 0) if field == "gl64" else st.params_u32(lg)
        for sl in slots:  # warm-up: every stream's workspace and the plans exist before timing
            e2e_step(sl)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(k):
            e2e_step(slots[i % E2E_SLOTS])
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / k
        ok = ok and all(bool(torch.equal(sl["out"], ref_host)) for sl in slots)
        t0 = time.perf_counter()
        for _ in range(k):
            e2e_step(slots[0])
            slots[0]["stream"].synchronize()
        dt_serial = (time.perf_counter() - t0) / k
        ok = ok and bool(torch.equal(slots[0]["out"], ref_host))
        e2e = {"value": world * 2 * n / dt / 1e9, "unit": "Gelem/s", "h2d_bytes_per_step": n * esz,
               "d2h_bytes_per_step": n * esz, "ms_per_step": dt * 1e3,
               "api": ("stntt_ntt_gl64" if field == "gl64" else "stntt_ntt_u32")
               + f" forward then inverse per step, pinned copy in before and out after; steps on {E2E_SLOTS} "
               "streams with their own buffers",
               "serial": {"value": world * 2 * n / dt_serial / 1e9, "ms_per_step": dt_serial * 1e3,
                          "api": "the same, each step finished before the next starts"}}
        host = slots[0]["out"]
        host.copy_(ref_host)
        if field == "gl64":
            # the host-buffer convenience call, once per direction (each copies in and out)
            hv = host.numpy().view(np.uint64)
            ctx.ntt_gl64_host(hv, lg)
            ctx.ntt_gl64_host(hv, lg, inverse=True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(k):
                ctx.ntt_gl64_host(hv, lg)
                ctx.ntt_gl64_host(hv, lg, inverse=True)
            dt2 = (time.perf_counter() - t0) / k
            ok = ok and bool(torch.equal(host, ref_copy.cpu()))
            e2e["host_call"] = {"value": world * 2 * n / dt2 / 1e9, "ms_per_step": dt2 * 1e3,
                                "h2d_bytes_per_step": 2 * n * esz, "d2h_bytes_per_step": 2 * n * esz,
                                "api": "stntt_ntt_gl64_host, forward then inverse (each call copies in and out)"}
        del host, slots
    del m, data, ref_copy

    # The other configurations, one GPU only (the replica runs time the headline).
    secondary = None
    if world == 1 and args.workload == DEFAULT_WORKLOAD and not args.no_secondary:
        secondary = {}
        for name, (f2, l2) in (("gl64_2^20_fwd+inv", ("gl64", 20)), ("u32_2^26_fwd+inv", ("u32", 26)),
                               ("u32_2^20_fwd+inv", ("u32", 20)), ("u32_2^16_fwd+inv", ("u32", 16))):
            secondary[name] = secondary_single(ctx, st, torch, f2, l2, dev)
        torch.cuda.synchronize()
        bm = measure_batch_mix(st, torch, dev, args.mix_jobs, 10, 3)
        hbm, _ = peaks()
        secondary["gl64_batch_mix"] = {
            "value": bm["total"] / (bm["ms"] / 1e3) / 1e9, "unit": "Gelem/s", "ms_per_step": bm["ms"],
            "per_call_ms": bm["per_ms"], "speedup_vs_per_call": bm["per_ms"] / bm["ms"],
            "bit_exact_vs_per_call": bm["bit_exact"], "status_ok": bm["ok"], "jobs": len(bm["sizes"]),
            "elements": bm["total"], "hbm_frac": bm["b_alg"] / (bm["ms"] / 1e3) / 1e9 / hbm, "steps": 10,
            "launch": "one persistent launch replayed from a CUDA graph; per call: one launch sequence per job"}
        sv = measure_serve(st, torch, local, args.serve_requests or 20000, args.streams)
        secondary["serve_mix"] = {"latency_ms": sv["latency_ms"], "throughput": sv["throughput"],
                                  "requests": sv["requests"], "status_ok": sv["status_ok"],
                                  "rate_per_s": SERVE_RATE, "log_n_range": [SERVE_LO, SERVE_HI],
                                  "device_stalls_before_trace": sv["device_stalls_before_trace"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(field, lg)

    if rank == 0:
        line = {
            "metric": METRIC if args.workload == DEFAULT_WORKLOAD else f"NTT Gelem/s ({args.workload})",
            "value": value, "unit": "Gelem/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64" if field == "gl64" else "u32",
            "data": "synthetic (splitmix64 uniform residues in [0,p), generated on the device)",
            "config": {"workload": args.workload, "field": field, "n": n, "batch": 1,
                       "step": "forward + inverse, in place", "l2": "flushed between steps (256 MiB write)",
                       "launch": "CUDA graph per transform, replayed" if lg <= 22 else "direct C-ABI calls",
                       "tma": args.tma, "parallelism": f"replicas x{world}"},
            "e2e": e2e, "roofline": roofline, "int_roofline": int_roofline, "cpu_baseline": cpu, "clocks": clocks,
            "gpu_launches": 2 * passes * args.steps, "round_trip_ok": ok, "secondary": secondary,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
