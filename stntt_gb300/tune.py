"""Autotuner for transform plans: pass split, elements per thread, columns per CTA
(and, with --batched, the pass split of jobs in the persistent batched launch).

For one (field, log_n) it enumerates plan shapes the library accepts
(``stntt_set_plan``), times each forward transform with CUDA events on a
buffer large enough to fill the GPU, keeps the fastest, and stores it in a
JSON cache keyed by the device (name | SM count | driver | capability, from
``stntt_device_key``). ``apply_cache(ctx)`` replays cached choices into a
context. Extends the reference's manual sweep over block sizes
(src/bench.cu:88-91, ntt_kernel.cuh:27).

    python -m stntt_gb300.tune --field gl64 --log-n 16 20 24
"""

from __future__ import annotations

import argparse
import itertools
import json
import os
import time
from pathlib import Path
from typing import Iterable

import stntt_gb300 as st

DEFAULT_CACHE = Path(os.environ.get("STNTT_TUNE_CACHE", str(Path.home() / ".cache" / "stntt_gb300" / "plans.json")))
# Plans the tuner chose on this project's GB300s, keyed "name|SM count" (no driver):
# applied to every new Context on a matching device unless STNTT_NO_TUNED_PLANS=1.
PACKAGED = Path(__file__).resolve().parent / "tuned_plans.json"


def splits(log_n: int, max_pass: int = 13) -> list[list[int]]:
    out = []
    if log_n <= max_pass:
        out.append([log_n])
    for a in range(max(1, log_n - max_pass), min(max_pass, log_n - 1) + 1):
        out.append([a, log_n - a])
    if log_n >= 18:
        for a in range(6, max_pass + 1):
            for b in range(6, max_pass + 1):
                c = log_n - a - b
                if 6 <= c <= max_pass:
                    out.append([a, b, c])
    return out


def vec_candidates(field: int, logs: list[int]) -> Iterable[tuple[list[int], list[int], list[int]]]:
    """The vector-lines build (STNTT_PASS_VEC) of a multi-pass split whose
    passes are 2^7..2^10 points: 8 or 16 points per line per pass (also 4
    where every pass is 2^9..2^11 points), 4 or 8
    line groups per CTA (V = 4 lines per thread for the 32-bit field, 2 for
    Goldilocks); two-pass splits with 2^11 or 2^12-point passes (the wide
    tiles that reach two HBM passes at 2^22..2^24 points, and spread single
    small transforms over more CTAs) take 1, 2 or 4 line groups, within 512
    threads and 200 KiB of shared memory."""
    if len(logs) < 2 or not all(7 <= lg <= 12 for lg in logs):
        return
    if len(logs) > 2 and any(lg > 10 for lg in logs):
        return
    v = 2 if field == st.FIELD_GL64 else 4
    w = 8 if field == st.FIELD_GL64 else 4
    wide = any(lg > 10 for lg in logs)
    per_line = (8 | st.PASS_VEC, 16 | st.PASS_VEC)
    if all(9 <= lg <= 11 for lg in logs):
        per_line += (4 | st.PASS_VEC,)  # twice the threads: for single transforms too small to fill the SMs
    for es in itertools.product(per_line, repeat=len(logs)):
        for g in ((1, 2, 4) if wide else (4, 8)):  # line groups per CTA
            # the row pass (last) also with the other group count: a warp's
            # load covers 32 / groups consecutive points of each row it
            # touches, so fewer groups fill more of each 32-byte sector
            # (32-bit 2^26 [9, 9, 8]: 8 / 8 / 4 groups 0.783 ms per forward +
            # inverse against 0.796 with 8 everywhere)
            for g_last in ((g,) if wide else (4, 8)):
                ok, cols = True, []
                for i, (lg, e) in enumerate(zip(logs, es)):
                    gi = g_last if i == len(logs) - 1 else g
                    gg = gi if lg > 10 else max(gi, 4)
                    threads = gg * (1 << lg) // (e & 0xff)
                    if threads > (512 if lg > 10 else 1024) or gg * v * (1 << lg) * w > 200 * 1024:
                        ok = False
                    cols.append(gg * v)
                if ok:
                    yield list(logs), list(es), cols


def cluster_candidates(field: int, logs: list[int]) -> Iterable[tuple[list[int], list[int], list[int]]]:
    """The vector-lines cluster build (STNTT_PASS_CLUSTER, 8 points per line)
    for the 2^11..2^13-point passes of a two-pass split, the other pass in the
    vector-lines build: 4 or 8 line groups per cluster or CTA, within 1024
    threads, the SM's 65536 registers (64 or 80 per thread) and 200 KiB of
    shared memory per CTA."""
    if len(logs) != 2 or not all(7 <= lg <= 13 for lg in logs) or max(logs) < 11:
        return
    v = 2 if field == st.FIELD_GL64 else 4
    w = 8 if field == st.FIELD_GL64 else 4
    regs = 80 if field == st.FIELD_GL64 else 64
    for g in (4, 8):
        es, ok = [], True
        for lg in logs:
            if lg >= 11:
                log1 = (lg + 1) // 2
                threads = (g << (lg - log1 - 3)) * ((1 << log1) // 8)
                ok &= threads <= 1024 and threads * regs <= 65536 and g * v * (1 << lg) * w // 8 <= 200 * 1024
                es.append(8 | st.PASS_VEC | st.PASS_CLUSTER)
            else:
                ok &= lg <= 10
                es.append(8 | st.PASS_VEC)
        if ok:
            yield list(logs), es, [g * v] * 2


def candidates(field: int, log_n: int, full: bool = False,
               vec: bool = False) -> Iterable[tuple[list[int], list[int], list[int]]]:
    """Plan shapes to try: every columns-per-CTA choice, 16 or 32 elements per
    thread (and 8 where every pass is 2^7..2^11 points); without `full`, only
    the three most even two-pass splits and the most even three-pass split;
    with `vec`, also the vector-lines build of every two- or three-pass split
    of 2^7..2^10-point passes, and two-pass splits with cluster passes."""
    sp = splits(log_n)
    if vec:
        for logs in sp:
            if len(logs) >= 2:
                yield from vec_candidates(field, logs)
                yield from cluster_candidates(field, logs)
    if not full:
        two = sorted([s for s in sp if len(s) <= 2], key=lambda s: max(s) - min(s))[:3]
        three = sorted([s for s in sp if len(s) == 3], key=lambda s: max(s) - min(s))[:1]
        sp = two + three
    for logs in sp:
        L_min = 1 << min(logs)
        es = [e for e in (16, 32) if e <= L_min]
        if all(7 <= lg <= 11 for lg in logs) and len(logs) > 1:
            es = [8] + es  # twice the threads per tile: for transforms too small to fill the SMs
        for e in es or [0]:
            per_pass = []
            for lg in logs:
                L = 1 << lg
                if len(logs) == 1:
                    per_pass.append([0])
                else:
                    cs = [c for c in (1, 2, 4, 8, 16, 32, 64) if c * L <= (1 << 15)]
                    per_pass.append(cs)
            for combo in itertools.product(*per_pass):
                yield logs, [e] * len(logs), list(combo)


def _time_plan(ctx: st.Context, field: int, log_n: int, data, p: int, root: int, batch: int, reps: int,
               flush, inverse_too: bool = False) -> float:
    """Mean device time of one forward call (CUDA events around each call),
    with L2 flushed before every call as in bench.py. Calls of fewer than 2^22
    elements are captured once as a CUDA graph and replayed, as bench.py times
    them (a direct call's host work can leave gaps between its kernels).
    inverse_too: time bench.py's step instead, the forward call then the
    inverse (one graph each)."""
    import torch

    stream = torch.cuda.Stream(device=data.device)
    sp = stream.cuda_stream

    def call(inv: bool):
        if field == st.FIELD_GL64:
            return lambda: ctx.ntt_gl64(data, log_n, batch, inverse=inv, stream=sp)
        return lambda: ctx.ntt_u32(data, log_n, batch, p, root, inverse=inv, stream=sp)

    runs = [call(False), call(True)] if inverse_too else [call(False)]
    with torch.cuda.stream(stream):
        for run in runs:
            run()
        stream.synchronize()
        if (batch << log_n) < (1 << 22):
            graphs = []
            for run in runs:
                graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(graph, stream=stream, capture_error_mode="relaxed"):
                    run()
                graphs.append(graph)
            parts = [g.replay for g in graphs]
        else:
            parts = runs

        def step():
            for part in parts:
                part()

        step()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) * 1e3 / reps  # microseconds per call


def tune(ctx: st.Context, field: int, log_n: int, reps: int = 10, full: bool = False, verbose: bool = False,
         batch: int = 0, vec: bool = False, verify: int = 0):
    """Return (best_spec, best_us, all_results) for one size; leaves the best plan set.
    batch 0: enough transforms for 2^24 elements (a GPU-filling batch).
    verify k > 1: re-time the k fastest forward candidates as forward + inverse
    steps and keep the fastest of those (verify_top)."""
    import torch

    batch = batch or max(1, (1 << 24) >> log_n)
    small = (batch << log_n) < (1 << 22)  # these calls use the small-call shape
    n = batch << log_n
    if field == st.FIELD_GL64:
        data = torch.empty(n, dtype=torch.int64, device=f"cuda:{ctx.device}")
        st.fill_uniform_gl64(data, 99)
        p = root = 0
    else:
        p, root = st.params_u32(log_n)
        data = torch.empty(n, dtype=torch.int32, device=f"cuda:{ctx.device}")
        st.fill_uniform_u32(data, 99, p)
    flush = torch.empty(64 << 20, dtype=torch.int32, device=f"cuda:{ctx.device}")  # 256 MiB, twice L2
    results = []
    for logs, es, cs in candidates(field, log_n, full, vec):
        try:
            ctx.set_plan(field, log_n, logs, es, cs, small=small)
            us = _time_plan(ctx, field, log_n, data, p, root, batch, reps, flush)
        except st.StnttError as e:
            if verbose:
                print("skip", logs, es, cs, e)
            continue
        results.append({"logs": logs, "E": es, "C": cs, "us": us, "batch": batch})
        if verbose:
            print(f"{logs} E={es} C={cs}: {us:.1f} us", flush=True)
    results.sort(key=lambda r: r["us"])
    best = results[0]
    if verify > 1:
        def step_us(r):
            ctx.set_plan(field, log_n, r["logs"], r["E"], r["C"], small=small)
            return _time_plan(ctx, field, log_n, data, p, root, batch, reps, flush, inverse_too=True)

        best = verify_top(results, verify, step_us)[0]
        if verbose:
            print(f"verified {verify}: {best['logs']} E={best['E']} C={best['C']}: {best['step_us']:.1f} us per "
                  "forward + inverse", flush=True)
    ctx.set_plan(field, log_n, best["logs"], best["E"], best["C"], small=small)
    return best, results


def verify_top(results: list[dict], k: int, step_us) -> list[dict]:
    """The k fastest forward-only candidates (results sorted by "us"), each
    given "step_us" = step_us(candidate) (bench.py's forward + inverse step),
    sorted by it. The forward-only ranking can miss: at Goldilocks 2^20 it put
    [10, 10] (4 and 16 points per line) level with [11, 9], which the bench's
    step times at 67.5 against 60.9 us."""
    top = results[:k]
    for r in top:
        r["step_us"] = step_us(r)
    return sorted(top, key=lambda r: r["step_us"])


def batched_candidates(log_n: int) -> list[list[int]]:
    """Pass splits a job can take inside the persistent batched launch: one
    pass, or (from 2^13 points: a work item holds 8192 elements of one job)
    two of 2^4..2^13 points each."""
    out = [[log_n]] if 4 <= log_n <= 13 else []
    if log_n >= 13:
        for a in range(4, 14):
            if 4 <= log_n - a <= 13:
                out.append([a, log_n - a])
    return out


def tune_batched(ctx: st.Context, field: int, log_n: int, reps: int = 10, verbose: bool = False, jobs: int = 0):
    """Pass split for jobs of one size in the persistent batched launch: times
    stntt_batch_launch (captured in a CUDA graph and replayed, as in the bench's
    uneven mix) on `jobs` same-size transforms, half forward and half inverse,
    2^25 elements in all by default (more than L2 holds). Returns (best, all
    results) and leaves the best split set."""
    import torch

    jobs = jobs or max(8, (1 << 25) >> log_n)
    n = 1 << log_n
    dev = f"cuda:{ctx.device}"
    if field == st.FIELD_GL64:
        data = torch.empty(jobs * n, dtype=torch.int64, device=dev)
        st.fill_uniform_gl64(data, 98)
        p = root = 0
        esz = 8
    else:
        p, root = st.params_u32(log_n)
        data = torch.empty(jobs * n, dtype=torch.int32, device=dev)
        st.fill_uniform_u32(data, 98, p)
        esz = 4
    job_list = [st.Job(field, log_n, i % 2, p, root, 0, data.data_ptr() + esz * n * i) for i in range(jobs)]
    stream = torch.cuda.Stream(device=dev)
    results = []
    for logs in batched_candidates(log_n):
        try:
            ctx.set_plan(field, log_n, logs, batched=True)
            b = ctx.batch_create(job_list)
        except st.StnttError as e:
            if verbose:
                print("skip", logs, e)
            continue
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                b.launch(stream=stream)
            for _ in range(2):
                g.replay()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                g.replay()
            e1.record()
            torch.cuda.synchronize()
            ok = b.status() == 0
        finally:
            b.close()
        if not ok:
            continue
        us = e0.elapsed_time(e1) * 1e3 / reps
        results.append({"logs": logs, "E": [16] * len(logs), "C": [0] * len(logs), "us": us, "batch": jobs,
                        "batched": True})
        if verbose:
            print(f"batched {logs}: {us:.1f} us", flush=True)
    results.sort(key=lambda r: r["us"])
    best = results[0]
    ctx.set_plan(field, log_n, best["logs"], batched=True)
    return best, results


def _key(device: int) -> str:
    return st.device_key(device)


def load_cache(path: Path = DEFAULT_CACHE) -> dict:
    try:
        return json.loads(Path(path).read_text())
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path: Path = DEFAULT_CACHE) -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    os.replace(tmp, path)


def _device_class(key: str) -> str:
    return "|".join(key.split("|")[:2])  # GPU name | SM count


def apply_cache(ctx: st.Context, path: Path = DEFAULT_CACHE) -> int:
    """Set every cached plan for this device on `ctx`; returns how many.
    Exact device keys win; otherwise the packaged plans for the device class."""
    key = _key(ctx.device)
    entries = dict(load_cache(PACKAGED).get(_device_class(key), {}))
    entries.update(load_cache(path).get(key, {}))
    k = 0
    for name, e in entries.items():
        # "field:log_n", "field:log_n:b1" for single-transform calls, "field:log_n:batch"
        # for jobs of the persistent batched launch
        parts = name.split(":")
        field = st.FIELD_GL64 if parts[0] == "gl64" else st.FIELD_U32
        tag = parts[2] if len(parts) > 2 else ""
        ctx.set_plan(field, int(parts[1]), e["logs"], e["E"], e["C"], small=tag == "b1", batched=tag == "batch")
        k += 1
    return k


def record(ctx: st.Context, field: int, log_n: int, best: dict, path: Path = DEFAULT_CACHE) -> None:
    """Store a tuned shape; timed on single transforms that do not fill the GPU
    (batch * n < 2^22), it is stored as the small-call shape ("...:b1")."""
    cache = load_cache(path)
    ent = cache.setdefault(_key(ctx.device), {})
    small = (best["batch"] << log_n) < (1 << 22)
    suffix = ":batch" if best.get("batched") else (":b1" if small else "")
    ent[f"{'gl64' if field == st.FIELD_GL64 else 'u32'}:{log_n}" + suffix] = {
        "logs": best["logs"], "E": best["E"], "C": best["C"], "us": best["us"], "batch": best["batch"],
        "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    save_cache(cache, path)


def package(cache: Path, out: Path = PACKAGED) -> None:
    """Fold a tuner cache into the packaged plans (keyed by device class)."""
    src = load_cache(cache)
    dst = load_cache(out)
    for key, entries in src.items():
        cls = dst.setdefault(_device_class(key), {})
        for name, e in entries.items():
            cls[name] = {k: e[k] for k in ("logs", "E", "C", "us")}
    save_cache(dst, out)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--field", choices=["gl64", "u32"], default="gl64")
    ap.add_argument("--log-n", type=int, nargs="+", default=[20, 24])
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--full", action="store_true")
    ap.add_argument("--batch", type=int, default=0, help="transforms per timed call (0: 2^24 elements' worth)")
    ap.add_argument("--cache", default=str(DEFAULT_CACHE))
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--out", default=None, help="also write all timings here (JSON)")
    ap.add_argument("--package", action="store_true", help="fold the results into the packaged plans")
    ap.add_argument("--batched", action="store_true",
                    help="tune the pass split of jobs in the persistent batched launch instead")
    ap.add_argument("--vec", action="store_true", help="also try the vector-lines build of three-pass splits")
    ap.add_argument("--verify", type=int, default=0,
                    help="re-time the k fastest forward candidates as forward + inverse steps (bench.py's step)")
    args = ap.parse_args()
    field = st.FIELD_GL64 if args.field == "gl64" else st.FIELD_U32
    ctx = st.Context(0)
    allres = {}
    for lg in args.log_n:
        if args.batched:
            best, res = tune_batched(ctx, field, lg, args.reps, args.verbose, args.batch)
            record(ctx, field, lg, best, Path(args.cache))
            allres[f"{args.field}:{lg}:batch"] = res
            print(json.dumps({"size": f"{args.field}:{lg}:batch", "best": best, "candidates": len(res)}), flush=True)
            continue
        best, res = tune(ctx, field, lg, args.reps, args.full, args.verbose, args.batch, args.vec, args.verify)
        record(ctx, field, lg, best, Path(args.cache))
        allres[f"{args.field}:{lg}" + (":b1" if (best["batch"] << lg) < (1 << 22) else "")] = res
        print(json.dumps({"size": f"{args.field}:{lg}", "best": best, "candidates": len(res)}), flush=True)
    if args.out:
        Path(args.out).write_text(json.dumps(allres, indent=1))
    if args.package:
        package(Path(args.cache))
    ctx.close()


if __name__ == "__main__":
    main()
