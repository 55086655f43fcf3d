"""Serving loop for Proth candidates on one GPU.

Candidates arrive over time (seeded Poisson arrivals; n log-uniform in
[10000, 300000], k odd in [3, 10^5)).  On arrival they are trial-divided on the
GPU by every prime below 2^32 (pg_sieve_strike against the primes a pg_sieve
holds in device memory, queued on a stream of its own beside the batch, so the
division overlaps the squaring work instead of pausing it); survivors are submitted to the batched engine (pg_batch), which
admits them under an HBM budget (the per-candidate device footprint of their
FFT length), keeps residues and their checkpoints (every 10,000 squarings) on
the device, and returns verdicts.  Reported: p50/p99 time-to-verdict (arrival to
verdict) and tests/hour, swept over arrival rates until throughput stops
growing.

    python -m prothlogic_gb300.serve --rates 16,32,64,128,256,512 --window 40
"""
import argparse
import json
import statistics
import time

from . import Batch, PrefilterStream, slot_footprint, workloads


def _pct(xs, q):
    if not xs:
        return None
    xs = sorted(xs)
    i = min(len(xs) - 1, max(0, int(round(q / 100.0 * (len(xs) - 1)))))
    return xs[i]


def serve(arrivals, budget_bytes=16 << 30, max_slots=1024, prefilter_bound=1 << 32, slice_steps=400,
          time_limit=None, window=None):
    """Run the loop over `arrivals` [(t_arrive_s, k, n)] (sorted by time).

    Returns per-candidate records and a summary.  Wall-clock times are host
    times since the start of the run.  Arrivals wait for the pre-filter stream
    (one call in flight, every candidate that arrived meanwhile in the next
    call); the batch advances `slice_steps` squarings per loop turn while the
    pre-filter works.  `window`: the arrival window in seconds (default: the
    last arrival); delivered throughput is counted over its second half, where
    the loop is in its steady state, and candidates still running at
    `time_limit` count as not delivered."""
    b = Batch(max_slots)
    b.set_budget(budget_bytes)
    pf = PrefilterStream(bound=prefilter_bound)
    t0 = time.perf_counter()
    i = 0
    meta = {}
    records = []
    waiting = []    # arrived, not yet handed to the pre-filter
    inflight = []   # in the pre-filter call now running
    busy_s = 0.0
    while True:
        now = time.perf_counter() - t0
        while i < len(arrivals) and arrivals[i][0] <= now:
            waiting.append(arrivals[i])
            i += 1
        factors = pf.poll()
        if factors is not None:
            done_t = time.perf_counter() - t0
            for (ta, k, n), f in zip(inflight, factors):
                if f:
                    records.append({"k": k, "n": n, "t_arrive": ta, "t_verdict": done_t, "verdict": 0,
                                    "factor": f, "tested": False})
                else:
                    tag = len(meta)
                    meta[tag] = (ta, k, n)
                    b.submit(k, n, tag)
            inflight = []
        if waiting and not pf.busy():
            inflight, waiting = waiting[:pf.cap], waiting[pf.cap:]
            pf.start([(k, n) for _, k, n in inflight])
        q, r, f = b.pending()
        if q + r + f > 0:
            t_run = time.perf_counter()
            b.run(slice_steps)
            busy_s += time.perf_counter() - t_run
            t_now = time.perf_counter() - t0
            for res in b.poll():
                ta, k, n = meta[res["tag"]]
                records.append({"k": k, "n": n, "t_arrive": ta, "t_verdict": t_now, "verdict": res["verdict"],
                                "res64": res["res64"], "fft_len": res["fft_len"], "status": res["status"],
                                "bumps": res["fft_bumps"], "tested": True})
        elif pf.busy():
            time.sleep(0.001)
        elif i < len(arrivals):
            time.sleep(max(0.0, min(0.5, arrivals[i][0] - (time.perf_counter() - t0))))
        elif not waiting:
            break
        if time_limit is not None and time.perf_counter() - t0 > time_limit:
            break
    wall = time.perf_counter() - t0
    pf.close()
    b.close()
    tested = [r for r in records if r["tested"]]
    lat = [r["t_verdict"] - r["t_arrive"] for r in tested]
    lat_all = [r["t_verdict"] - r["t_arrive"] for r in records]
    span = max((r["t_verdict"] for r in records), default=0.0)
    win = window if window is not None else (arrivals[-1][0] if arrivals else 0.0)
    half = [r for r in tested if win / 2 <= r["t_verdict"] <= win]
    survivors = len(meta)
    summary = {
        "arrived": i, "completed": len(records), "prefilter_rejected": len(records) - len(tested),
        "tested": len(tested), "admitted": survivors, "unfinished": survivors - len(tested),
        "primes": sum(1 for r in tested if r["verdict"] == 1),
        "p50_s": _pct(lat, 50), "p99_s": _pct(lat, 99), "p50_all_s": _pct(lat_all, 50),
        "p99_all_s": _pct(lat_all, 99), "wall_s": wall, "window_s": win,
        "offered_tests_per_hour": survivors / win * 3600.0 if win > 0 else 0.0,
        "delivered_tests_per_hour": len(half) / (win / 2) * 3600.0 if win > 0 else 0.0,
        "tests_per_hour": len(tested) / span * 3600.0 if span > 0 else 0.0,
        "candidates_per_hour": len(records) / span * 3600.0 if span > 0 else 0.0,
        "gpu_busy_frac": busy_s / wall if wall > 0 else 0.0,
        "errors": sum(1 for r in tested if r.get("status", 0) != 0),
    }
    return records, summary


def sweep(rates, window_s=30.0, drain_s=60.0, seed=5, **kw):
    """Geometric sweep of arrival rates; stops once delivered tests/hour grows
    by less than 10 % from one rate to the next (saturation)."""
    out = []
    best = 0.0
    for lam in rates:
        count = max(1, int(lam * window_s * 1.5))
        arrivals = [(t, k, n) for t, k, n in workloads.serving(count, lam, seed=seed) if t <= window_s]
        _, s = serve(arrivals, time_limit=window_s + drain_s, window=window_s, **kw)
        s["rate_per_s"] = lam
        s["hbm_footprint_example_bytes"] = slot_footprint(3, 100000)
        out.append(s)
        print(json.dumps(s), flush=True)
        if best and s["delivered_tests_per_hour"] < 1.1 * best:
            break
        best = max(best, s["delivered_tests_per_hour"])
    return out


def prefilter_timing(seed=5, sizes=(1, 30, 300, 3000), slice_steps=400, slice_slots=60):
    """Host time of one pre-filter call per size, from the call to the answers
    on the host, for the allocating pg_prefilter, pg_prefilter_noalloc and a
    resident pg_sieve (the three must agree), then the time of one batch slice
    alone and beside a strike of each size."""
    from . import prefilter
    arr = workloads.serving(max(sizes) * 2, 256, seed=seed)
    cands = [(k, n) for _, k, n in arr]
    big = cands[:max(sizes)]
    out = {}
    for m in sizes:
        if m >= 30:
            t = time.perf_counter()
            prefilter(cands[:m])
            out[f"alloc_{m}"] = time.perf_counter() - t
    t = time.perf_counter()
    streams = {"resident": PrefilterStream()}
    out["resident_create"] = time.perf_counter() - t
    streams["noalloc"] = PrefilterStream(resident=False)
    want = prefilter(big)

    def wait(pf):
        while True:
            r = pf.poll()
            if r is not None:
                return r
            time.sleep(0.0002)

    for name, pf in streams.items():
        for m in sizes:
            t = time.perf_counter()
            pf.start(cands[:m])
            wait(pf)
            out[f"{name}_{m}"] = time.perf_counter() - t
        pf.start(big)
        if wait(pf) != want:
            raise RuntimeError(f"{name} pre-filter disagrees with pg_prefilter")
    survivors = [c for c, f in zip(big, want) if not f][:slice_slots]
    b = Batch(1024)
    for i, (k, n) in enumerate(survivors):
        b.submit(k, n, i)
    b.run(slice_steps)
    t = time.perf_counter()
    b.run(slice_steps)
    out["slice_alone"] = time.perf_counter() - t
    for name, pf in streams.items():
        for m in (30, max(sizes)):
            pf.start(cands[:m])
            t = time.perf_counter()
            b.run(slice_steps)
            out[f"slice_with_{name}_{m}"] = time.perf_counter() - t
            wait(pf)
    b.close()
    for pf in streams.values():
        pf.close()
    return {k: round(v, 4) for k, v in out.items()}


def strike_target(count=3000, seed=5):
    """One pg_sieve_strike of `count` candidates of the serving workload against
    every prime below 2^32 (a small profiling target: the sieve's 1.6 GB table,
    the candidates, one strike).  Returns the number the strike rejected."""
    import torch
    from . import Sieve
    cands = [(k, n) for _, k, n in workloads.serving(count, 256, seed=seed)][:count]
    sieve = Sieve(1 << 32, len(cands))
    ks = torch.tensor([k for k, _ in cands], dtype=torch.int64, device="cuda")
    ns = torch.tensor([n for _, n in cands], dtype=torch.int32, device="cuda")
    out = torch.zeros(len(cands), dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    sieve.strike(ks.data_ptr(), ns.data_ptr(), len(cands), out.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    rejected = int((out != 0).sum().item())
    sieve.close()
    return rejected


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rates", default="2,4,8,16,32")
    ap.add_argument("--window", type=float, default=30.0)
    ap.add_argument("--drain", type=float, default=60.0)
    ap.add_argument("--budget-gb", type=float, default=16.0)
    ap.add_argument("--slots", type=int, default=1024)
    ap.add_argument("--prefilter-timing", action="store_true",
                    help="time single pre-filter calls and a batch slice beside them, then exit")
    ap.add_argument("--strike-target", type=int, default=0, metavar="COUNT",
                    help="one resident-sieve strike of COUNT candidates (a profiling target), then exit")
    args = ap.parse_args()
    if args.prefilter_timing:
        print(json.dumps(prefilter_timing()))
        return
    if args.strike_target:
        print(json.dumps({"candidates": args.strike_target, "rejected": strike_target(args.strike_target)}))
        return
    rates = [float(x) for x in args.rates.split(",")]
    res = sweep(rates, window_s=args.window, drain_s=args.drain, budget_bytes=int(args.budget_gb * (1 << 30)),
                max_slots=args.slots)
    print(json.dumps({"sweep": res}))


if __name__ == "__main__":
    main()
