#!/usr/bin/env python3
"""Headline benchmark: ns per modular squaring of one Proth candidate k*2^n+1
with n = 1,048,576 (k odd, uniform in [3, 2^20) from seed 2, x0 = a), with a
Gerbicz check over blocks of 1,000 squarings.

One "step" is one Gerbicz block of 1,000 squarings.  The default run times
K = 10 steps (10,000 squarings) after W = 3 warm-up steps; the Gerbicz
verification of all K blocks runs inside the last timed step.

  value  device time (CUDA events on the engine's stream) per squaring, residue
         resident on the device, L2 flushed between steps;
  e2e    the same metric through the public C ABI with host buffers, one
         step per run of the configuration: upload the input residue
         (pg_set_residue, H2D), 10,000 squarings with a Gerbicz check every
         1,000, return the verified result (pg_get_residue, D2H);
  --impl reference  the reference algorithm on this host's cores (the C oracle
         restatement of prothlogic4.2's engine; the reference's AVX-512 code
         itself only builds on x86-64), same metric and config.

Beside the headline, the line carries the other single-GPU configurations:
`batched` (4,096 candidates at n = 65,536), `batched_uneven` (2,048 candidates,
n log-uniform in [8,192, 262,144]) and `single_test` (whole tests at n = 32,768),
each against one-at-a-time on the GPU and the reference algorithm on all host
cores.  The serving sweep (Poisson arrivals) runs as prothlogic_gb300/serve.py.

Multi-GPU: candidates do not shard, so N > 1 runs N independent replicas
(one process per GPU) and `value` is the whole-job time per squaring.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from prothlogic_gb300 import workloads  # noqa: E402

METRIC = "ns per mod-squaring (n=1,048,576)"
UNIT = "ns/squaring"
SQ_PER_STEP = 1000
E2E_SQ_PER_STEP = 10 * SQ_PER_STEP  # one run of the configuration: 10,000 squarings, Gerbicz every 1,000


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
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
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dp_ops_per_point(plan_F):
    """FP64 instructions per complex point of one squaring, counted from the kernels."""
    def fft(F):
        lg = int(math.log2(F))
        n4 = lg // 2
        ops = 7 * (n4 - 1) + 4  # radix-4 stages with twiddles (7/pt) and the twiddle-free last one (4/pt)
        if lg & 1:
            ops = 7 * n4 + 2    # all radix-4 stages keep twiddles, then a radix-2 stage (2/pt)
        return ops
    F = plan_F
    if len(F) == 3:
        first = 2 + fft(F[0]) + 4
        mid = fft(F[1]) + 4
        inner = 2 * fft(F[2]) + 4
        last = 4 + fft(F[0]) + 4 + 6
        return first + 2 * mid + inner + last
    first = 2 + fft(F[0]) + 4
    inner = 2 * fft(F[1]) + 4
    last = 4 + fft(F[0]) + 4 + 6
    return first + inner + last


def profile_traffic():
    """(DRAM bytes of one squaring, the launch shape they were captured on) from
    the ncu capture data committed under profiles/, or (None, None)."""
    try:
        with open(os.path.join(ROOT, "profiles", "squaring_n1048576.json")) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_squaring"]), d["profiled_shape"]
    except (OSError, KeyError, ValueError):
        return None, None


def large_parity(k, a, squarings, residue):
    """'ok' / 'MISMATCH' for the residue after `squarings` squarings of x0 = a at
    the n = 2^20 configuration, against the GMP values in tests/golden (RES64
    every 1,000 squarings up to 200,000); 'unchecked: ...' beyond them."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            g = json.load(f)["large"]
    except (OSError, KeyError):
        return "unchecked: golden vector missing"
    if g["k"] != k or g["a"] != a:
        return "unchecked: golden vector is for another candidate"
    if squarings % g["every"] or squarings > len(g["res64"]) * g["every"]:
        return f"unchecked: {squarings} squarings is beyond the golden vector ({len(g['res64']) * g['every']})"
    want = g["res64"][squarings // g["every"] - 1]
    return "ok" if format(residue & ((1 << 64) - 1), "016x") == want else "MISMATCH"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pgd = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pgd = dist
    return world, rank, local, pgd


def barrier(pgd):
    if pgd is not None:
        pgd.barrier()


def max_over_ranks(pgd, v):
    if pgd is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pgd.all_reduce(t, op=pgd.ReduceOp.MAX)
    return float(t.item())


def cpu_sample_seconds():
    return float(os.environ.get("PROTH_CPU_SAMPLE_S", "15"))


def cpu_flags_note():
    from oracle.build_oracle import bench_flags
    return " ".join(f for f in bench_flags() if f not in ("-std=c11", "-fPIC", "-shared"))


def cpu_reference_setup(k, n):
    """(callable that times `count` squarings and returns seconds, kind, L, flags):
    the unmodified reference engine (oracle/_ref) where it was built (x86-64 with
    AVX-512), else the C restatement built with the reference's optimisation flags."""
    from oracle.build_oracle import build_ref
    from tests import _oracle
    fast = _oracle.bench_lib()
    L = fast.ora_choose_L(n, k)
    a = int(fast.ora_choose_base(k, n))
    ref = build_ref() if os.environ.get("PROTH_USE_REF", "1") == "1" else None
    if ref:
        def run(count):
            out = subprocess.run([ref, "time", str(k), str(n), str(L), str(count)], capture_output=True, text=True,
                                 check=True, cwd="/tmp")
            return float(out.stdout.strip().splitlines()[-1]) * 1e-6 * count
        return run, "reference", L, "SETUP:25 (-O3 -march=native -mavx512f ... -ffast-math)"
    ctx = _oracle.Ctx(L, fast)
    x = _oracle.to_limbs(a, L // 4)

    def run(count):
        t0 = time.perf_counter()
        fast.ora_run_squarings(ctx.h, x, n, k, count)
        return time.perf_counter() - t0
    run.ctx = ctx  # keeps the context alive
    return run, "port", L, cpu_flags_note()


def time_cpu_reference(k, n, budget_s, min_sq=4):
    """ns per squaring of the reference algorithm on one host core, over a sample of
    about budget_s seconds; returns (ns, kind, squarings, L, flags)."""
    run, kind, L, flags = cpu_reference_setup(k, n)
    t1 = run(1)
    count = max(min_sq, int(budget_s / max(t1, 1e-6)))
    dt = run(count)
    return dt / count * 1e9, kind, count, L, flags


def run_reference(args, world, rank, pgd):
    """The reference arm: the reference's CPU algorithm for this metric and
    workload on this host (one thread: the reference's per-candidate engine is
    single-threaded, SETUP:25 builds it without OpenMP).  Each step times the
    same bounded sample of squarings; only the oracle library is loaded."""
    if rank != 0:
        return 0
    k, n = workloads.large()
    run, kind, L, flags = cpu_reference_setup(k, n)
    per_step_budget = max(0.2, cpu_sample_seconds() / max(1, args.steps + args.warmup))
    t1 = run(1)
    sq_per_step = max(1, int(per_step_budget / max(t1, 1e-6)))
    for _ in range(args.warmup):
        run(sq_per_step)
    secs = [run(sq_per_step) for _ in range(args.steps)]
    v = sum(secs) / (sq_per_step * args.steps) * 1e9
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(secs) * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded candidate, no dataset)",
            "config": {"workload": "large: n=1048576, k odd in [3,2^20) seed 2, x0=a", "k": k, "n": n,
                       "fft_len_L": L, "squarings_per_step": sq_per_step,
                       "step": f"{sq_per_step} squarings of the reference algorithm (a bounded sample; the GPU "
                               f"arm's step is {SQ_PER_STEP} squarings, the metric is per squaring)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": kind, "flags": flags,
                             "host_cores": os.cpu_count(),
                             "sample": f"{sq_per_step} squarings per step x {args.steps} steps at n=1048576, "
                                       f"L={L}, one thread (the reference's per-candidate engine is "
                                       "single-threaded)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _chosen(rows):
    """'f0xf1[xf2] g_mid/g_inner (of N shapes)' for the shape the autotuner picked."""
    r = [x for x in rows if x["chosen"]][0]
    radices = "x".join(str(r[f]) for f in ("f0", "f1", "f2")[: r["passes"]])
    if r.get("resident"):
        return (f"{radices} resident in shared memory, {r['resident']} CTA(s) x {r['resident_threads']} threads "
                f"per residue (fastest of {len(rows)} bit-identical shapes)")
    mid = (f"middle fused in clusters of {r['cluster']} CTAs" if r.get("cluster")
           else f"g{r['g_mid']}/{r['g_inner']}")
    outer = r.get("tpb_outer") or r["tpb"]
    tpb = (f"{r['tpb']} thread(s)/butterfly" if outer == r["tpb"]
           else f"{r['tpb']} thread(s)/butterfly ({outer} in the first and last passes)")
    if r.get("edge"):
        tpb += ", last+first passes fused"
    if r.get("pinned"):
        return f"{radices} {mid} {tpb} (pinned by PROTH_SHAPE)"
    how = ("fastest in situ of the tuner's three fastest" if "us_in_situ" in r else "fastest")
    return f"{radices} {mid} {tpb} ({how} of {len(rows)} bit-identical shapes)"


def _top_shapes(rows, count=5):
    """The fastest valid shapes as (label, us per squaring), fastest first."""
    def label(r):
        radices = "x".join(str(r[f]) for f in ("f0", "f1", "f2")[: r["passes"]])
        if r.get("resident"):
            return f"{radices} res{r['resident']}x{r['resident_threads']}"
        mid = f"cl{r['cluster']}" if r.get("cluster") else f"g{r['g_mid']}/{r['g_inner']}"
        return (f"{radices} {mid} tpb{r['tpb']}/{r.get('tpb_outer') or r['tpb']}"
                + (" edge" if r.get("edge") else ""))
    ok = sorted((r for r in rows if r["valid"]), key=lambda r: r["us_per_step"])
    return [[label(r), round(r["us_per_step"], 2)] + ([round(r["us_in_situ"], 2)] if "us_in_situ" in r else [])
            for r in ok[:count]]


def _chosen_radices(rows):
    r = [x for x in rows if x["chosen"]][0]
    return tuple(r[f] for f in ("f0", "f1", "f2")[: r["passes"]])


GZ_EXTRA = 1500  # squarings per test spent on its end-of-chain Gerbicz check (1000 + 500 on average)


def cpu_tests_per_hour(cands, sq_sample, budget_s=None):
    """Reference-algorithm tests/hour on all host cores (one test per thread, as the
    reference's dispatcher runs them, prothlogic4.2/dcore.cpp:125-188), from every
    candidate truncated to `sq_sample` squarings and scaled to its full n - 1."""
    from tests import _oracle
    threads = os.cpu_count() or 1
    count = len(cands)
    ks = (ctypes.c_uint64 * count)(*[k for k, _ in cands])
    ns = (ctypes.c_uint * count)(*[n for _, n in cands])
    wall = _oracle.bench_lib().ora_bench_tests(ks, ns, count, threads, sq_sample, None)
    # each test also runs the a^k powering (bitlen(k) - 1 squarings) before its chain
    pow_sq = statistics.mean(max(0, k.bit_length() - 1) for k, _ in cands)
    full = statistics.mean(n - 1 for _, n in cands) + pow_sq
    scale = full / (sq_sample + pow_sq)
    return {"tests_per_hour": count * 3600.0 / (wall * scale), "cores": threads, "kind": "port",
            "flags": cpu_flags_note(),
            "sample": f"{count} tests on {threads} threads, each truncated to {sq_sample} squarings "
                      f"({wall:.1f} s), scaled by {scale:.0f} to full tests"}


def single_sample(pg, reps=3, cpu_sq=1000):
    """Configuration 1: whole Proth tests at n = 32768, one at a time on the GPU
    (pg_proth_test: gate, base, a^k, n - 1 squarings with the Gerbicz check,
    verdict), next to the reference algorithm's tests/hour on all host cores.
    The candidate is the first seed-1 draw that passes the reference's
    small-prime gate (a gated candidate is answered without a squaring)."""
    cands = workloads.single(16)
    k, n = next(c for c in cands if not pg.gate_rejects(*c))
    lg = pg.pick_fft_len(k, n).bit_length() - 1
    rows = pg.autotune(lg, slots=1, iters=200)
    r = pg.proth_test(k, n)  # warm-up: plan, weights, graphs
    secs = []
    for _ in range(reps):
        t0 = time.perf_counter()
        r = pg.proth_test(k, n)
        secs.append(time.perf_counter() - t0)
    sec = statistics.median(secs)
    want = golden_test(k, n)
    parity = "unchecked"
    if want is not None:
        ok = (r["verdict"], r["base"], format(r["res64"], "016x")) == (want["verdict"], want["base"], want["res64"])
        parity = "ok" if ok else "MISMATCH"
    threads = os.cpu_count() or 1
    cpu = cpu_tests_per_hour([(k, n)] * (2 * threads), cpu_sq)
    gpu_tph = 3600.0 / sec
    return {"workload": f"single: k={k}, n={n} (first seed-1 draw past the small-prime gate; "
                        f"{cands.index((k, n))} earlier draws are gated)",
            "k": k, "n": n, "fft_len": 1 << lg, "base": r["base"], "verdict": r["verdict"],
            "res64": format(r["res64"], "016x"), "parity_vs_reference": parity, "status": r["status"],
            "gerbicz_checks": r["gerbicz_checks"], "seconds_per_test_gpu": sec,
            "us_per_squaring_gpu": sec * 1e6 / (n - 1 + k.bit_length()),
            "gpu_tests_per_hour_one_at_a_time": gpu_tph, "shape": _chosen(rows),
            "cpu": cpu, "cpu_seconds_per_test_one_core": cpu["cores"] * 3600.0 / cpu["tests_per_hour"],
            "gpu_over_cpu_per_test": cpu["cores"] * 3600.0 / cpu["tests_per_hour"] / sec,
            "gpu_one_at_a_time_over_cpu_all_cores": gpu_tph / cpu["tests_per_hour"],
            "sample": f"median of {reps} whole tests after one warm-up test"}


def golden_test(k, n):
    """The reference's own result for the whole test k*2^n+1 (tests/golden), or None."""
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            g = json.load(f)
    except OSError:
        return None
    return next((t for t in g["tests"] + g["known"] if (t["k"], t["n"]) == (k, n)), None)


def shim_sample(pg):
    """Through the reference's engine API (fft_init / fft_square_karatsuba /
    fft_destroy) with the reference's own calling pattern: the squaring loop of
    execute_proth_test_fft (proth_logic.cpp:442-552), one fft_square_karatsuba per
    squaring on the caller's host limbs at the length auto_tune_fft_len picks
    (prothlogic_gb300/compat/compat_driver.cpp test).  The whole n = 32,768 test,
    and a 5,000-squaring sample of 843*2^120002+1."""
    from prothlogic_gb300 import build as b
    out = {}
    for k, n, steps in [(9505, 32768, 0), (843, 120002, 5000)]:
        L = 256
        while n / L > 18.0:
            L *= 2
        a = pg.choose_base(k, n)
        x0 = pow(a, k, k * (1 << n) + 1)
        r = subprocess.run([b.COMPAT_DRIVER, "test", str(k), str(n), str(L), str(steps)], input=format(x0, "x"),
                           capture_output=True, text=True, check=True).stdout.split()
        rec = {"k": k, "n": n, "L": L, "squarings": int(r[3]), "us_per_squaring": float(r[4]),
               "max_err": float(r[5])}
        if not steps:
            rec.update(verdict=int(r[1]), res64=r[2])
            want = golden_test(k, n)
            rec["parity_vs_reference"] = ("unchecked" if want is None else
                                          "ok" if (int(r[1]), r[2]) == (want["verdict"], want["res64"])
                                          else "MISMATCH")
        out[f"n={n}"] = rec
    out["note"] = ("per-call path: the caller's limbs go to the device only when changed, the residue comes "
                   "back after every squaring, Gerbicz blocks of 1,000 verified on schedule")
    return out


def serving_sample(pg, rates=(16, 64, 256), window_s=20.0, drain_s=20.0):
    """Configuration 5, short: Poisson arrivals (n log-uniform in [10,000, 300,000],
    k odd < 10^5, seed 5) at each rate for `window_s` seconds, trial division by
    every prime < 2^32 on its own stream, survivors through one Gerbicz-checked
    batch under a 16 GiB budget; `drain_s` more seconds for the last verdicts."""
    from prothlogic_gb300 import serve
    rows = []
    for lam in rates:
        count = max(1, int(lam * window_s * 1.5))
        arrivals = [(t, k, n) for t, k, n in workloads.serving(count, lam, seed=5) if t <= window_s]
        _, sm = serve.serve(arrivals, time_limit=window_s + drain_s, window=window_s)
        rows.append({"rate_per_s": lam, "arrived": sm["arrived"],
                     "prefilter_rejected_frac": sm["prefilter_rejected"] / max(1, sm["completed"]),
                     "tested": sm["tested"], "unfinished": sm["unfinished"], "p50_s": sm["p50_s"],
                     "p99_s": sm["p99_s"], "p50_all_s": sm["p50_all_s"],
                     "delivered_tests_per_hour": sm["delivered_tests_per_hour"],
                     "completed_tests_per_hour": sm["tests_per_hour"],
                     "offered_tests_per_hour": sm["offered_tests_per_hour"], "errors": sm["errors"]})
    return {"workload": f"serving: Poisson arrivals for {window_s:.0f} s per rate, n log-uniform in "
                        "[10000, 300000], k odd < 10^5 seed 5, pre-filter primes < 2^32",
            "rows": rows,
            "summary": {f"lambda={r['rate_per_s']}": [None if r["p50_s"] is None else round(r["p50_s"], 2),
                                                       None if r["p99_s"] is None else round(r["p99_s"], 2),
                                                       round(r["completed_tests_per_hour"]),
                                                       round(r["offered_tests_per_hour"])] for r in rows},
            "summary_columns": "p50 s, p99 s (arrival to verdict of tested candidates), tests/hour completed "
                               "(tests finished / time of the last verdict), offered (survivors of the "
                               "pre-filter per hour of arrivals); the full-length sweep is the serve module's CLI"}


def whole_batch(pg, cands, max_slots, parity_count=32, seed=11):
    """Every candidate through one Gerbicz-checked batch to its verdict (wall
    clock, submission to the last verdict), then a seeded subset of the tested
    ones recomputed with GMP (processes spawned after the GPU work)."""
    b = pg.Batch(max_slots)
    t0 = time.perf_counter()
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(0)
    wall = time.perf_counter() - t0
    res = {r["tag"]: r for r in b.poll()}
    b.close()
    tested = [i for i, r in res.items() if r["base"]]
    errors = sum(1 for r in res.values() if r["status"] != 0)
    parity = "unchecked"
    from tests import _gmp
    if _gmp.available() and tested:
        import random
        pick = random.Random(seed).sample(tested, min(parity_count, len(tested)))
        want = _gmp.proth_tests([cands[i] for i in pick])
        bad = [cands[i] for i, w in zip(pick, want)
               if (res[i]["verdict"], res[i]["base"], res[i]["res64"]) != w]
        parity = (f"ok ({len(pick)} of {len(tested)} tested candidates equal GMP)" if not bad
                  else f"MISMATCH at {bad[:4]}")
    return {"verdicts": len(res), "tested": len(tested), "primes": sum(1 for r in res.values() if r["verdict"] == 1),
            "errors": errors, "wall_s": wall, "tests_per_hour": len(tested) * 3600.0 / wall,
            "gerbicz_checks": sum(r["gerbicz_checks"] for r in res.values()),
            "gerbicz_failures": sum(r["gerbicz_failures"] for r in res.values()), "parity": parity}


def one_at_a_time_us(pg, k, n, iters=500):
    """Device-timed squarings of one candidate alone on the GPU (tuned one-residue shape)."""
    e = pg.Engine(k, n, flags=pg.FLAG_NO_GERBICZ)
    e.set_residue(3)
    e.time_squarings(100)
    ms, _ = e.time_squarings(iters)
    e.close()
    return ms * 1e3 / iters


def uneven_sample(pg, cpu_sq=60):
    """Uneven batch: 2,048 candidates, n log-uniform in [8192, 262144], k odd < 10^5
    (seed 4), every FFT-length class with its autotuned shape, the whole workload
    through one batch to the last verdict.  One at a time: per class, 500
    squarings of one candidate alone, scaled to every member's chain."""
    all_c = workloads.uneven(count=2048)
    cands = [(k, n) for k, n in all_c if not pg.gate_rejects(k, n)]
    classes = {}
    for k, n in cands:
        classes.setdefault(pg.pick_fft_len(k, n).bit_length() - 1, []).append((k, n))
    t_one = 0.0
    per_class = {}
    for lg, members in sorted(classes.items()):
        to = _chosen(pg.autotune(lg, slots=1, iters=200))
        one_sq = one_at_a_time_us(pg, *members[0]) * 1e-6
        work = sum(n - 1 + max(0, k.bit_length() - 1) + GZ_EXTRA for k, n in members)
        t_one += work * one_sq
        tm = _chosen(pg.autotune(lg, slots=min(len(members), 1024), iters=50))
        per_class[f"2^{lg}"] = {"candidates": len(members), "one_at_a_time_us_per_squaring": one_sq * 1e6,
                                "shape_batched": tm, "shape_one_at_a_time": to}
    whole = whole_batch(pg, all_c, 2048)
    pg.tune_clear()
    tph_batch = whole["tests_per_hour"]
    tph_one = len(cands) * 3600.0 / t_one
    cpu = cpu_tests_per_hour(cands, cpu_sq)
    return {"workload": "uneven: 2048 candidates, n log-uniform in [8192, 262144], k odd in [3,10^5) seed 4",
            "tested": len(cands), "classes": per_class, "whole_run": whole, "parity": whole["parity"],
            "batched_tests_per_hour": tph_batch, "one_at_a_time_tests_per_hour": tph_one,
            "batched_over_one_at_a_time": tph_batch / tph_one,
            "cpu_reference_tests_per_hour": cpu["tests_per_hour"],
            "batched_over_cpu": tph_batch / cpu["tests_per_hour"], "cpu": cpu,
            "sample": "batched: the whole workload to its last verdict (wall clock); one at a time: 500 "
                      "squarings of one candidate per class alone, scaled to each member's chain plus 1,500 "
                      f"for its Gerbicz check; {len(cands)} of 2048 pass the reference's gate"}


def batched_sample(pg):
    """Batched vs one-at-a-time tests/hour at n = 65536 (4096 candidates, k odd in
    [3, 10^6), seed 3): the whole workload through one batch to the last verdict."""
    cands = workloads.uniform(count=4096)
    n = cands[0][1]
    lg = pg.pick_fft_len(cands[0][0], n).bit_length() - 1
    tuned_many = _chosen(pg.autotune(lg, slots=1024, iters=50))
    tuned_one = _chosen(pg.autotune(lg, slots=1, iters=200))
    whole = whole_batch(pg, cands, 4096)
    # n-1 squarings + the a^k powering (bitlen(k) - 1 <= 19) + the Gerbicz check at the
    # end of each chain: one block (1000) of the product chain and on average half a
    # block of tail recompute (the same allowance for the one-at-a-time engine)
    sq_per_test = n - 1 + 19 + GZ_EXTRA
    us1 = one_at_a_time_us(pg, cands[0][0], n, iters=2000)
    tph_single = 3600.0 / (us1 * 1e-6 * sq_per_test)
    passing = [(k, nn) for k, nn in cands if not pg.gate_rejects(k, nn)]
    cpu = cpu_tests_per_hour(passing[: 4 * (os.cpu_count() or 1)], 200)
    pg.tune_clear()
    tph_batch = whole["tests_per_hour"]
    return {"workload": "uniform: 4096 candidates, n=65536, k odd in [3,10^6) seed 3",
            "whole_run": whole, "parity": whole["parity"],
            "batched_tests_per_hour": tph_batch, "one_at_a_time_tests_per_hour": tph_single,
            "batched_over_one_at_a_time": tph_batch / tph_single,
            "one_at_a_time_us_per_squaring": us1,
            "shape_batched": tuned_many, "shape_one_at_a_time": tuned_one,
            "cpu_reference_tests_per_hour": cpu["tests_per_hour"],
            "batched_over_cpu": tph_batch / cpu["tests_per_hour"], "cpu": cpu,
            "sample": "batched: all 4,096 candidates to their last verdict (wall clock); one at a time: 2,000 "
                      "squarings of one candidate alone scaled to n-1+19 squarings plus 1,500 for the Gerbicz "
                      "check; CPU: the reference algorithm on all host cores, truncated tests scaled"}


def run_gpu(args, world, rank, local, pgd):
    import prothlogic_gb300 as pg
    pg.set_device(local)
    k, n = workloads.large()
    a = pg.choose_base(k, n)
    K, W = args.steps, args.warmup
    peaks = measured_peaks()
    fp64_tflops = pg.measure_fp64_peak()
    lg = pg.pick_fft_len(k, n).bit_length() - 1
    pinned = os.environ.get("PROTH_SHAPE")  # e.g. to rerun a measured shape under ncu (its timings mislead the tuner)
    if pinned:
        shape = parse_shape(pinned, lg)
        pg.tune_set(pg.TUNE_ONE, shape)
        tune_rows = [dict(shape, us_per_step=0.0, valid=1, chosen=1, pinned=1)]
    else:
        # launch shape for one residue at this length: the tuner's three fastest on bare
        # chains, timed again on one verified interval of this workload (K blocks)
        tune_rows = pg.autotune_engine(k, n, base=a, blocks=K, block=SQ_PER_STEP, top=3, iters=400)

    eng = pg.Engine(k, n)
    M = eng.fft_len
    # warm-up: W blocks, each verified
    eng.set_gerbicz(SQ_PER_STEP, 0)
    eng.set_residue(a)
    for _ in range(W):
        eng.square(SQ_PER_STEP)

    # timed: K blocks of 1,000 squarings, verification of all K blocks in the last step
    eng.set_gerbicz(SQ_PER_STEP, K)
    eng.set_residue(a)
    pg.flush_l2()
    sampler = ClockSampler(local)
    launches0 = pg.launch_count()
    nvtx = None
    if os.environ.get("PROTH_NVTX") == "1":  # name the timed region for an ncu launch list (--nvtx-include timed/)
        import torch
        nvtx = torch.cuda.nvtx
    barrier(pgd)
    sampler.start()
    if nvtx:
        nvtx.range_push("timed")
    step_ms = []
    for _ in range(K):
        step_ms.append(eng.square_timed(SQ_PER_STEP))
        pg.flush_l2()  # untimed, between steps
    if nvtx:
        nvtx.range_pop()
    clocks = sampler.stop()
    launches = pg.launch_count() - launches0 - K  # minus the flush memsets (not counted anyway)
    total_ms = max_over_ranks(pgd, sum(step_ms))
    stats = eng.stats()
    res = eng.get_residue()
    max_err = eng.max_err()
    # per-kernel device times of one squaring, kernels launched one by one with
    # events around each (untimed; serialised like an ncu launch list, so the
    # shares compare with one)
    prof = [eng.profile_step() for _ in range(20)]
    chosen = [r for r in tune_rows if r["chosen"]][0]
    if len(prof[0]) == 5:
        names = ["k_first", "k_mid_fwd", "k_inner", "k_mid_inv", "k_last"]
    elif chosen["passes"] == 3:
        names = ["k_first", "k_block", "k_last"]  # middle passes fused in one cluster kernel
    else:
        names = ["k_first", "k_inner", "k_last"]
    per_k = [statistics.median(p[i] for p in prof) * 1e3 for i in range(len(names))]
    kernels_live = [{"kernel": nm, "us": t, "share": t / sum(per_k)} for nm, t in zip(names, per_k)]
    value = total_ms * 1e6 / (K * SQ_PER_STEP * world)

    # parity of the timed run: RES64 after K*1000 squarings of x0 = a (GMP values)
    parity = large_parity(k, a, K * SQ_PER_STEP, res)

    # e2e through the public API with host buffers: each step is one run of the
    # configuration (set the residue, 10,000 squarings with a Gerbicz check every
    # 1,000, read back the verified residue)
    eng.set_gerbicz(SQ_PER_STEP, 0)
    x = a
    barrier(pgd)
    t0 = time.perf_counter()
    for _ in range(K):
        eng.set_residue(x)
        eng.square(E2E_SQ_PER_STEP)
        x = eng.get_residue()
    e2e_s = max_over_ranks(pgd, time.perf_counter() - t0)
    e2e = e2e_s * 1e9 / (K * E2E_SQ_PER_STEP * world)
    parity_e2e = large_parity(k, a, K * E2E_SQ_PER_STEP, x)
    nl_in = (x.bit_length() + 63) // 64
    h2d = M * 4 + (M // 8) * 16 + 128          # digits, run carries, slot state
    d2h = M * 4 + 8 + 128                       # canonical digits, top digit, slot state

    # roofline: algorithmic bytes 32*E per squaring, E = ceil(W/8), W = n + bitlen(k)
    Wbits = n + k.bit_length()
    E = math.ceil(Wbits / 8)
    t_sq = value * 1e-9 * world
    bytes_alg = 32 * E
    hbm_peak = peaks.get("hbm_gbs")
    achieved_gbs = bytes_alg / t_sq / 1e9
    dp_ops = dp_ops_per_point(_chosen_radices(tune_rows)) * M
    dp_rate = dp_ops / t_sq / 1e12                 # T instr/s
    dp_peak = fp64_tflops / 2.0                    # DFMA instr/s from the live probe
    traffic, traffic_shape = profile_traffic()

    if rank != 0:
        eng.close()
        return 0
    eng.close()
    batched = batched_sample(pg) if os.environ.get("PROTH_BENCH_BATCH", "1") == "1" else None
    uneven = uneven_sample(pg) if os.environ.get("PROTH_BENCH_UNEVEN", "1") == "1" else None
    single = single_sample(pg) if os.environ.get("PROTH_BENCH_SINGLE", "1") == "1" else None
    shim = shim_sample(pg) if os.environ.get("PROTH_BENCH_SHIM", "1") == "1" else None
    serving = serving_sample(pg) if os.environ.get("PROTH_BENCH_SERVING", "1") == "1" else None
    cpu_ns, cpu_kind, cpu_used, cpu_L, cpu_fl = time_cpu_reference(k, n, cpu_sample_seconds())
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded candidate, no dataset)",
        "config": {"workload": "large: n=1048576, k odd in [3,2^20) seed 2, x0=a, Gerbicz block 1000",
                   "k": k, "n": n, "base_a": a, "fft_len": M, "squarings_per_step": SQ_PER_STEP,
                   "gerbicz": f"block {SQ_PER_STEP}, {K} blocks verified in the last step",
                   "l2": "flushed between steps (512 MiB write)", "parity_res64": parity,
                   "parity_res64_e2e": parity_e2e,
                   "gerbicz_checks": stats["gerbicz_checks"], "gerbicz_failures": stats["gerbicz_failures"],
                   "fft_bumps": stats["fft_bumps"], "max_err": max_err, "shape": _chosen(tune_rows),
                   "shape_candidates_fastest": _top_shapes(tune_rows),
                   "shape_candidates_columns": "shape, us per squaring in the tuner (bare chain), us per "
                                               "squaring on a verified interval of this workload"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak if hbm_peak else None, "traffic": traffic,
                     "kernels_live": kernels_live,
                     "note": f"measured hbm_gbs peak; unit = one squaring (its {len(names)} kernels); traffic "
                             f"= DRAM bytes of one squaring's launches under ncu (shape {traffic_shape}; cold caches; "
                             "L2-resident in steady state); the real bound is the FP64 pipe, see roofline_fp64"},
        "roofline_fp64": {"bound": "fp64", "achieved": dp_rate, "peak": dp_peak, "unit": "T DP instr/s",
                          "frac": dp_rate / dp_peak, "dp_instr_per_squaring": dp_ops,
                          "peak_source": "live DFMA probe (pg_measure_fp64_peak), of measured",
                          "flops_alg_per_squaring": 5 * E * math.log2(E),
                          "achieved_alg_tflops": 5 * E * math.log2(E) / t_sq / 1e12,
                          "fp64_peak_tflops": fp64_tflops},
        "cpu_baseline": {"value": cpu_ns, "unit": UNIT, "cores": 1, "kind": cpu_kind, "flags": cpu_fl,
                         "host_cores": os.cpu_count(),
                         "sample": f"{cpu_used} squarings at n=1048576, L={cpu_L}, one host thread (the "
                                   "reference's per-candidate engine is single-threaded)"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "note": "per step: set_residue (H2D) + 10,000 squarings with a Gerbicz check every 1,000 + "
                        "verified get_residue (D2H)"},
        "clocks": clocks,
        "gpu_launches": launches,
        "batched": batched,
        "batched_uneven": uneven,
        "single_test": single,
        "reference_api_loop": shim,
        "serving": serving,
    }
    line["results"] = compact_results(line)  # last key: the summary survives a truncated tail
    print(json.dumps(line), flush=True)
    return 0


def compact_results(line):
    """The figures of every configuration in a few hundred characters."""
    def r(x, nd=1):
        return None if x is None else round(x, nd)
    out = {"ns_per_squaring_n2^20": r(line["value"], 0), "e2e": r(line["e2e"]["value"], 0),
           "parity": line["config"]["parity_res64"], "parity_e2e": line["config"]["parity_res64_e2e"],
           "fp64_frac": r(line["roofline_fp64"]["frac"], 3),
           "cpu_ns_per_squaring": r(line["cpu_baseline"]["value"], 0)}
    st = line.get("single_test")
    if st:
        out["single_n32768"] = {"us_per_sq": r(st["us_per_squaring_gpu"], 2), "s_per_test": r(st["seconds_per_test_gpu"], 3),
                                "gpu_tph": r(st["gpu_tests_per_hour_one_at_a_time"], 0),
                                "cpu_tph_all_cores": r(st["cpu"]["tests_per_hour"], 0), "parity": st["parity_vs_reference"]}
    for key, name in (("batched", "batched_n65536"), ("batched_uneven", "uneven")):
        b = line.get(key)
        if b:
            out[name] = {"tph": r(b["batched_tests_per_hour"], 0), "one_at_a_time_tph": r(b["one_at_a_time_tests_per_hour"], 0),
                         "x_one_at_a_time": r(b["batched_over_one_at_a_time"], 2),
                         "cpu_tph": r(b["cpu_reference_tests_per_hour"], 0), "x_cpu": r(b["batched_over_cpu"], 2)}
            if "parity" in b:
                out[name]["parity"] = b["parity"]
    sh = line.get("reference_api_loop")
    if sh:
        out["reference_api_loop_us_per_sq"] = {k: r(v["us_per_squaring"], 1) for k, v in sh.items() if k != "note"}
        out["reference_api_loop_parity"] = sh["n=32768"].get("parity_vs_reference")
    sv = line.get("serving")
    if sv:
        out["serving"] = sv.get("summary")
    return out


def uneven_full():
    """The whole uneven workload (2,048 candidates, every class, autotuned shapes)
    through one batch to the last verdict; wall-clock tests/hour, a seeded subset
    of the verdicts checked against GMP."""
    import prothlogic_gb300 as pg
    cands = workloads.uneven(count=2048)
    lgs = sorted({pg.pick_fft_len(k, n).bit_length() - 1 for k, n in cands})
    for lg in lgs:
        members = sum(1 for k, n in cands if pg.pick_fft_len(k, n).bit_length() - 1 == lg)
        pg.autotune(lg, slots=min(members, 1024), iters=50)
    whole = whole_batch(pg, cands, 2048)
    print(json.dumps(dict(whole, workload="uneven: 2048 candidates, n log-uniform in [8192, 262144], "
                                          "k odd in [3,10^5) seed 4", classes=[f"2^{lg}" for lg in lgs])))
    return 0


def ncu_batch_target():
    """Small profiling target for the batched path: 256 candidates at n = 65536, 100 steps."""
    import prothlogic_gb300 as pg
    b = pg.Batch(256)
    for i, (k, n) in enumerate(workloads.uniform(count=256)):
        b.submit(k, n, i)
    b.run(100)
    print("pending", b.pending())
    b.close()
    return 0


def parse_shape(spec, lg):
    """'64x32x32,gm=2,gi=4,tpb=1,cl=8' (or '16x128,gi=8,res=16,rnt=128') -> a
    tune-result dict for 2^lg points."""
    parts = spec.split(",")
    radices = [int(x) for x in parts[0].split("x")]
    shape = {"lg": lg, "slots": 1, "passes": len(radices), "f0": radices[0], "f1": radices[1],
             "f2": radices[2] if len(radices) > 2 else 0, "g_mid": 2, "g_inner": 2, "tpb": 1, "cluster": 0,
             "resident": 0, "resident_threads": 0, "edge": 0}
    names = {"gm": "g_mid", "gi": "g_inner", "tpb": "tpb", "cl": "cluster", "res": "resident",
             "rnt": "resident_threads", "edge": "edge", "tpb0": "tpb_outer"}
    for kv in parts[1:]:
        key, val = kv.split("=")
        shape[names[key]] = int(val)
    return shape


def ncu_target(shape=None, k=None, n=None, squarings=200):
    """Small profiling target: one residue (default the n = 1,048,576
    configuration), `squarings` squarings, no Gerbicz; `shape` (see
    parse_shape) pins the launch shape."""
    import prothlogic_gb300 as pg
    if k is None or n is None:
        k, n = workloads.large()
    if shape:
        lg = pg.pick_fft_len(k, n).bit_length() - 1
        pg.tune_set(pg.TUNE_ONE, parse_shape(shape, lg))
    e = pg.Engine(k, n, flags=pg.FLAG_NO_GERBICZ)
    e.set_residue(5)
    e.square(squarings)
    print("res64 %016x" % (e.get_residue() & ((1 << 64) - 1)))
    e.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ncu-target", action="store_true", help="run only the small profiling target")
    ap.add_argument("--shape", default=None, help="launch shape of the profiling target, e.g. 64x32x32,gi=4,cl=8")
    ap.add_argument("--k", type=int, default=None, help="profiling target: k (with --n)")
    ap.add_argument("--n", type=int, default=None, help="profiling target: n (with --k)")
    ap.add_argument("--squarings", type=int, default=200, help="profiling target: squarings")
    ap.add_argument("--uneven-full", action="store_true", help="run the whole uneven batch to completion")
    ap.add_argument("--ncu-batch-target", action="store_true", help="run only the small batched profiling target")
    args = ap.parse_args()
    if args.ncu_target:
        return ncu_target(args.shape, args.k, args.n, args.squarings)
    if args.ncu_batch_target:
        return ncu_batch_target()
    if args.uneven_full:
        return uneven_full()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local, pgd = dist_setup()
    if args.impl == "reference":
        rc = run_reference(args, world, rank, pgd)
    else:
        rc = run_gpu(args, world, rank, local, pgd)
    if pgd is not None:
        pgd.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
