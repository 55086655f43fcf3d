"""GPU parity: the CUDA engine (through the C ABI) against the reference's own
golden vectors, GMP and the oracle.  Integer results must be bit-exact."""
import json
import os
import random

import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.json")
M64 = (1 << 64) - 1


@pytest.fixture(scope="module")
def pg():
    import prothlogic_gb300 as pgm
    pgm.load()
    return pgm


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def _N(k, n):
    return k * (1 << n) + 1


def test_device_is_gb300(pg):
    import ctypes
    name = ctypes.create_string_buffer(64)
    sm = ctypes.c_int()
    assert pg.load().pg_device_info(name, 64, ctypes.byref(sm)) == 0, name.value
    assert sm.value >= 100


@pytest.mark.parametrize("k,n", [(3, 2048), (843, 4096), (9999, 5000), (77, 8300), (524287, 20000),
                                 (5, 32700), (12345, 65536), (999999, 131072), (3, 270000), (77, 600000)])
@pytest.mark.parametrize("path", ["persistent", "per-pass"])
def test_steps_match_python(pg, k, n, path):
    N = _N(k, n)
    x = random.Random(n * 31 + k).randrange(N)
    flags = pg.FLAG_NO_GRAPH | (pg.FLAG_PERSIST if path == "persistent" else 0)
    with pg.Engine(k, n, flags=flags) as e:
        e.set_residue(x)
        assert e.get_residue() == x
        for i in range(10):
            e.square(1)
            x = x * x % N
            assert e.get_residue() == x, f"step {i}"
        assert e.max_err() < 0.4


def test_reference_traces(pg, gmp, golden):
    """RES64 after every squaring equals the reference engine's (corrected L)."""
    for t in golden["traces"]:
        k, n = t["k"], t["n"]
        with pg.Engine(k, n) as e:
            e.pow_small(t["a"], k)
            if n <= 70000:
                assert e.get_residue() == gmp.powmod(t["a"], k, _N(k, n))
            for i, want in enumerate(t["res64"]):
                e.square(1)
                got = e.get_residue()
                assert format(got & M64, "016x") == want, (k, n, i)


@pytest.mark.parametrize("n", [524288, 1 << 20, 2000000])
def test_persistent_equals_per_pass_at_full_size(pg, n):
    """Long chains at the large lengths: the cooperative kernel and the per-pass
    kernels give identical residues (and equal to Python at the smaller n)."""
    k = 878261
    res = []
    for flags in (pg.FLAG_PERSIST, 0):
        with pg.Engine(k, n, flags=flags | pg.FLAG_NO_GERBICZ) as e:
            e.set_residue(5)
            e.square(300)
            res.append(e.get_residue())
            assert e.max_err() < 0.4
    assert res[0] == res[1]
    if n <= 524288:
        assert res[0] == pow(5, 1 << 300, _N(k, n))


def test_reference_full_tests(pg, golden):
    for t in golden["tests"]:
        r = pg.proth_test(t["k"], t["n"])
        assert r["status"] == 0
        assert r["verdict"] == t["verdict"], t
        assert r["base"] == t["base"], t
        assert format(r["res64"], "016x") == t["res64"], t


def test_known_answers(pg, golden):
    """843*2^120002+1 prime (a=5), 853 and 895 composite -- RES64 equal to the reference's."""
    for t in golden["known"]:
        r = pg.proth_test(t["k"], t["n"])
        assert (r["verdict"], r["base"], format(r["res64"], "016x")) == (t["verdict"], t["base"], t["res64"])
    assert pg.execute_proth_test_fft(843, 120002) is True


def test_large_configuration_residues(pg, golden):
    """n = 2^20: x0 = a, RES64 after every 1,000 of 10,000 squarings (GMP values)."""
    g = golden["large"]
    with pg.Engine(g["k"], g["n"]) as e:
        assert e.fft_len == 65536
        e.set_residue(g["a"])
        for i, want in enumerate(g["res64"]):
            e.square(g["every"])
            assert format(e.get_residue() & M64, "016x") == want, i
        assert e.max_err() < 0.4


def test_gmp_full_tests_batched(pg, golden):
    b = pg.Batch(16)
    for i, t in enumerate(golden["gmp_tests"]):
        b.submit(t["k"], t["n"], i)
    b.run(0)
    res = {r["tag"]: r for r in b.poll()}
    assert len(res) == len(golden["gmp_tests"])
    for i, t in enumerate(golden["gmp_tests"]):
        r = res[i]
        assert (r["verdict"], r["base"], format(r["res64"], "016x")) == (t["verdict"], t["base"], t["res64"]), t
    b.close()


def _config_sample(cands, count, seed):
    """A seeded sample of a configuration: mostly candidates past the small-prime
    gate, plus a few gated ones (answered at submission)."""
    rng = random.Random(seed)
    passing = [c for c in cands if not _gated(*c)]
    gated = [c for c in cands if _gated(*c)]
    return rng.sample(passing, count - 4) + rng.sample(gated, 4)


def _gated(k, n):
    from tests import _gmp
    return any(k % p and pow(2, n, p) == (-pow(k, -1, p)) % p for p in _gmp.GATE_PRIMES)


@pytest.mark.parametrize("config", ["uniform", "uneven"])
def test_batch_config_sample_vs_gmp(pg, gmp, config):
    """Per-candidate parity at configuration scale: a seeded 64-candidate sample of
    the 4,096-candidate uniform workload (n = 65,536, k < 10^6) or of the
    2,048-candidate uneven one (n log-uniform in [8,192, 262,144]) through one
    Gerbicz-checked batch; every verdict, base and RES64 equals GMP's."""
    from prothlogic_gb300 import workloads
    cands = workloads.uniform(count=4096) if config == "uniform" else workloads.uneven(count=2048)
    sample = _config_sample(cands, 64, seed=7 if config == "uniform" else 8)
    want = gmp.proth_tests(sample)  # spawned processes, beside this process's CUDA context
    b = pg.Batch(64)
    for i, (k, n) in enumerate(sample):
        b.submit(k, n, i)
    b.run(0)
    got = {r["tag"]: r for r in b.poll()}
    b.close()
    assert len(got) == len(sample)
    for i, (k, n) in enumerate(sample):
        r = got[i]
        assert r["status"] == 0, (k, n, r)
        assert (r["verdict"], r["base"], r["res64"]) == want[i], (k, n)


def test_batch_equals_single(pg, oracle):
    rng = random.Random(17)
    cands = [(2 * rng.randrange(1, 5000) + 1, rng.randrange(2048, 9000)) for _ in range(60)]
    b = pg.Batch(24)
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(0)
    res = {r["tag"]: r for r in b.poll()}
    assert len(res) == len(cands)
    for i, (k, n) in enumerate(cands[:12]):
        s = pg.proth_test(k, n)
        assert (res[i]["verdict"], res[i]["res64"], res[i]["base"]) == (s["verdict"], s["res64"], s["base"])
    for i, (k, n) in enumerate(cands):
        o = oracle.proth_test(k, n)
        assert (res[i]["verdict"], res[i]["res64"], res[i]["base"]) == (o["verdict"], o["res64"], o["base"]), (k, n)
    b.close()


def test_pow_small(pg):
    for k, n, a in [(843, 4096, 5), (999999, 65536, 3), (3, 2500, 37)]:
        N = _N(k, n)
        with pg.Engine(k, n) as e:
            e.pow_small(a, k)
            assert e.get_residue() == pow(a, k, N)
            e.pow_small(a, 1)
            assert e.get_residue() == a


def test_checkpoint_roundtrip(pg, tmp_path):
    k, n = 9999, 32768
    N = _N(k, n)
    path = str(tmp_path / "check.bin")
    with pg.Engine(k, n) as e:
        e.set_residue(7)
        e.square(500)
        e.checkpoint_save(path, 499)
        e.square(300)
        want = e.get_residue()
    assert want == pow(7, 1 << 800, N)
    with open(path, "rb") as f:
        raw = f.read()
    import struct
    ci, nl = struct.unpack("<QQ", raw[:16])
    assert ci == 499 and nl >= (n + 64) // 64
    x = int.from_bytes(raw[16:16 + 8 * nl], "little")
    assert x == pow(7, 1 << 500, N)
    with pg.Engine(k, n) as e2:
        assert e2.checkpoint_load(path) == 499
        e2.square(300)
        assert e2.get_residue() == want


def test_roundoff_bump_recovers(pg):
    """A forced, far too small FFT length overflows the rounding range; the
    engine rolls back, grows the length and still returns the exact residue."""
    k, n = 999999, 49100  # 24 bits per digit at length 2048: products leave FP64's exact range
    N = _N(k, n)
    with pg.Engine(k, n, fft_len_hint=2048, flags=pg.FLAG_FORCE_LEN) as e:
        assert e.fft_len == 2048
        e.set_residue(5)
        e.square(50)
        assert e.get_residue() == pow(5, 1 << 50, N)
        assert e.stats()["fft_bumps"] >= 1
        assert e.fft_len > 2048


def test_digit_width_limits(pg):
    with pytest.raises(pg.ProthGpuError):
        pg.Engine(3, 65536, fft_len_hint=1024, flags=pg.FLAG_FORCE_LEN)  # 64-bit digits
    with pytest.raises(pg.ProthGpuError):
        pg.Engine(3, 1000)  # below 6 bits per digit at the smallest length


def test_roundoff_without_bump_reports(pg):
    with pg.Engine(999999, 49100, fft_len_hint=2048, flags=pg.FLAG_FORCE_LEN | pg.FLAG_NO_BUMP) as e:
        e.set_residue(5)
        with pytest.raises(pg.ProthGpuError) as ei:
            e.square(20)
        assert ei.value.status == pg.PG_EROUNDOFF


@pytest.mark.parametrize("flags", [0, "nograph"])
def test_gerbicz_concurrent_verification(pg, gmp, flags):
    """The verification chain squares beside the residue in the last block of
    each interval; the result and the counters must be right on every path."""
    f = {0: 0, "nograph": pg.FLAG_NO_GRAPH}[flags]
    k, n = 878261, 1 << 20
    N = _N(k, n)
    with pg.Engine(k, n, flags=f) as e:
        e.set_gerbicz(100, 3)
        e.set_residue(5)
        e.square(700)
        assert e.stats()["gerbicz_checks"] >= 2 and e.stats()["gerbicz_failures"] == 0
        assert e.get_residue() == gmp.square_chain(5, 700, N, every=700)[0]


def test_gerbicz_clean_run(pg):
    k, n = 12345, 65536
    N = _N(k, n)
    with pg.Engine(k, n) as e:
        e.set_gerbicz(100, 4)
        e.set_residue(11)
        e.square(1000)
        st = e.stats()
        assert st["gerbicz_checks"] >= 2 and st["gerbicz_failures"] == 0
        assert e.get_residue() == pow(11, 1 << 1000, N)


@pytest.mark.parametrize("when", [30, 250, 399])
def test_gerbicz_detects_and_recovers_corruption(pg, when):
    """A silent error in a residue digit (injected on the device, nothing
    faults) is caught by the Gerbicz check; the engine rolls back and the
    returned residue is exact."""
    k, n = 999, 32768
    N = _N(k, n)
    with pg.Engine(k, n) as e:
        e.set_gerbicz(100, 3)
        e.set_residue(3)
        e.square(when)
        e.debug_corrupt(777, 5)
        e.square(600 - when)
        assert e.get_residue() == pow(3, 1 << 600, N)
        assert e.stats()["gerbicz_failures"] >= 1


def test_gerbicz_partial_block_corruption(pg):
    k, n = 999, 32768
    N = _N(k, n)
    with pg.Engine(k, n) as e:
        e.set_gerbicz(1000, 0)
        e.set_residue(3)
        e.square(120)
        e.debug_corrupt(5, -3)
        e.square(10)
        assert e.get_residue() == pow(3, 1 << 130, N)
        assert e.stats()["gerbicz_failures"] >= 1


def test_no_gerbicz_flag_skips_checks(pg):
    k, n = 999, 32768
    with pg.Engine(k, n, flags=pg.FLAG_NO_GERBICZ) as e:
        e.set_residue(3)
        e.square(300)
        assert e.get_residue() == pow(3, 1 << 300, _N(k, n))
        assert e.stats()["gerbicz_checks"] == 0


def test_reference_api_shim_is_a_drop_in(pg, gmp, golden):
    """A caller written only against the reference's fft_init / fft_square_karatsuba /
    fft_destroy (prothlogic4.2/fft_engine.h) reproduces the reference's RES64 trace."""
    import subprocess
    from prothlogic_gb300 import build as b
    drv = b.COMPAT_DRIVER
    assert os.path.exists(drv)
    for t in golden["traces"]:
        if t["n"] not in (32768, 65536):
            continue
        N = _N(t["k"], t["n"])
        x0 = gmp.powmod(t["a"], t["k"], N)
        steps = 60
        out = subprocess.run([drv, str(t["k"]), str(t["n"]), str(t["L"]), str(steps)], input=format(x0, "x"),
                             capture_output=True, text=True, check=True).stdout.split("\n")
        got = [ln.split()[1] for ln in out if ln.strip()]
        assert got == t["res64"][:steps], (t["k"], t["n"])


def _drive(args, stdin=""):
    import subprocess
    from prothlogic_gb300 import build as b
    return subprocess.run([b.COMPAT_DRIVER] + [str(a) for a in args], input=stdin, capture_output=True, text=True,
                          check=True).stdout


@pytest.mark.parametrize("k,n", [(9505, 32768), (843, 120002)])
def test_reference_autotune_through_shim(pg, k, n):
    """auto_tune_fft_len's probe (dcore.cpp:20-81: all-ones residue of (n+63)/64
    limbs, one limb short of a residue mod N, 100 squarings) gets the engine's real
    roundoff error through the shim and accepts its first length, as the
    reference engine does at these n (Run test:31: 0.00195 at n = 120002)."""
    out = _drive(["autotune", n, k]).split("\n")
    probes = [ln.split() for ln in out if ln.startswith("PROBE")]
    L = int([ln for ln in out if ln.startswith("L ")][0].split()[1])
    first = 256
    while n / first > 18.0:
        first *= 2
    assert len(probes) == 1 and int(probes[0][1]) == first == L
    assert 0.0 < float(probes[0][2]) < 0.30


def test_reference_loop_through_shim(pg, golden):
    """The squaring loop of execute_proth_test_fft (proth_logic.cpp:442-552), one
    fft_square_karatsuba per step on L/4 limbs at the autotuned L, through the
    shim: verdicts and RES64 of the reference's own golden tests (n = 32,768,
    2,049, 4,096; at n = 4,096 the L/4 limbs are one short of a residue mod N, so
    the caller's copy is truncated as the reference engine truncates it) and of its
    console log's known prime 843*2^120002+1 (a = 5, Run test:41)."""
    cases = [t for t in golden["tests"] if not t["gated"] and t["base"]]  # n = 32768, 2049, 4096
    cases += [t for t in golden["known"] if t["k"] == 843]
    assert len(cases) == 4
    for t in cases:
        k, n = t["k"], t["n"]
        L = 256
        while n / L > 18.0:
            L *= 2
        x0 = pow(t["base"], k, _N(k, n))
        res = _drive(["test", k, n, L], format(x0, "x")).split()
        assert res[0] == "RESULT"
        verdict, res64, steps, err = int(res[1]), res[2], int(res[3]), float(res[5])
        assert steps == n - 1
        assert (verdict, res64) == (t["verdict"], t["res64"]), (k, n)
        assert err < 0.4


def test_resume_from_reference_checkpoint(pg, golden, tmp_path):
    """A checkpoint file written by the reference's own save_checkpoint loads into
    the engine; resuming gives the GMP residue, and the engine's file keeps the
    reference layout."""
    import shutil
    import struct
    c = golden["ref_checkpoint"]
    src = os.path.join(os.path.dirname(GOLDEN), c["file"])
    path = str(tmp_path / "check.bin")
    shutil.copy(src, path)
    with pg.Engine(c["k"], c["n"]) as e:
        assert e.checkpoint_load(path) == c["current_i"]
        e.square(300)
        assert format(e.get_residue() & M64, "016x") == c["res64_after_300_more"]
        e.checkpoint_save(path, c["current_i"] + 300)
    raw = open(path, "rb").read()
    ci, nl = struct.unpack("<QQ", raw[:16])
    assert ci == c["current_i"] + 300 and nl == c["L"] // 4


def test_prefilter_matches_trial_division(pg, oracle):
    """GPU sieve + Montgomery trial division equals plain trial division."""
    rng = random.Random(9)
    cands = [(2 * rng.randrange(1, 50000) + 1, rng.randrange(2048, 300000)) for _ in range(60)]
    cands += [(3, 2048), (9999, 32768), (843, 120002), (5, 4096)]
    bound = 1 << 22
    got = pg.prefilter(cands, bound=bound)
    for (k, n), f in zip(cands, got):
        assert f == oracle.lib().ora_smallest_factor(k, n, bound), (k, n)
        if f:
            assert (k * pow(2, n, f) + 1) % f == 0
    assert got[-2] == 0  # 843*2^120002+1 is prime


def test_prefilter_full_bound(pg):
    """Primes up to 2^32: the gate primes are found, and a known prime passes."""
    cands = [(843, 120002), (3, 2048), (1275, 4399)]
    got = pg.prefilter(cands, bound=1 << 32)
    assert got[0] == 0 and got[1] == 19
    for (k, n), f in zip(cands, got):
        if f:
            assert (k * pow(2, n, f) + 1) % f == 0


def test_batch_hbm_budget_admission(pg):
    """Admission by device footprint: with room for two candidates at a time,
    six still all finish, exactly."""
    cands = [(2 * i + 3, 4096 + 37 * i) for i in range(6)]
    fp = pg.slot_footprint(*cands[0])
    b = pg.Batch(8)
    b.set_budget(int(2.5 * fp))
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(50)
    q, r, f = b.pending()
    assert r <= 2
    b.run(0)
    res = {x["tag"]: x for x in b.poll()}
    assert len(res) == 6
    for i, (k, n) in enumerate(cands):
        N = _N(k, n)
        a = res[i]["base"]
        if a:
            y = pow(a, (N - 1) // 2, N)
            assert res[i]["res64"] == y & M64 and res[i]["verdict"] == (y == N - 1)
    b.close()


def test_batch_resumes_from_device_checkpoint(pg, oracle):
    """A candidate whose digits are corrupted after its 10,000-squaring device
    checkpoint fails its range check and resumes from that checkpoint, one FFT
    length up; its verdict and RES64 stay exact."""
    cands = [(1275, 15013), (99, 15501), (105, 15500)]
    assert not any(pg.gate_rejects(k, n) for k, n in cands)  # all three must run
    b = pg.Batch(4)
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(12000)
    b.debug_corrupt(1, 100, 1 << 30)  # pushes a digit out of its range: the next squaring flags it
    b.run(0)
    res = {x["tag"]: x for x in b.poll()}
    assert len(res) == 3
    assert res[1]["fft_bumps"] >= 1
    for i, (k, n) in enumerate(cands):
        o = oracle.proth_test(k, n)
        assert (res[i]["verdict"], res[i]["res64"], res[i]["base"]) == (o["verdict"], o["res64"], o["base"])
    b.close()


def test_serving_loop_small(pg):
    from prothlogic_gb300 import serve
    arrivals = [(0.05 * i, 2 * (37 * i % 4000) + 3, 6000 + 211 * i) for i in range(16)]
    recs, s = serve.serve(arrivals, budget_bytes=1 << 30, max_slots=64, prefilter_bound=1 << 24)
    assert s["completed"] == 16 and s["errors"] == 0
    assert s["p50_s"] is not None and s["p99_s"] >= s["p50_s"]
    for r in recs:
        N = _N(r["k"], r["n"])
        if r["tested"]:
            a = pg.choose_base(r["k"], r["n"])
            if a:
                y = pow(a, (N - 1) // 2, N)
                assert r["res64"] == y & M64
        else:
            assert N % r["factor"] == 0


def _passing(seed, count, lo, hi, pg):
    rng = random.Random(seed)
    out = []
    while len(out) < count:
        k, n = 2 * rng.randrange(1, 5000) + 1, rng.randrange(lo, hi)
        if not pg.gate_rejects(k, n) and pg.choose_base(k, n):
            out.append((k, n))
    return out


def test_batch_gerbicz_clean_run(pg, gmp):
    """Every batched candidate is Gerbicz-verified once at the end of its chain,
    with no failure, and its residue is exact."""
    cands = _passing(77, 4, 5200, 9000, pg)
    b = pg.Batch(8)
    b.set_gerbicz(1000)
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(0)
    res = {r["tag"]: r for r in b.poll()}
    assert len(res) == len(cands)
    for i, (k, n) in enumerate(cands):
        N = _N(k, n)
        y = gmp.powmod(res[i]["base"], (N - 1) // 2, N)
        assert res[i]["status"] == 0
        assert res[i]["res64"] == y & M64 and res[i]["verdict"] == (y == N - 1)
        assert res[i]["gerbicz_checks"] == 1 and res[i]["gerbicz_failures"] == 0
    b.close()


def test_batch_gerbicz_detects_corruption(pg, gmp):
    """A digit changed by +1 stays inside its range, so only the Gerbicz check
    can see it: the candidate fails its verification, goes back to its last
    verified residue and still ends exact; the others are untouched."""
    cands = _passing(78, 3, 7000, 9000, pg)
    b = pg.Batch(4)
    b.set_gerbicz(1000)
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(3500)
    b.debug_corrupt(1, 37, 1)
    b.run(0)
    res = {r["tag"]: r for r in b.poll()}
    assert len(res) == len(cands)
    assert res[1]["gerbicz_failures"] >= 1 and res[1]["gerbicz_checks"] >= 2
    for i, (k, n) in enumerate(cands):
        N = _N(k, n)
        y = gmp.powmod(res[i]["base"], (N - 1) // 2, N)
        assert res[i]["status"] == 0
        assert res[i]["res64"] == y & M64 and res[i]["verdict"] == (y == N - 1), i
        if i != 1:
            assert res[i]["gerbicz_failures"] == 0
    b.close()


def test_batch_without_gerbicz_flag(pg, gmp):
    cands = _passing(79, 3, 3000, 4000, pg)
    b = pg.Batch(4, flags=pg.FLAG_NO_GERBICZ)
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(0)
    res = {r["tag"]: r for r in b.poll()}
    for i, (k, n) in enumerate(cands):
        N = _N(k, n)
        y = gmp.powmod(res[i]["base"], (N - 1) // 2, N)
        assert res[i]["res64"] == y & M64 and res[i]["gerbicz_checks"] == 0
    b.close()


def test_largest_length_vs_gmp(pg, gmp):
    """2^19 points, the length of the reference console's largest candidate
    199971*2^5435752+1: squarings from a random residue equal GMP's."""
    k, n = 199971, 5435752
    N = _N(k, n)
    x = random.Random(19).randrange(N)
    want = gmp.square_chain(x, 100, N, every=50)
    with pg.Engine(k, n) as e:
        assert e.fft_len == 1 << 19
        e.set_residue(x)
        for w in want:
            e.square(50)
            assert e.get_residue() == w
        assert e.max_err() < 0.4
