"""Launch-shape autotuner: every compiled shape must give the same residues as
GMP, the tuner must pick one, and engines / batches built after tuning must
stay bit-exact under the tuned shape."""
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
    pgm.tune_clear()
    yield pgm
    pgm.tune_clear()  # later tests use the default shapes


def test_autotune_one_residue_picks_a_valid_shape(pg):
    rows = pg.autotune(12, slots=1, iters=50)
    assert len(rows) >= 3
    assert all(r["valid"] == 1 for r in rows), rows  # all shapes bit-identical
    chosen = [r for r in rows if r["chosen"]]
    assert len(chosen) == 1
    assert chosen[0]["us_per_step"] == min(r["us_per_step"] for r in rows)
    got = pg.tune_get(12, pg.TUNE_ONE)
    assert (got["f0"], got["f1"], got["g_inner"]) == (chosen[0]["f0"], chosen[0]["f1"], chosen[0]["g_inner"])


@pytest.mark.parametrize("k,n", [(3, 60000), (999, 250000), (1000003, 400000), (878261, 1048576),
                                 (999999, 1500000), (199971, 5435752)])
def test_every_shape_is_exact_against_gmp(pg, gmp, k, n):
    """Each compiled shape at the length of (k, n), set by hand, squares a random
    residue 60 times exactly."""
    lg = pg.pick_fft_len(k, n).bit_length() - 1
    rows = pg.autotune(lg, slots=1, iters=50)
    N = k * (1 << n) + 1
    x = random.Random(lg).randrange(N)
    want = gmp.square_chain(x, 60, N, every=60)[0]
    for r in rows:
        pg.tune_set(pg.TUNE_ONE, r)
        with pg.Engine(k, n, flags=pg.FLAG_NO_GERBICZ) as e:
            e.set_residue(x)
            e.square(60)
            assert e.get_residue() == want, r
    pg.tune_clear()


def test_tuned_engine_matches_large_configuration(pg):
    """n = 2^20 under the shape the tuner picks: RES64 after 1,000 and 2,000
    squarings equal the GMP values."""
    with open(GOLDEN) as f:
        g = json.load(f)["large"]
    pg.autotune(16, slots=1, iters=100)
    assert pg.tune_get(16, pg.TUNE_ONE) is not None
    with pg.Engine(g["k"], g["n"]) as e:
        e.set_residue(g["a"])
        for i in range(2):
            e.square(g["every"])
            assert format(e.get_residue() & M64, "016x") == g["res64"][i], i
    pg.tune_clear()


@pytest.mark.parametrize("cluster,tpb", [(4, 1), (8, 1), (16, 1), (8, 2), (16, 2)])
def test_fused_middle_exact_with_gerbicz(pg, cluster, tpb):
    """n = 2^20 with the three middle passes of each squaring in one cluster
    kernel (shape set by hand) and the Gerbicz check on, whose products still run
    the three-kernel middle: RES64 after 1,000 and 2,000 squarings equal the GMP
    values, and a squaring is three kernels."""
    with open(GOLDEN) as f:
        g = json.load(f)["large"]
    pg.tune_set(pg.TUNE_ONE, {"lg": 16, "slots": 1, "passes": 3, "f0": 16, "f1": 64, "f2": 64,
                              "g_mid": 2, "g_inner": 2, "tpb": tpb, "cluster": cluster})
    try:
        with pg.Engine(g["k"], g["n"]) as e:
            e.set_residue(g["a"])
            for i in range(2):
                e.square(g["every"])
                assert format(e.get_residue() & M64, "016x") == g["res64"][i], i
            assert e.stats()["gerbicz_checks"] >= 2
            _, kernels = e.time_squarings(50)
            assert kernels == 3
    finally:
        pg.tune_clear()


@pytest.mark.parametrize("when", [30, 250])
def test_fused_middle_gerbicz_recovers_corruption(pg, gmp, when):
    """A digit corrupted on the device between squarings of the fused-middle
    shape (2^15 points, 32*32*32, clusters of 8) is caught by the Gerbicz check;
    the rollback and the squarings redone through the cluster kernel give the
    exact residue."""
    k, n = 1000003, 400000
    lg = pg.pick_fft_len(k, n).bit_length() - 1
    assert lg == 15
    N = k * (1 << n) + 1
    pg.tune_set(pg.TUNE_ONE, {"lg": lg, "slots": 1, "passes": 3, "f0": 32, "f1": 32, "f2": 32, "g_mid": 2,
                              "g_inner": 4, "tpb": 1, "cluster": 8})
    try:
        with pg.Engine(k, n) as e:
            e.set_gerbicz(100, 3)
            e.set_residue(3)
            e.square(when)
            e.debug_corrupt(777, 5)
            e.square(600 - when)
            assert e.get_residue() == gmp.square_chain(3, 600, N, every=600)[0]
            assert e.stats()["gerbicz_failures"] >= 1
        with pg.Engine(k, n) as e:
            e.set_residue(3)
            assert e.time_squarings(50)[1] == 3  # the cluster kernel was in use
    finally:
        pg.tune_clear()


def test_autotune_engine_picks_on_a_verified_interval(pg, gmp):
    """autotune_engine times the tuner's fastest shapes on a Gerbicz-checked run
    of the candidate itself, installs the fastest there, and engines under it are
    exact."""
    k, n = 1000003, 400000  # 2^15 points
    rows = pg.autotune_engine(k, n, blocks=2, block=200, top=2, iters=100)
    timed = [r for r in rows if "us_in_situ" in r]
    chosen = [r for r in rows if r["chosen"]]
    assert len(timed) == 2 and len(chosen) == 1
    assert chosen[0]["us_in_situ"] == min(r["us_in_situ"] for r in timed)
    got = pg.tune_get(15, pg.TUNE_ONE)
    keys = ("passes", "f0", "f1", "f2", "g_mid", "g_inner", "tpb", "tpb_outer", "cluster")
    assert tuple(got[f] for f in keys) == tuple(chosen[0][f] for f in keys)
    N = k * (1 << n) + 1
    with pg.Engine(k, n) as e:
        e.set_residue(3)
        e.square(300)
        assert e.get_residue() == gmp.square_chain(3, 300, N, every=300)[0]
    pg.tune_clear()


def test_tuned_batch_full_tests_exact(pg, gmp):
    rows = pg.autotune(12, slots=64, iters=50)
    assert any(r["chosen"] for r in rows) and all(r["valid"] for r in rows)
    rng = random.Random(12)
    cands = [(2 * rng.randrange(1, 500000) + 1, 65536) for _ in range(6)]
    b = pg.Batch(16)
    for i, (k, n) in enumerate(cands):
        b.submit(k, n, i)
    b.run(0)
    res = {r["tag"]: r for r in b.poll()}
    assert len(res) == len(cands)
    for i, (k, n) in enumerate(cands):
        N = k * (1 << n) + 1
        a = res[i]["base"]
        if a:
            y = gmp.powmod(a, (N - 1) // 2, N)
            assert res[i]["res64"] == y & M64 and res[i]["verdict"] == (y == N - 1)
    b.close()
    pg.tune_clear()


def test_tune_set_rejects_shapes_that_are_not_compiled(pg):
    bad = {"lg": 12, "slots": 1, "passes": 2, "f0": 16, "f1": 256, "f2": 0, "g_mid": 2, "g_inner": 2, "tpb": 1}
    with pytest.raises(pg.ProthGpuError):
        pg.tune_set(pg.TUNE_ONE, bad)


# k_resident instances (radices, CTAs per residue, threads per CTA) for lone residues
RESIDENT_LONE = [(9, 16, 32, 4, 128), (10, 32, 32, 4, 256), (10, 32, 32, 4, 128), (10, 16, 64, 8, 128),
                 (11, 16, 128, 16, 128), (11, 16, 128, 16, 64), (11, 32, 64, 8, 256), (11, 32, 64, 8, 128),
                 (12, 32, 128, 16, 256), (12, 32, 128, 16, 128), (13, 64, 128, 16, 512), (13, 64, 128, 16, 256),
                 (14, 128, 128, 16, 1024), (14, 128, 128, 16, 512), (14, 128, 128, 16, 256)]
# an n at each length (k = 9505): the FFT length the engine picks for it is 2^lg
RESIDENT_N = {9: 8000, 10: 16000, 11: 32768, 12: 60000, 13: 120000, 14: 250000}


def _resident_shape(lg, f0, f1, cl, nt):
    # the per-pass kernels of the shape (Gerbicz products) need an inner kernel instance
    return {"lg": lg, "slots": 1, "passes": 2, "f0": f0, "f1": f1, "f2": 0, "g_mid": 2,
            "g_inner": 4 if f1 == 32 else 2, "tpb": 1, "cluster": 0, "resident": cl, "resident_threads": nt}


@pytest.mark.parametrize("lg,f0,f1,cl,nt", RESIDENT_LONE)
def test_resident_lone_residue_exact(pg, gmp, lg, f0, f1, cl, nt):
    """A lone residue held in the shared memory of a cluster of CTAs (k_resident):
    exact after single squarings (one launch each), after a chain of 300 (one
    launch), and through the a^k powering (small-multiplier schedule) and the
    Gerbicz-checked chain whose products run on the per-pass kernels."""
    k, n = 9505, RESIDENT_N[lg]
    assert pg.pick_fft_len(k, n) == 1 << lg
    pg.tune_set(pg.TUNE_ONE, _resident_shape(lg, f0, f1, cl, nt))
    try:
        N = k * (1 << n) + 1
        x = random.Random(lg * 100 + cl + nt).randrange(N)
        with pg.Engine(k, n, flags=pg.FLAG_NO_GERBICZ) as e:
            e.set_residue(x)
            for i in range(4):
                e.square(1)
                x = x * x % N
                assert e.get_residue() == x, i
            e.square(300)
            assert e.get_residue() == gmp.square_chain_proth(x, 300, k, n, every=300)[0]
        with pg.Engine(k, n) as e:
            e.pow_small(3, k)
            assert e.get_residue() == pow(3, k, N)
            e.square(2500)
            assert e.get_residue() == gmp.square_chain_proth(pow(3, k, N), 2500, k, n, every=2500)[0]
            assert e.stats()["gerbicz_checks"] >= 1
    finally:
        pg.tune_clear()


def test_resident_whole_test_matches_reference(pg):
    """The reference's own golden test at n = 32,768 (k = 9,505, base 3) with its
    squarings resident in a 16-CTA cluster: verdict and RES64 unchanged."""
    with open(GOLDEN) as f:
        t = [t for t in json.load(f)["tests"] if (t["k"], t["n"]) == (9505, 32768)][0]
    pg.tune_set(pg.TUNE_ONE, _resident_shape(11, 16, 128, 16, 128))
    try:
        r = pg.proth_test(9505, 32768)
        assert (r["verdict"], r["base"], format(r["res64"], "016x")) == (t["verdict"], t["base"], t["res64"])
    finally:
        pg.tune_clear()


@pytest.mark.parametrize("lg,f0,f1,cl,nt,n,count", [(12, 64, 64, 1, 256, 65536, 24), (12, 64, 64, 1, 1024, 65536, 24),
                                                     (11, 32, 64, 1, 256, 30000, 24), (13, 64, 128, 2, 512, 120000, 16),
                                                     (14, 128, 128, 4, 512, 170000, 6)])
def test_resident_batch_exact(pg, gmp, lg, f0, f1, cl, nt, n, count):
    """Batch residues on k_resident (one CTA each, or two or four): seeded
    candidates to verdict through a Gerbicz-checked batch, equal to GMP."""
    from prothlogic_gb300 import workloads
    pg.tune_set(pg.TUNE_MANY, {"lg": lg, "slots": 2, "passes": 2, "f0": f0, "f1": f1, "f2": 0, "g_mid": 2,
                               "g_inner": 2, "tpb": 1, "cluster": 0, "resident": cl, "resident_threads": nt})
    try:
        rng = random.Random(nt + lg)
        if n == 65536:
            cands = rng.sample(workloads.uniform(count=4096), count)
        else:
            cands = [(2 * rng.randrange(1, 50000) + 1, n) for _ in range(count)]
        assert all(pg.pick_fft_len(k, nn) == 1 << lg for k, nn in cands)
        want = gmp.proth_tests(cands)
        b = pg.Batch(count)
        for i, (k, nn) in enumerate(cands):
            b.submit(k, nn, i)
        b.run(0)
        got = {r["tag"]: r for r in b.poll()}
        b.close()
        for i in range(len(cands)):
            assert got[i]["status"] == 0
            assert (got[i]["verdict"], got[i]["base"], got[i]["res64"]) == want[i], cands[i]
    finally:
        pg.tune_clear()


@pytest.mark.parametrize("shape", [
    {"passes": 3, "f0": 64, "f1": 32, "f2": 32, "g_mid": 2, "g_inner": 4, "tpb": 1, "cluster": 8},
    {"passes": 3, "f0": 16, "f1": 64, "f2": 64, "g_mid": 2, "g_inner": 2, "tpb": 2, "cluster": 0},
    {"passes": 3, "f0": 16, "f1": 64, "f2": 64, "g_mid": 2, "g_inner": 2, "tpb": 1, "cluster": 8, "tpb_outer": 2},
])
def test_edge_fused_chain_matches_large_configuration(pg, shape):
    """n = 2^20 with the last pass of every squaring and the first pass of the next
    in one kernel (k_edge, carry hand-over through release/acquire flags), the
    Gerbicz check on (graph-replayed chains, the check chain on a second stream,
    products on the plain kernels): RES64 after 1,000 and 2,000 squarings equal
    the GMP values."""
    with open(GOLDEN) as f:
        g = json.load(f)["large"]
    pg.tune_set(pg.TUNE_ONE, dict(shape, lg=16, slots=1, edge=1))
    try:
        with pg.Engine(g["k"], g["n"]) as e:
            e.set_residue(g["a"])
            for i in range(2):
                e.square(g["every"])
                assert format(e.get_residue() & M64, "016x") == g["res64"][i], i
            assert e.stats()["gerbicz_failures"] == 0
    finally:
        pg.tune_clear()


@pytest.mark.parametrize("lg,k,n,f0,f1,tpb", [(11, 9505, 32768, 32, 64, 4), (12, 77, 60000, 64, 64, 1),
                                             (13, 3, 130000, 64, 128, 2)])
def test_edge_fused_chain_steps_exact(pg, gmp, lg, k, n, f0, f1, tpb):
    """Two-pass lengths with k_edge: exact after single squarings (a chain of one
    has no fused pass), after chains of 7 and 130 (fused passes, graph replay and
    a remainder), and across a rollback-free Gerbicz run."""
    assert pg.pick_fft_len(k, n) == 1 << lg
    pg.tune_set(pg.TUNE_ONE, {"lg": lg, "slots": 1, "passes": 2, "f0": f0, "f1": f1, "f2": 0, "g_mid": 2,
                              "g_inner": 2, "tpb": tpb, "cluster": 0, "edge": 1})
    try:
        N = k * (1 << n) + 1
        x = random.Random(lg).randrange(N)
        with pg.Engine(k, n, flags=pg.FLAG_NO_GERBICZ) as e:
            e.set_residue(x)
            e.square(1)
            x = x * x % N
            assert e.get_residue() == x
            for c in (7, 130):
                e.square(c)
                x = gmp.square_chain_proth(x, c, k, n, every=c)[0]
                assert e.get_residue() == x, c
        with pg.Engine(k, n) as e:
            e.set_residue(x)
            e.square(2300)
            assert e.get_residue() == gmp.square_chain_proth(x, 2300, k, n, every=2300)[0]
    finally:
        pg.tune_clear()
