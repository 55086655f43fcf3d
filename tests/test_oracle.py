"""The oracle (CPU restatement of the reference path) pinned against GMP and
against golden vectors produced by the unmodified reference engine."""
import json
import os
import random

import pytest

from tests import _oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.json")
M64 = (1 << 64) - 1


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def _N(k, n):
    return k * (1 << n) + 1


@pytest.mark.parametrize("k,n", [(3, 2048), (843, 4096), (9999, 5000), (77, 8300), (524287, 20000), (5, 32700)])
def test_oracle_steps_match_gmp(gmp, oracle, k, n):
    N = _N(k, n)
    L = oracle.lib().ora_choose_L(n, k)
    x = random.Random(k * 7 + n).randrange(N)
    ctx = oracle.Ctx(L)
    chain = gmp.square_chain(x, 12, N)
    for i in range(12):
        x, err = ctx.square_mod(x, k, n)
        assert x == chain[i], f"step {i}"
        assert err < 0.4


def test_oracle_matches_reference_traces(golden, gmp, oracle):
    checked = 0
    for t in golden["traces"]:
        if t["n"] > 70000:
            continue
        k, n, L = t["k"], t["n"], t["L"]
        N = _N(k, n)
        x = gmp.powmod(t["a"], k, N)
        ctx = oracle.Ctx(L)
        a = oracle.to_limbs(x, L // 4)
        for i, want in enumerate(t["res64"]):
            oracle.lib().ora_square_mod(ctx.h, a, n, k)
            assert format(int(a[0]), "016x") == want, (k, n, i)
        checked += 1
    assert checked >= 6


def test_bench_build_reproduces_reference_traces(golden, gmp, oracle):
    """The CPU-baseline build of the restatement (the reference's -O3 -march/-mcpu=native
    -funroll-loops -ffast-math) still gives the reference's residues at the corrected
    length, so the timed baseline computes the same squarings."""
    fast = oracle.bench_lib()
    checked = 0
    for t in golden["traces"]:
        if t["n"] > 70000:
            continue
        k, n, L = t["k"], t["n"], t["L"]
        N = _N(k, n)
        h = fast.ora_create(L)
        a = oracle.to_limbs(gmp.powmod(t["a"], k, N), L // 4)
        for i, want in enumerate(t["res64"]):
            err = fast.ora_square_mod(h, a, n, k)
            assert format(int(a[0]), "016x") == want, (k, n, i)
            assert err < 0.4
        fast.ora_destroy(h)
        checked += 1
    assert checked >= 6


def test_oracle_reproduces_reference_autotune_bug(golden, gmp, oracle):
    """At the length the reference's autotune picks, n + bitlen(k) > 16 L and the
    residues are wrong; the oracle reproduces those wrong residues bit for bit."""
    for t in golden["autotune_bug"]:
        k, n, L = t["k"], t["n"], t["autotune_L"]
        assert n + k.bit_length() + 64 > 16 * L
        assert oracle.lib().ora_autotune_L(n, k) == L or oracle.lib().ora_autotune_L(n, k) > L
        N = _N(k, n)
        ctx = oracle.Ctx(L)
        a = oracle.to_limbs(gmp.powmod(t["a"], k, N), L // 4)
        got = []
        for _ in t["ref_res64"]:
            oracle.lib().ora_square_mod(ctx.h, a, n, k)
            got.append(format(int(a[0]), "016x"))
        assert got == t["ref_res64"]
        assert t["first_mismatch_step"] is not None
        assert oracle.lib().ora_choose_L(n, k) == t["corrected_L"]


def test_oracle_full_tests_match_reference(golden, oracle):
    for t in golden["tests"]:
        if t["n"] > 10000:
            continue
        r = oracle.proth_test(t["k"], t["n"], t["L"])
        assert r["verdict"] == t["verdict"], t
        assert r["base"] == t["base"], t
        assert format(r["res64"], "016x") == t["res64"], t


def test_oracle_single_config_candidate(golden, oracle):
    t = next(t for t in golden["tests"] if t["n"] == 32768 and not t["gated"])
    r = oracle.proth_test(t["k"], t["n"], t["L"])
    assert (r["verdict"], format(r["res64"], "016x")) == (t["verdict"], t["res64"])


def test_known_answer_bases(golden, oracle, gmp):
    # 843*2^120002+1 is prime with a = 5; 853 and 895 composite (reference console log)
    for t in golden["known"]:
        assert oracle.lib().ora_choose_base(t["k"], t["n"]) == t["base"]
        assert not oracle.lib().ora_gate_rejects(t["k"], t["n"])
    assert [t["verdict"] for t in golden["known"]] == [1, 0, 0]
    assert golden["known"][0]["base"] == 5


@pytest.mark.slow
@pytest.mark.skipif(not os.environ.get("PROTH_SLOW"), reason="set PROTH_SLOW=1 (about 90 s)")
def test_oracle_known_prime_full(golden, oracle):
    t = golden["known"][0]
    r = oracle.proth_test(t["k"], t["n"], t["L"])
    assert r["verdict"] == 1 and format(r["res64"], "016x") == t["res64"]


def test_gate_base_jacobi_vs_gmp(gmp, oracle):
    rng = random.Random(11)
    L = oracle.lib()
    for _ in range(60):
        k = 2 * rng.randrange(1, 50000) + 1
        n = rng.randrange(2, 400)
        N = _N(k, n)
        for a in [2, 3, 5, 7, 9, 12, 37, 97]:
            assert L.ora_jacobi_small(a, k, n) == gmp.jacobi(a, N), (a, k, n)
        for p in [3, 5, 7, 11, 13, 67]:
            assert bool(L.ora_gate_divisible(k, n, p)) == (N % p == 0 and k % p != 0), (k, n, p)


def test_reduce_random(oracle):
    rng = random.Random(5)
    for _ in range(40):
        k = 2 * rng.randrange(1, 1 << 20) + 1
        n = rng.randrange(64, 3000)
        N = _N(k, n)
        nl = (2 * n + 200) // 64
        x = rng.randrange(1 << (64 * nl - 3))
        a = oracle.to_limbs(x, nl)
        assert oracle.lib().ora_reduce(a, nl, n, k) == 0
        assert oracle.from_limbs(a) == x % N


def test_choose_L_capacity(oracle):
    for n in [2048, 5000, 32768, 65536, 120002, 262144, 1 << 20]:
        for k in [3, 9999, 999999, (1 << 20) - 1]:
            L = oracle.lib().ora_choose_L(n, k)
            assert n + k.bit_length() + 64 <= 16 * L
            assert L & (L - 1) == 0


def test_reference_checkpoint_fixture_layout(golden, gmp):
    """The checkpoint written by the reference's save_checkpoint: header
    {uint64 current_i, size_t n_limbs} then little-endian limbs."""
    import struct
    c = golden["ref_checkpoint"]
    raw = open(os.path.join(os.path.dirname(GOLDEN), c["file"]), "rb").read()
    ci, nl = struct.unpack("<QQ", raw[:16])
    assert ci == c["current_i"] and nl == c["L"] // 4 and len(raw) == 16 + 8 * nl
    x = int.from_bytes(raw[16:], "little")
    N = _N(c["k"], c["n"])
    want = gmp.square_chain(gmp.powmod(c["a"], c["k"], N), c["squarings_from_a_pow_k"], N,
                            every=c["squarings_from_a_pow_k"])[0]
    assert x == want


def test_oracle_smallest_factor(oracle):
    rng = random.Random(4)
    for _ in range(30):
        k = 2 * rng.randrange(1, 5000) + 1
        n = rng.randrange(10, 3000)
        N = _N(k, n)
        want = next((p for p in range(3, 20000, 2) if all(p % q for q in range(3, int(p ** 0.5) + 1, 2))
                     and N % p == 0), 0)
        assert oracle.lib().ora_smallest_factor(k, n, 20000) == want
