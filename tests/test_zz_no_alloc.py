"""pg_prefilter_noalloc (fixed device scratch, caller-owned device buffers)
against pg_prefilter (the allocating entry point) and against the oracle's
plain trial division (ora_smallest_factor) on the same candidates.

Integer results, so the comparison is exact.  Two calls in a row share the one
scratch array; the second must not see anything the first left behind."""
import ctypes
import random

import pytest

pytestmark = pytest.mark.gpu

PG_ETOOBIG = 11


@pytest.fixture(scope="module")
def pg():
    import prothlogic_gb300 as pgm
    pgm.load()
    return pgm


def _random(seed, count):
    rng = random.Random(seed)
    return [(2 * rng.randrange(1, 500000) + 1, rng.randrange(1000, 300000)) for _ in range(count)]


def _with_factor_above_segment(seed, count):
    """k*2^n+1 divisible by a prime p in (2^22, 2^23): about one in eight of
    these has p as its smallest factor, so the live list carries such candidates
    past the smallest primes before the factor is found."""
    rng = random.Random(seed)
    out = []
    while len(out) < count:
        p = rng.randrange((1 << 22) + 1, 1 << 23, 2)
        if any(p % q == 0 for q in range(3, int(p ** 0.5) + 1, 2)):
            continue
        n = rng.randrange(1000, 300000)
        k = (-pow(2, -n, p)) % p
        if k % 2 == 0:
            k += p
        out.append((k, n))
    return out


def _call(pg, torch, cands, bound):
    lib = pg.load()
    ks = torch.tensor([k for k, _ in cands], dtype=torch.int64, device="cuda")
    ns = torch.tensor([n for _, n in cands], dtype=torch.int32, device="cuda")
    out = torch.full((len(cands),), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.pg_prefilter_noalloc(ctypes.c_void_p(ks.data_ptr()), ctypes.c_void_p(ns.data_ptr()), len(cands),
                                  bound, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    stream.synchronize()
    return rc, [int(x) for x in out.cpu().tolist()]


def test_noalloc_prefilter_matches_prefilter_two_calls(pg):
    torch = pytest.importorskip("torch")
    from tests import _oracle
    calls = [
        (_random(31, 300) + _with_factor_above_segment(21, 40), 1 << 26),
        (_with_factor_above_segment(22, 40) + _random(32, 500) + [(3, 2048), (843, 120002)], 1 << 24),
    ]
    results = []
    for cands, bound in calls:
        expected = pg.prefilter(cands, bound=bound)
        assert sum(1 for f in expected if f > (1 << 22)) >= 2
        rc, got = _call(pg, torch, cands, bound)
        assert rc == 0, pg.load().pg_strerror(rc).decode()
        assert got == expected
        assert got == [_oracle.lib().ora_smallest_factor(k, n, bound) for k, n in cands]
        results.append(got)
    assert results[1][-2:] == [19, 0]  # 19 | 3*2^2048+1; 843*2^120002+1 is prime


def test_noalloc_prefilter_order_and_duplicates(pg):
    """Candidates in any order of n, repeated ones, and a single candidate: the
    device ranks them by n before the walk; answers stay those of trial division."""
    torch = pytest.importorskip("torch")
    from tests import _oracle
    cands = _random(41, 50)
    cands = cands[::-1] + cands[:7] + _with_factor_above_segment(23, 10)
    bound = 1 << 24
    for batch in (cands, cands[:1]):
        rc, got = _call(pg, torch, batch, bound)
        assert rc == 0
        assert got == [_oracle.lib().ora_smallest_factor(k, n, bound) for k, n in batch]


def test_noalloc_prefilter_rejects_more_than_its_scratch_holds(pg):
    torch = pytest.importorskip("torch")
    lib = pg.load()
    count = 65536 + 1
    ks = torch.full((count,), 3, dtype=torch.int64, device="cuda")
    ns = torch.full((count,), 2048, dtype=torch.int32, device="cuda")
    out = torch.zeros((count,), dtype=torch.int64, device="cuda")
    rc = lib.pg_prefilter_noalloc(ctypes.c_void_p(ks.data_ptr()), ctypes.c_void_p(ns.data_ptr()), count, 1 << 20,
                                  ctypes.c_void_p(out.data_ptr()), None)
    assert rc == PG_ETOOBIG
    assert "65536" in lib.pg_strerror(rc).decode()
