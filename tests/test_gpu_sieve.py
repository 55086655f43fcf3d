"""pg_sieve (every odd prime below the bound held on the device, trial division
queued on a stream) against the oracle's plain trial division
(ora_smallest_factor) and against pg_prefilter, on the same candidates.

Integer results, so every comparison is exact.  The candidates include ones
with a planted factor just above a stage boundary of the strike (the live list
must carry them past the small primes), k above 2^32 (the split of k into two
32-bit halves), repeated candidates and any order of n."""
import ctypes
import random

import pytest

pytestmark = pytest.mark.gpu

PG_EINVAL = 1
PG_ETOOBIG = 11


@pytest.fixture(scope="module")
def pg():
    import prothlogic_gb300 as pgm
    pgm.load()
    return pgm


def _is_prime(p):
    if p < 2:
        return False
    for q in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        if p % q == 0:
            return p == q
    d, s = p - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37):
        x = pow(a, d, p)
        if x in (1, p - 1):
            continue
        for _ in range(s - 1):
            x = x * x % p
            if x == p - 1:
                break
        else:
            return False
    return True


def _planted(seed, count, lo, hi, k_bits=None):
    """k*2^n+1 divisible by a prime p in [lo, hi); k odd, below 2^k_bits when
    given (k = the residue -2^-n mod p plus a multiple of p)."""
    rng = random.Random(seed)
    out = []
    while len(out) < count:
        p = rng.randrange(lo | 1, hi, 2)
        if not _is_prime(p):
            continue
        n = rng.randrange(1000, 300000)
        k = (-pow(2, -n, p)) % p
        if k_bits:
            k += p * rng.randrange(0, (1 << k_bits) // p)
        if k % 2 == 0:
            k += p
        out.append((k, n))
    return out


def _random(seed, count, k_max=500000):
    rng = random.Random(seed)
    return [(2 * rng.randrange(1, k_max) + 1, rng.randrange(1000, 300000)) for _ in range(count)]


def _strike(sieve, torch, cands):
    ks = torch.tensor([k for k, _ in cands], dtype=torch.int64, device="cuda")
    ns = torch.tensor([n for _, n in cands], dtype=torch.int32, device="cuda")
    out = torch.full((len(cands),), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    sieve.strike(ks.data_ptr(), ns.data_ptr(), len(cands), out.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    return [int(x) for x in out.cpu().tolist()]


def test_sieve_matches_trial_division_two_strikes(pg):
    torch = pytest.importorskip("torch")
    from tests import _oracle
    bound = 1 << 24
    s = pg.Sieve(bound, 4096)
    try:
        assert s.primes() == 1077870  # odd primes below 2^24 (pi(2^24) = 1,077,871)
        strikes = [
            _random(51, 200) + _planted(61, 40, (1 << 22) + 1, (1 << 22) + 5000)
            + _planted(62, 40, (1 << 19) + 1, (1 << 19) + 3000) + [(3, 2048), (843, 120002)],
            _planted(63, 10, (1 << 13), (1 << 13) + 200) + _random(52, 300)
            + _planted(64, 30, (1 << 23), 1 << 24, k_bits=40) + _random(53, 30, k_max=1 << 39),
        ]
        for cands in strikes:
            got = _strike(s, torch, cands)
            want = [_oracle.lib().ora_smallest_factor(k, n, bound) for k, n in cands]
            assert got == want
            assert got == pg.prefilter(cands, bound=bound)
            # smallest factors found past the 2^19 and 2^22 stage boundaries (6 and 11 of them)
            assert sum(1 for f in got if f > (1 << 19)) >= 6
        assert sum(1 for k, _ in strikes[1] if k >= (1 << 32)) >= 30
        first = _strike(s, torch, strikes[0])
        assert first[-2:] == [19, 0]  # 19 | 3*2^2048+1; 843*2^120002+1 is prime
    finally:
        s.close()


def test_sieve_order_duplicates_and_edges(pg):
    """Candidates in any order of n, repeated ones, one candidate alone, a bound
    that ends inside a window and a bound with no primes below it."""
    torch = pytest.importorskip("torch")
    from tests import _oracle
    cands = _random(71, 60)
    cands = cands[::-1] + cands[:9] + _planted(72, 6, (1 << 16) + 1, (1 << 16) + 900)
    for bound in ((1 << 19) + 3, 1 << 21, 3):
        s = pg.Sieve(bound, 128)
        try:
            for batch in (cands, cands[:1], cands[-3:]):
                got = _strike(s, torch, batch)
                assert got == [_oracle.lib().ora_smallest_factor(k, n, bound) for k, n in batch]
        finally:
            s.close()


def test_sieve_full_bound(pg):
    """Every odd prime below 2^32 (203,280,220 of them): factors planted just
    below 2^32 and near 2^31 are found (or a smaller one that divides), answers
    equal pg_prefilter's, and the part of each answer below 2^24 is the oracle's."""
    torch = pytest.importorskip("torch")
    from tests import _oracle
    s = pg.Sieve(1 << 32, 1024)
    try:
        assert s.primes() == 203280220
        cands = (_planted(81, 6, (1 << 32) - 20000, 1 << 32) + _planted(82, 6, (1 << 31) - 5000, (1 << 31) + 5000)
                 + _random(83, 200) + [(843, 120002), (3, 2048)])
        got = _strike(s, torch, cands)
        assert got == pg.prefilter(cands, bound=1 << 32)
        assert got[-2:] == [0, 19]
        for (k, n), f in zip(cands, got):
            if f:
                assert _is_prime(f) and (k * pow(2, n, f) + 1) % f == 0
            small = _oracle.lib().ora_smallest_factor(k, n, 1 << 24)
            assert small == (f if f and f < (1 << 24) else 0)
        for (k, n), f in zip(cands[:12], got[:12]):
            assert f and f <= (1 << 32)
    finally:
        s.close()


def test_sieve_limits(pg):
    torch = pytest.importorskip("torch")
    lib = pg.load()
    h = ctypes.c_void_p()
    assert lib.pg_sieve_create(1 << 20, 65537, ctypes.byref(h)) == PG_ETOOBIG
    assert lib.pg_sieve_create((1 << 32) + 1, 16, ctypes.byref(h)) == PG_EINVAL
    assert lib.pg_sieve_create(2, 16, ctypes.byref(h)) == PG_EINVAL
    assert lib.pg_sieve_create(1 << 20, 0, ctypes.byref(h)) == PG_EINVAL
    s = pg.Sieve(1 << 20, 16)
    try:
        assert s.primes() == 82024  # pi(2^20) = 82,025
        ks = torch.full((17,), 3, dtype=torch.int64, device="cuda")
        ns = torch.full((17,), 2048, dtype=torch.int32, device="cuda")
        out = torch.zeros((17,), dtype=torch.int64, device="cuda")
        rc = lib.pg_sieve_strike(s._h, ctypes.c_void_p(ks.data_ptr()), ctypes.c_void_p(ns.data_ptr()), 17,
                                 ctypes.c_void_p(out.data_ptr()), None)
        assert rc == PG_ETOOBIG
        assert _strike(s, torch, []) == []
    finally:
        s.close()
