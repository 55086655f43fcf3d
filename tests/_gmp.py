"""ctypes binding to the system GMP (libgmp.so.10): the independent arithmetic
check for the oracle and the engine.  Test infrastructure only."""
import ctypes
import ctypes.util


class _Mpz(ctypes.Structure):
    _fields_ = [("alloc", ctypes.c_int), ("size", ctypes.c_int), ("d", ctypes.c_void_p)]


_lib = None
_F = {}  # short name -> GMP function (avoids class-private name mangling of __gmpz_*)


def available():
    try:
        _load()
        return True
    except OSError:
        return False


def _load():
    global _lib
    if _lib is None:
        name = "libgmp.so.10"
        lib = ctypes.CDLL(name)
        P = ctypes.POINTER(_Mpz)
        for fn, args, res in [("__gmpz_init", [P], None), ("__gmpz_clear", [P], None),
                              ("__gmpz_set_str", [P, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
                              ("__gmpz_get_str", [ctypes.c_char_p, ctypes.c_int, P], ctypes.c_void_p),
                              ("__gmpz_powm", [P, P, P, P], None), ("__gmpz_mul", [P, P, P], None),
                              ("__gmpz_mod", [P, P, P], None), ("__gmpz_jacobi", [P, P], ctypes.c_int),
                              ("__gmpz_sizeinbase", [P, ctypes.c_int], ctypes.c_size_t),
                              ("__gmpz_tdiv_q_2exp", [P, P, ctypes.c_ulong], None),
                              ("__gmpz_tdiv_r_2exp", [P, P, ctypes.c_ulong], None),
                              ("__gmpz_fdiv_qr_ui", [P, P, P, ctypes.c_ulong], ctypes.c_ulong),
                              ("__gmpz_mul_2exp", [P, P, ctypes.c_ulong], None),
                              ("__gmpz_add", [P, P, P], None), ("__gmpz_sub", [P, P, P], None),
                              ("__gmpz_cmp", [P, P], ctypes.c_int)]:
            f = getattr(lib, fn)
            f.argtypes = args
            f.restype = res
            _F[fn[len("__gmpz_"):]] = f
        _lib = lib
    return _lib


class Z:
    def __init__(self, v=0):
        self.m = _Mpz()
        _load()
        _F["init"](ctypes.byref(self.m))
        self.set(v)

    def __del__(self):
        if _F:
            _F["clear"](ctypes.byref(self.m))

    def set(self, v):
        _load()
        _F["set_str"](ctypes.byref(self.m), format(int(v), "x").encode(), 16)

    def get(self):
        n = _F["sizeinbase"](ctypes.byref(self.m), 16) + 2
        buf = ctypes.create_string_buffer(n)
        _F["get_str"](buf, 16, ctypes.byref(self.m))
        return int(buf.value.decode(), 16)


def powmod(a, e, m):
    r, A, E, M = Z(), Z(a), Z(e), Z(m)
    _F["powm"](ctypes.byref(r.m), ctypes.byref(A.m), ctypes.byref(E.m), ctypes.byref(M.m))
    return r.get()


def jacobi(a, n):
    A, N = Z(a), Z(n)
    return _F["jacobi"](ctypes.byref(A.m), ctypes.byref(N.m))


def square_chain(x, steps, m, every=1):
    """x^(2^i) mod m for i = every, 2*every, ..., steps (GMP arithmetic)."""
    out = []
    X, M = Z(x), Z(m)
    for i in range(1, steps + 1):
        _F["mul"](ctypes.byref(X.m), ctypes.byref(X.m), ctypes.byref(X.m))
        _F["mod"](ctypes.byref(X.m), ctypes.byref(X.m), ctypes.byref(M.m))
        if i % every == 0:
            out.append(X.get())
    return out


def square_chain_proth(x, steps, k, n, every=1):
    """x^(2^i) mod N, N = k*2^n+1, for i = every, 2*every, ..., steps.  Each
    square x^2 = H*2^n + Lo is reduced with k*2^n = -1 (mod N): H = q*k + r gives
    x^2 = Lo + r*2^n - q (mod N), then at most a few additions or subtractions
    of N.  Only GMP arithmetic; much faster than mpz_mod at n ~ 2^20."""
    out = []
    N = Z(k * (1 << n) + 1)
    X, H, Lo, Q, R, T = Z(x), Z(), Z(), Z(), Z(), Z()
    zero = Z(0)
    b = ctypes.byref
    for i in range(1, steps + 1):
        _F["mul"](b(X.m), b(X.m), b(X.m))
        _F["tdiv_q_2exp"](b(H.m), b(X.m), n)
        _F["tdiv_r_2exp"](b(Lo.m), b(X.m), n)
        _F["fdiv_qr_ui"](b(Q.m), b(R.m), b(H.m), k)
        _F["mul_2exp"](b(T.m), b(R.m), n)
        _F["add"](b(X.m), b(Lo.m), b(T.m))
        _F["sub"](b(X.m), b(X.m), b(Q.m))
        while _F["cmp"](b(X.m), b(zero.m)) < 0:
            _F["add"](b(X.m), b(X.m), b(N.m))
        while _F["cmp"](b(X.m), b(N.m)) >= 0:
            _F["sub"](b(X.m), b(X.m), b(N.m))
        if i % every == 0:
            out.append(X.get())
    return out


GATE_PRIMES = [3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67]
BASES = [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37] + list(range(2, 100))


def proth_test(k, n):
    """(verdict, base, res64) of the Proth test of N = k*2^n+1 as the reference
    decides it (prothlogic4.2/proth_logic.cpp:400-577): a gate prime <= 67
    dividing N gives composite with base 0 and no residue; otherwise a is the
    first listed base with Jacobi(a, N) = -1 (none: composite, residue 0), and
    x = a^((N-1)/2) = (a^k)^(2^(n-1)) mod N, prime iff x = N-1; res64 = x mod 2^64."""
    for p in GATE_PRIMES:
        if k % p and pow(2, n, p) == (-pow(k, -1, p)) % p:
            return 0, 0, 0
    N = k * (1 << n) + 1
    a = next((b for b in BASES if jacobi(b, N) == -1), 0)
    if a == 0:
        return 0, 0, 0
    x = powmod(a, k, N)
    if n > 1:
        x = square_chain_proth(x, n - 1, k, n, every=n - 1)[0]
    return int(x == N - 1), a, x & ((1 << 64) - 1)


def proth_tests(cands, processes=None):
    """proth_test over many candidates in a process pool (spawn: safe to start
    after the CUDA context exists)."""
    import multiprocessing
    import os
    ctx = multiprocessing.get_context("spawn")
    with ctx.Pool(processes or os.cpu_count() or 1) as pool:
        return pool.starmap(proth_test, cands, chunksize=1)
