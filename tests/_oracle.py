"""ctypes binding to the oracle library (oracle/_build/liboracle.so), the CPU
restatement of the reference's squaring path.  Test infrastructure only."""
import ctypes
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
from oracle.build_oracle import build_oracle, build_oracle_bench  # noqa: E402

u64 = ctypes.c_uint64
_lib = None
_bench_lib = None


def lib():
    """The exact oracle (oracle/_build/liboracle.so)."""
    global _lib
    if _lib is None:
        _lib = _bind(ctypes.CDLL(build_oracle()))
    return _lib


def bench_lib():
    """The same restatement built with the reference's optimisation flags
    (oracle/_build/liboracle_bench.so): only for timing the CPU baseline."""
    global _bench_lib
    if _bench_lib is None:
        _bench_lib = _bind(ctypes.CDLL(build_oracle_bench()))
    return _bench_lib


def _bind(L):
    L.ora_create.restype = ctypes.c_void_p
    L.ora_create.argtypes = [ctypes.c_size_t]
    L.ora_destroy.argtypes = [ctypes.c_void_p]
    L.ora_square_mod.restype = ctypes.c_double
    L.ora_square_mod.argtypes = [ctypes.c_void_p, ctypes.POINTER(u64), ctypes.c_uint, u64]
    L.ora_engine_square.argtypes = [ctypes.c_void_p, ctypes.POINTER(u64), ctypes.c_size_t, ctypes.c_uint, u64]
    L.ora_last_max_err.restype = ctypes.c_double
    L.ora_last_max_err.argtypes = [ctypes.c_void_p]
    L.ora_reduce.restype = ctypes.c_int
    L.ora_reduce.argtypes = [ctypes.POINTER(u64), ctypes.c_size_t, ctypes.c_uint, u64]
    L.ora_choose_L.restype = ctypes.c_size_t
    L.ora_choose_L.argtypes = [ctypes.c_uint, u64]
    L.ora_autotune_L.restype = ctypes.c_size_t
    L.ora_autotune_L.argtypes = [ctypes.c_uint, u64]
    L.ora_choose_base.restype = u64
    L.ora_choose_base.argtypes = [u64, ctypes.c_uint]
    L.ora_jacobi_small.restype = ctypes.c_int
    L.ora_jacobi_small.argtypes = [u64, u64, ctypes.c_uint]
    L.ora_gate_rejects.restype = ctypes.c_int
    L.ora_gate_rejects.argtypes = [u64, ctypes.c_uint]
    L.ora_gate_divisible.restype = ctypes.c_int
    L.ora_gate_divisible.argtypes = [u64, ctypes.c_uint, u64]
    L.ora_powm_small.argtypes = [ctypes.c_void_p, ctypes.POINTER(u64), u64, u64, ctypes.c_uint, u64]
    L.ora_proth_test.restype = ctypes.c_int
    L.ora_proth_test.argtypes = [u64, ctypes.c_uint, ctypes.c_size_t, ctypes.POINTER(u64), ctypes.POINTER(u64),
                                 ctypes.POINTER(ctypes.c_double), ctypes.POINTER(u64), ctypes.c_size_t]
    L.ora_run_squarings.restype = ctypes.c_double
    L.ora_run_squarings.argtypes = [ctypes.c_void_p, ctypes.POINTER(u64), ctypes.c_uint, u64, u64]
    L.ora_smallest_factor.restype = u64
    L.ora_smallest_factor.argtypes = [u64, ctypes.c_uint, u64]
    L.ora_bench_tests.restype = ctypes.c_double
    L.ora_bench_tests.argtypes = [ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_uint), ctypes.c_size_t,
                                  ctypes.c_int, u64, ctypes.POINTER(u64)]
    return L


def to_limbs(x, nl):
    return (u64 * nl).from_buffer_copy(int(x).to_bytes(8 * nl, "little"))


def from_limbs(a):
    return int.from_bytes(bytes(a), "little")


class Ctx:
    def __init__(self, L, library=None):
        self.L = L
        self.lib = library or lib()
        self.h = self.lib.ora_create(L)
        assert self.h

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ora_destroy(self.h)
            self.h = None

    def square_mod(self, x, k, n, steps=1):
        a = to_limbs(x, self.L // 4)
        err = 0.0
        for _ in range(steps):
            err = max(err, lib().ora_square_mod(self.h, a, n, k))
        return from_limbs(a), err

    def engine_square(self, x, k, n, n_limbs=None):
        nl = n_limbs or self.L // 4
        a = to_limbs(x, max(nl, self.L // 4))
        lib().ora_engine_square(self.h, a, nl, n, k)
        return from_limbs(a), lib().ora_last_max_err(self.h)


def proth_test(k, n, L=0, trace_len=0):
    a, r, e = u64(), u64(), ctypes.c_double()
    tr = (u64 * trace_len)() if trace_len else None
    v = lib().ora_proth_test(k, n, L, ctypes.byref(a), ctypes.byref(r), ctypes.byref(e), tr, trace_len)
    return {"verdict": v, "base": a.value, "res64": r.value, "max_err": e.value,
            "trace": [int(t) for t in tr] if tr else []}
