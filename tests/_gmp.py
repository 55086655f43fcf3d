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
                              ("__gmpz_sizeinbase", [P, ctypes.c_int], ctypes.c_size_t)]:
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
