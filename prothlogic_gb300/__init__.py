"""prothlogic_gb300 -- GB300-native engine for the Proth modular-squaring path.

The compute path is libprothgpu.so (hand-written sm_103a CUDA kernels + a C++
host engine behind the C ABI declared in include/prothgpu.h).  This module is a
thin ctypes binding that mirrors the reference's engine interface
(prothlogic4.2/fft_engine.h: init for k,n / square / last_max_diff, and
proth_logic.h: execute_proth_test_fft).  There is no CPU fallback: every call
that needs the device raises ProthGpuError when the library or the GPU is
missing.
"""
import ctypes
import os

from . import build as _build_mod

__all__ = ["ProthGpuError", "Engine", "Batch", "proth_test", "execute_proth_test_fft",
           "load", "pick_fft_len", "gate_rejects", "choose_base", "host_roundtrip", "prefilter",
           "PrefilterStream"]

PG_OK = 0
PG_EINVAL = 1
PG_EROUNDOFF = 3
PG_EGERBICZ = 4
PG_ESTATE = 9
PG_ETOOBIG = 11
FLAG_NO_GERBICZ = 0x1
FLAG_NO_BUMP = 0x2
FLAG_NO_GRAPH = 0x4
FLAG_FORCE_LEN = 0x8
FLAG_NO_PERSIST = 0x10
FLAG_PERSIST = 0x20

_u64 = ctypes.c_uint64
_u32 = ctypes.c_uint32
_i32 = ctypes.c_int32
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t


class PgResult(ctypes.Structure):
    _fields_ = [("k", _u64), ("n", _u32), ("base", _u32), ("verdict", _i32), ("status", _i32),
                ("res64", _u64), ("tag", _u64), ("fft_len", _u32), ("fft_bumps", _u32),
                ("gerbicz_checks", _u32), ("gerbicz_failures", _u32), ("max_err", ctypes.c_double),
                ("seconds", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class PgTuneResult(ctypes.Structure):
    _fields_ = [("lg", _u32), ("slots", _u32), ("passes", _u32), ("f0", _u32), ("f1", _u32), ("f2", _u32),
                ("g_mid", _u32), ("g_inner", _u32), ("tpb", _u32), ("cluster", _u32), ("tpb_outer", _u32),
                ("resident", _u32), ("resident_threads", _u32), ("edge", _u32), ("us_per_step", ctypes.c_double),
                ("valid", _i32), ("chosen", _i32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ProthGpuError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = _lib.pg_strerror(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else msg)


_lib = None

# symbol name -> (restype, argtypes); the exported surface of include/prothgpu.h
SIGNATURES = {
    "pg_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "pg_version": (ctypes.c_int, []),
    "pg_device_info": (ctypes.c_int, [ctypes.c_char_p, _sz, ctypes.POINTER(ctypes.c_int)]),
    "pg_pick_fft_len": (_u32, [_u64, _u32]),
    "pg_gate_rejects": (ctypes.c_int, [_u64, _u32]),
    "pg_choose_base": (_u64, [_u64, _u32]),
    "pg_host_roundtrip": (ctypes.c_int, [_u64, _u32, _u32, ctypes.POINTER(_u64), _sz, ctypes.POINTER(_u64), _sz]),
    "pg_create": (ctypes.c_int, [_u64, _u32, _u32, _u32, ctypes.POINTER(_vp)]),
    "pg_destroy": (ctypes.c_int, [_vp]),
    "pg_set_residue": (ctypes.c_int, [_vp, ctypes.POINTER(_u64), _sz]),
    "pg_get_residue": (ctypes.c_int, [_vp, ctypes.POINTER(_u64), _sz]),
    "pg_square": (ctypes.c_int, [_vp, _u64]),
    "pg_peek_residue": (ctypes.c_int, [_vp, ctypes.POINTER(_u64), _sz, ctypes.POINTER(_sz), ctypes.POINTER(_u64)]),
    "pg_pow_small": (ctypes.c_int, [_vp, _u64, _u64]),
    "pg_max_err": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "pg_fft_len": (ctypes.c_int, [_vp, ctypes.POINTER(_u32)]),
    "pg_set_gerbicz": (ctypes.c_int, [_vp, _u32, _u32]),
    "pg_stats": (ctypes.c_int, [_vp, ctypes.POINTER(_u64), ctypes.POINTER(_u32), ctypes.POINTER(_u32),
                                ctypes.POINTER(_u32)]),
    "pg_debug_corrupt": (ctypes.c_int, [_vp, _u32, _i32]),
    "pg_measure_fp64_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "pg_square_timed": (ctypes.c_int, [_vp, _u64, ctypes.POINTER(ctypes.c_double)]),
    "pg_flush_l2": (ctypes.c_int, []),
    "pg_launch_count": (_u64, []),
    "pg_set_device": (ctypes.c_int, [ctypes.c_int]),
    "pg_time_squarings": (ctypes.c_int, [_vp, _u64, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_u32)]),
    "pg_profile_step": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), _u32, ctypes.POINTER(_u32)]),
    "pg_checkpoint_save": (ctypes.c_int, [_vp, ctypes.c_char_p, _u64]),
    "pg_checkpoint_load": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_u64)]),
    "pg_proth_test": (ctypes.c_int, [_u64, _u32, _u32, ctypes.POINTER(PgResult)]),
    "pg_prefilter": (ctypes.c_int, [ctypes.POINTER(_u64), ctypes.POINTER(_u32), _sz, _u64, ctypes.POINTER(_u64)]),
    "pg_prefilter_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, _sz, _u64, ctypes.c_void_p, ctypes.c_void_p]),
    "pg_sieve_create": (ctypes.c_int, [_u64, _sz, ctypes.POINTER(_vp)]),
    "pg_sieve_strike": (ctypes.c_int, [_vp, ctypes.c_void_p, ctypes.c_void_p, _sz, ctypes.c_void_p, ctypes.c_void_p]),
    "pg_sieve_primes": (ctypes.c_int, [_vp, ctypes.POINTER(_u64)]),
    "pg_sieve_destroy": (ctypes.c_int, [_vp]),
    "pg_batch_create": (ctypes.c_int, [_u32, _u32, ctypes.POINTER(_vp)]),
    "pg_batch_destroy": (ctypes.c_int, [_vp]),
    "pg_batch_submit": (ctypes.c_int, [_vp, _u64, _u32, _u64]),
    "pg_batch_run": (ctypes.c_int, [_vp, _u64]),
    "pg_batch_poll": (ctypes.c_int, [_vp, ctypes.POINTER(PgResult), _sz, ctypes.POINTER(_sz)]),
    "pg_batch_run_timed": (ctypes.c_int, [_vp, _u64, ctypes.POINTER(ctypes.c_double)]),
    "pg_batch_pending": (ctypes.c_int, [_vp, ctypes.POINTER(_sz), ctypes.POINTER(_sz), ctypes.POINTER(_sz)]),
    "pg_batch_set_budget": (ctypes.c_int, [_vp, _u64]),
    "pg_batch_debug_corrupt": (ctypes.c_int, [_vp, _u64, _u32, _i32]),
    "pg_slot_footprint": (_u64, [_u64, _u32]),
    "pg_batch_set_gerbicz": (ctypes.c_int, [_vp, _u64]),
    "pg_autotune": (ctypes.c_int, [_u32, _u32, _u32, ctypes.POINTER(PgTuneResult), _sz, ctypes.POINTER(_sz)]),
    "pg_tune_get": (ctypes.c_int, [_u32, _u32, ctypes.POINTER(PgTuneResult)]),
    "pg_tune_set": (ctypes.c_int, [_u32, ctypes.POINTER(PgTuneResult)]),
    "pg_tune_clear": (ctypes.c_int, []),
}

TUNE_ONE, TUNE_MANY = 0, 1


def load(build_if_missing=True):
    """Load libprothgpu.so (building it in-tree with nvcc when absent or stale)."""
    global _lib
    if _lib is None:
        if build_if_missing:
            _build_mod.build()
        if not os.path.exists(_build_mod.LIB):
            raise ProthGpuError(8, "libprothgpu.so is not built")
        lib = ctypes.CDLL(_build_mod.LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _check(rc, what):
    if rc != PG_OK:
        raise ProthGpuError(rc, what)


def _to_limbs(x, nl):
    return (_u64 * nl).from_buffer_copy(int(x).to_bytes(8 * nl, "little"))


def _from_limbs(arr):
    return int.from_bytes(bytes(arr), "little")


def measure_fp64_peak():
    """Measured DFMA throughput of the current GPU in TFLOP/s."""
    v = ctypes.c_double()
    _check(load().pg_measure_fp64_peak(ctypes.byref(v)), "pg_measure_fp64_peak")
    return v.value


def flush_l2():
    _check(load().pg_flush_l2(), "pg_flush_l2")


def launch_count():
    return int(load().pg_launch_count())


def set_device(device):
    _check(load().pg_set_device(device), "pg_set_device")


def prefilter(cands, bound=1 << 32):
    """Smallest odd prime factor < bound of each k*2^n+1 (0 if none), on the GPU."""
    m = len(cands)
    ks = (_u64 * max(m, 1))(*[k for k, _ in cands])
    ns = (_u32 * max(m, 1))(*[n for _, n in cands])
    out = (_u64 * max(m, 1))()
    _check(load().pg_prefilter(ks, ns, m, bound, out), "pg_prefilter")
    return [int(out[i]) for i in range(m)]


PREFILTER_NOALLOC_MAX_COUNT = 65536
SIEVE_MAX_COUNT = 65536


class Sieve:
    """Every odd prime below `bound` held in device memory (pg_sieve_create:
    sieved once, 8 bytes a prime), for trial division of up to `max_count`
    candidates per strike.  strike() queues the division on a CUDA stream and
    returns at once (no allocation, no host synchronisation)."""

    def __init__(self, bound=1 << 32, max_count=SIEVE_MAX_COUNT):
        self.bound = int(bound)
        self.max_count = int(max_count)
        self._h = _vp()
        _check(load().pg_sieve_create(self.bound, self.max_count, ctypes.byref(self._h)), "pg_sieve_create")

    def primes(self):
        c = _u64()
        _check(load().pg_sieve_primes(self._h, ctypes.byref(c)), "pg_sieve_primes")
        return int(c.value)

    def strike(self, d_ks, d_ns, count, d_factor, stream):
        """d_ks / d_ns / d_factor: device addresses (int64, int32, int64 arrays);
        stream: a cudaStream_t value (0: the legacy default stream)."""
        _check(load().pg_sieve_strike(self._h, ctypes.c_void_p(d_ks), ctypes.c_void_p(d_ns), count,
                                      ctypes.c_void_p(d_factor), ctypes.c_void_p(stream)), "pg_sieve_strike")

    def close(self):
        if self._h:
            load().pg_sieve_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PrefilterStream:
    """Trial division of newly arrived candidates queued on a CUDA stream of its
    own, so it runs on the GPU beside the batch instead of between its slices.
    resident=True (the default): a Sieve made here holds the primes below the
    bound in device memory and each call only divides; resident=False:
    pg_prefilter_noalloc, which sieves again in every call and allocates
    nothing.  The device and pinned host buffers are allocated once here (torch
    provides them and the stream); each call copies the candidates in, queues
    the division and the copy of its answers back, and returns at once; poll()
    hands the answers over when the work has finished.  One call at a time (the
    calls share the sieve's or the pre-filter's device scratch)."""

    def __init__(self, bound=1 << 32, cap=PREFILTER_NOALLOC_MAX_COUNT, resident=True):
        import torch
        self._torch = torch
        self.bound = int(bound)
        self.cap = int(cap)
        self.sieve = Sieve(self.bound, self.cap) if resident else None
        self.stream = torch.cuda.Stream()
        self.h_k = torch.empty(self.cap, dtype=torch.int64, pin_memory=True)
        self.h_n = torch.empty(self.cap, dtype=torch.int32, pin_memory=True)
        self.h_f = torch.empty(self.cap, dtype=torch.int64, pin_memory=True)
        self.d_k = torch.empty(self.cap, dtype=torch.int64, device="cuda")
        self.d_n = torch.empty(self.cap, dtype=torch.int32, device="cuda")
        self.d_f = torch.empty(self.cap, dtype=torch.int64, device="cuda")
        self._count = None
        self._event = None
        # the first noalloc call on a device sets its scratch up, synchronously:
        # do it now (and warm the strike path the same way)
        self.start([(3, 2048)])
        self._event.synchronize()
        self.poll()

    def busy(self):
        return self._count is not None

    def start(self, cands):
        if self.busy():
            raise ProthGpuError(9, "PrefilterStream.start: a call is still running")
        m = len(cands)
        if m > self.cap:
            raise ProthGpuError(PG_ETOOBIG, f"PrefilterStream.start: {m} candidates (at most {self.cap})")
        torch = self._torch
        self.h_k[:m] = torch.tensor([k for k, _ in cands], dtype=torch.int64)
        self.h_n[:m] = torch.tensor([n for _, n in cands], dtype=torch.int32)
        with torch.cuda.stream(self.stream):
            self.d_k[:m].copy_(self.h_k[:m], non_blocking=True)
            self.d_n[:m].copy_(self.h_n[:m], non_blocking=True)
            if self.sieve is not None:
                self.sieve.strike(self.d_k.data_ptr(), self.d_n.data_ptr(), m, self.d_f.data_ptr(),
                                  self.stream.cuda_stream)
            else:
                _check(load().pg_prefilter_noalloc(self.d_k.data_ptr(), self.d_n.data_ptr(), m, self.bound,
                                                   self.d_f.data_ptr(), self.stream.cuda_stream),
                       "pg_prefilter_noalloc")
            self.h_f[:m].copy_(self.d_f[:m], non_blocking=True)
            self._event = torch.cuda.Event()
            self._event.record(self.stream)
        self._count = m

    def poll(self):
        """The smallest factors of the last call's candidates (0: none below the
        bound) once it has finished, else None."""
        if not self.busy() or not self._event.query():
            return None
        m, self._count = self._count, None
        return [int(x) for x in self.h_f[:m].tolist()]

    def close(self):
        if self.busy():
            self._event.synchronize()
            self._count = None
        if self.sieve is not None:
            self.sieve.close()


def slot_footprint(k, n):
    """Device bytes one admitted candidate holds."""
    return int(load().pg_slot_footprint(k, n))


def autotune(lg, slots=1, iters=200):
    """Time every compiled launch shape at 2^lg points on `slots` residues; the
    fastest bit-exact one becomes the shape of later engines (slots == 1) or
    batch classes (slots > 1) at that length.  Returns one dict per shape."""
    cap = 256
    out = (PgTuneResult * cap)()
    cnt = _sz()
    _check(load().pg_autotune(lg, slots, iters, out, cap, ctypes.byref(cnt)), f"pg_autotune(lg={lg})")
    return [out[i].as_dict() for i in range(min(cap, cnt.value))]


def tune_get(lg, mode=TUNE_ONE):
    """Shape in use at 2^lg points for `mode`, or None when none was tuned or set."""
    r = PgTuneResult()
    rc = load().pg_tune_get(lg, mode, ctypes.byref(r))
    if rc == PG_ESTATE:
        return None
    _check(rc, "pg_tune_get")
    return r.as_dict()


def tune_set(mode, shape):
    """Install a shape dict (as returned by autotune/tune_get) for `mode`."""
    r = PgTuneResult(**{f: shape[f] for f, _ in PgTuneResult._fields_ if f in shape})
    if "tpb" not in shape:
        r.tpb = 1
    _check(load().pg_tune_set(mode, ctypes.byref(r)), "pg_tune_set")


def tune_clear():
    _check(load().pg_tune_clear(), "pg_tune_clear")


def pick_fft_len(k, n):
    return load().pg_pick_fft_len(k, n)


def gate_rejects(k, n):
    return bool(load().pg_gate_rejects(k, n))


def choose_base(k, n):
    return int(load().pg_choose_base(k, n))


def host_roundtrip(k, n, M, x):
    nl = max(1, (x.bit_length() + 63) // 64)
    out_nl = n // 64 + 4
    out = (_u64 * out_nl)()
    _check(load().pg_host_roundtrip(k, n, M, _to_limbs(x, nl), nl, out, out_nl), "pg_host_roundtrip")
    return _from_limbs(out)


class Engine:
    """One candidate k*2^n+1 on the whole GPU (fft_init / fft_square_karatsuba / fft_destroy)."""

    _h = None

    def __init__(self, k, n, fft_len_hint=0, flags=0):
        lib = load()
        h = _vp()
        _check(lib.pg_create(k, n, fft_len_hint, flags, ctypes.byref(h)), "pg_create")
        self._h = h
        self.k, self.n = k, n
        self.N = k * (1 << n) + 1
        self._nl = n // 64 + 3

    def close(self):
        if self._h:
            load().pg_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_residue(self, x):
        nl = max(1, (int(x).bit_length() + 63) // 64)
        _check(load().pg_set_residue(self._h, _to_limbs(int(x), nl), nl), "pg_set_residue")

    def get_residue(self):
        out = (_u64 * self._nl)()
        _check(load().pg_get_residue(self._h, out, self._nl), "pg_get_residue")
        return _from_limbs(out)

    def square(self, iters=1):
        _check(load().pg_square(self._h, iters), "pg_square")

    def pow_small(self, base, exponent):
        _check(load().pg_pow_small(self._h, base, exponent), "pg_pow_small")

    def max_err(self, reset=False):
        v = ctypes.c_double()
        _check(load().pg_max_err(self._h, ctypes.byref(v), 1 if reset else 0), "pg_max_err")
        return v.value

    @property
    def fft_len(self):
        v = _u32()
        _check(load().pg_fft_len(self._h, ctypes.byref(v)), "pg_fft_len")
        return v.value

    def set_gerbicz(self, block, verify_every_blocks=0):
        _check(load().pg_set_gerbicz(self._h, block, verify_every_blocks), "pg_set_gerbicz")

    def stats(self):
        sq, c, f, b = _u64(), _u32(), _u32(), _u32()
        _check(load().pg_stats(self._h, ctypes.byref(sq), ctypes.byref(c), ctypes.byref(f), ctypes.byref(b)),
               "pg_stats")
        return {"squarings": sq.value, "gerbicz_checks": c.value, "gerbicz_failures": f.value,
                "fft_bumps": b.value}

    def square_timed(self, iters):
        """pg_square with CUDA events on the engine stream around it; returns ms."""
        ms = ctypes.c_double()
        _check(load().pg_square_timed(self._h, iters, ctypes.byref(ms)), "pg_square_timed")
        return ms.value

    def time_squarings(self, iters):
        """Device-timed squarings (CUDA events on the engine stream): (ms, kernels per squaring)."""
        ms, kps = ctypes.c_double(), _u32()
        _check(load().pg_time_squarings(self._h, iters, ctypes.byref(ms), ctypes.byref(kps)), "pg_time_squarings")
        return ms.value, kps.value

    def profile_step(self):
        """Per-kernel device times (ms) of one squaring, kernels launched one by one."""
        arr = (ctypes.c_double * 8)()
        cnt = _u32()
        _check(load().pg_profile_step(self._h, arr, 8, ctypes.byref(cnt)), "pg_profile_step")
        return [arr[i] for i in range(cnt.value)]

    def debug_corrupt(self, index, delta):
        _check(load().pg_debug_corrupt(self._h, index, delta), "pg_debug_corrupt")

    def checkpoint_save(self, path, current_i):
        _check(load().pg_checkpoint_save(self._h, os.fsencode(path), current_i), "pg_checkpoint_save")

    def checkpoint_load(self, path):
        ci = _u64()
        _check(load().pg_checkpoint_load(self._h, os.fsencode(path), ctypes.byref(ci)), "pg_checkpoint_load")
        return ci.value


def autotune_engine(k, n, base=None, blocks=10, block=1000, top=3, iters=400):
    """Launch shape for engines at the FFT length of k*2^n+1, chosen for the work
    an engine does.  pg_autotune times every compiled shape on bare squaring
    chains; its `top` fastest are then timed on one Gerbicz-checked interval of
    this candidate -- `blocks` blocks of `block` squarings, the verification
    chain squared beside the residue in the last block, as Engine.square runs
    it -- and the fastest there is installed for later engines (the two
    rankings can differ).  Returns the autotune rows: the installed one has
    "chosen" set, each timed one carries "us_in_situ" (us per squaring)."""
    lg = pick_fft_len(k, n).bit_length() - 1
    if lg < 0:
        raise ProthGpuError(PG_EINVAL, f"autotune_engine(k={k}, n={n}): no FFT length")
    rows = autotune(lg, slots=1, iters=iters)
    x0 = base if base else (choose_base(k, n) or 3)  # any residue times the same
    best = None
    for r in sorted((r for r in rows if r["valid"]), key=lambda r: r["us_per_step"])[:top]:
        tune_set(TUNE_ONE, r)
        with Engine(k, n) as e:
            e.set_gerbicz(block, blocks)
            e.set_residue(x0)
            e.square(block)                       # graphs, plans, weights
            e.set_residue(x0)
            ms = e.square_timed(blocks * block)
        r["us_in_situ"] = ms * 1e3 / (blocks * block)
        if best is None or r["us_in_situ"] < best["us_in_situ"]:
            best = r
    if best is not None:
        tune_set(TUNE_ONE, best)
        for r in rows:
            r["chosen"] = 1 if r is best else 0
    return rows


def proth_test(k, n, flags=0):
    """Full Proth test on the GPU; returns the result record as a dict."""
    r = PgResult()
    _check(load().pg_proth_test(k, n, flags, ctypes.byref(r)), f"pg_proth_test(k={k}, n={n})")
    return r.as_dict()


def execute_proth_test_fft(k, n):
    """Reference-shaped entry point (proth_logic.h:12): True when k*2^n+1 is a Proth prime."""
    return proth_test(k, n)["verdict"] == 1


class Batch:
    """Many candidates per launch, grouped by FFT length (the reference's worker pool)."""

    _h = None

    def __init__(self, max_slots_per_class=256, flags=0):
        h = _vp()
        _check(load().pg_batch_create(max_slots_per_class, flags, ctypes.byref(h)), "pg_batch_create")
        self._h = h

    def close(self):
        if self._h:
            load().pg_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def submit(self, k, n, tag=0):
        _check(load().pg_batch_submit(self._h, k, n, tag), "pg_batch_submit")

    def run(self, max_steps=0):
        _check(load().pg_batch_run(self._h, max_steps), "pg_batch_run")

    def set_gerbicz(self, block):
        """Gerbicz block length in class steps (before the first run)."""
        _check(load().pg_batch_set_gerbicz(self._h, block), "pg_batch_set_gerbicz")

    def run_timed(self, max_steps):
        """pg_batch_run with CUDA events on the class streams; returns device ms."""
        ms = ctypes.c_double()
        _check(load().pg_batch_run_timed(self._h, max_steps, ctypes.byref(ms)), "pg_batch_run_timed")
        return ms.value

    def poll(self, cap=4096):
        arr = (PgResult * cap)()
        cnt = _sz()
        _check(load().pg_batch_poll(self._h, arr, cap, ctypes.byref(cnt)), "pg_batch_poll")
        return [arr[i].as_dict() for i in range(cnt.value)]

    def debug_corrupt(self, tag, index, delta):
        _check(load().pg_batch_debug_corrupt(self._h, tag, index, delta), "pg_batch_debug_corrupt")

    def set_budget(self, hbm_bytes):
        """Cap the device bytes held by admitted candidates (admission by HBM footprint)."""
        _check(load().pg_batch_set_budget(self._h, int(hbm_bytes)), "pg_batch_set_budget")

    def pending(self):
        q, r, f = _sz(), _sz(), _sz()
        _check(load().pg_batch_pending(self._h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(f)),
               "pg_batch_pending")
        return q.value, r.value, f.value
