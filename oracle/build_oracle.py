"""Build the oracle (test infrastructure) into oracle/_build/.

Only tests/, the smoke check and bench.py's CPU legs load what this builds.

  liboracle.so        the exact oracle: gcc -O3, no value-changing flags.
  liboracle_bench.so  the same C restatement built with the reference's own
                      optimisation flags (SETUP:25: -O3 -march=native
                      -funroll-loops -fomit-frame-pointer -ffast-math; on
                      aarch64 -mcpu=native stands for -march=native, the
                      AVX-512 flags have no counterpart).  Used only to time
                      the CPU baseline; tests check that it still reproduces
                      the reference's residues.

Also builds the reference harness oracle/_ref/ref_harness when the reference
sources are named (PROTH_REF_SRC, or the `src` argument) and the host is
x86-64 (see oracle/ref/build_ref.sh).
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
BENCH_LIB = os.path.join(HERE, "_build", "liboracle_bench.so")
SRC = os.path.join(HERE, "proth_oracle.c")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")

EXACT_FLAGS = ["-O3", "-std=c11", "-fPIC", "-shared", "-Wall"]


def bench_flags():
    """The reference's SETUP:25 optimisation flags, as they apply to this host."""
    native = "-mcpu=native" if platform.machine() in ("aarch64", "arm64") else "-march=native"
    return ["-O3", native, "-funroll-loops", "-fomit-frame-pointer", "-ffast-math", "-std=c11", "-fPIC", "-shared"]


def _stale(out):
    deps = [SRC, os.path.join(HERE, "proth_oracle.h"), os.path.abspath(__file__)]
    return not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps)


def _build(out, flags, force):
    if not force and not _stale(out):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + ".tmp"
    subprocess.check_call(["gcc"] + flags + ["-o", tmp, SRC, "-lm", "-lpthread"])
    os.replace(tmp, out)
    return out


def build_oracle(force=False):
    return _build(LIB, EXACT_FLAGS, force)


def build_oracle_bench(force=False):
    return _build(BENCH_LIB, bench_flags(), force)


def ref_src(src=None):
    """Directory of the reference's prothlogic4.2 sources: the argument, else
    PROTH_REF_SRC, else None."""
    return src or os.environ.get("PROTH_REF_SRC") or None


def build_ref(force=False, src=None):
    """Returns the harness path, or None where the reference cannot be built
    (sources not named or absent, or not an x86-64 host)."""
    if os.path.exists(REF_BIN) and not force:
        return REF_BIN
    src = ref_src(src)
    if not src or not os.path.isdir(src) or platform.machine() != "x86_64":
        return None
    r = subprocess.run(["bash", os.path.join(HERE, "ref", "build_ref.sh"), src], capture_output=True, text=True)
    return REF_BIN if r.returncode == 0 and os.path.exists(REF_BIN) else None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_oracle_bench(force=True))
    print(build_ref(force=True))
