"""Build the oracle (test infrastructure, the checker) into oracle/_build/liboracle.so.

Only tests/, the smoke check and bench.py's CPU-baseline leg load it.
Also builds the reference harness oracle/_ref/ref_harness when the reference
sources are present and the host is x86-64 (see oracle/ref/build_ref.sh).
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "proth_oracle.c")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")


def build_oracle(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "proth_oracle.h"))):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-Wall", "-o", tmp, SRC,
                           "-lm", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


def build_ref(force=False):
    """Returns the harness path, or None where the reference cannot be built."""
    src = os.environ.get("PROTH_REF_SRC", "/root/reference/prothlogic4.2")
    if os.path.exists(REF_BIN) and not force:
        return REF_BIN
    if not os.path.isdir(src) or platform.machine() != "x86_64":
        return None
    r = subprocess.run(["bash", os.path.join(HERE, "ref", "build_ref.sh")], capture_output=True, text=True)
    return REF_BIN if r.returncode == 0 and os.path.exists(REF_BIN) else None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
