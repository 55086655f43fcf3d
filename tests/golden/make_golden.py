"""Generate tests/golden/golden.json from the reference itself and GMP.

Run where the reference sources, an x86-64 host for the reference's AVX-512
engine and libgmp.so.10 are present (PROTH_REF_SRC names the reference's
prothlogic4.2 directory):

    PROTH_REF_SRC=<path to prothlogic4.2> python tests/golden/make_golden.py
    python tests/golden/make_golden.py --large-only    # GMP only: the n = 2^20 section

Sources of truth, in order:
  * oracle/_ref/ref_harness  -- the UNMODIFIED reference engine (fft_engine.cpp,
    llr_fft_pack.cpp, proth_logic.cpp) built by oracle/ref/build_ref.sh;
  * GMP (mpz_powm / mpz_mul + mpz_mod) through ctypes, cross-checking every
    vector the reference produced.
Residues are stored as RES64 (limb 0) plus a SHA-256 of the full canonical
residue, so the fixture stays small.
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.build_oracle import build_ref  # noqa: E402
from prothlogic_gb300 import workloads  # noqa: E402
from tests import _gmp  # noqa: E402

M64 = (1 << 64) - 1


def digest(x):
    return hashlib.sha256(x.to_bytes((x.bit_length() + 7) // 8 or 1, "little")).hexdigest()


def corrected_L(n, k):
    L = 256
    while n / L > 18.0:
        L *= 2
    while n + k.bit_length() + 64 > 16 * L:
        L *= 2
    return L


def autotune_start_L(n):
    L = 256
    while n / L > 18.0:
        L *= 2
    return L


def base_of(k, n):
    N = k * (1 << n) + 1
    for b in [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37]:
        if _gmp.jacobi(b, N) == -1:
            return b
    for b in range(2, 100):
        if _gmp.jacobi(b, N) == -1:
            return b
    return 0


def run_ref(args, cwd, stdin=None):
    out = subprocess.run([REF] + [str(a) for a in args], cwd=cwd, capture_output=True, text=True, check=True,
                         input=stdin)
    return out.stdout


def _str_args(args):
    return [str(a) for a in args]


def ref_trace(k, n, L, x0, steps, cwd):
    out = run_ref(["trace", k, n, L, steps, "-"], cwd, stdin=format(x0, "x"))
    rows = [ln.split() for ln in out.strip().splitlines() if ln and ln[0].isdigit()]
    return [int(r[1], 16) for r in rows]


def ref_test(k, n, L, cwd):
    out = run_ref(["test", k, n, L], cwd)
    out = "".join(ch for ch in out if ch == "\n" or 32 <= ord(ch) < 127)  # the reference rings a bell on primes
    last = out.strip().splitlines()[-1].split()
    return int(last[0]), int(last[1], 16), float(last[2])


LARGE_BLOCKS = 200  # RES64 every 1,000 squarings up to 200,000: bench runs of up to 200 steps are checked


def large_section():
    """The n = 2^20 configuration: x0 = a, RES64 after every 1,000 squarings up
    to LARGE_BLOCKS * 1,000 (GMP, with the Proth-form reduction)."""
    k, n = workloads.large()
    a = base_of(k, n)
    chain = _gmp.square_chain_proth(a, LARGE_BLOCKS * 1000, k, n, every=1000)
    print("large", k, n, a, flush=True)
    return {"k": k, "n": n, "a": a, "x0": "a", "every": 1000,
            "res64": [format(c & M64, "016x") for c in chain], "final_sha256": digest(chain[-1])}


def update_large_only():
    """Recompute only the large section of an existing golden.json (GMP only;
    needs neither the reference sources nor an x86-64 host)."""
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(out) as f:
        g = json.load(f)
    g["large"] = large_section()
    with open(out, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", out)


def main():
    global REF
    REF = build_ref()
    if REF is None:
        sys.exit("reference harness unavailable (needs the reference sources on x86-64)")
    g = {"generator": "tests/golden/make_golden.py", "traces": [], "autotune_bug": [], "tests": [],
         "known": [], "large": {}, "gmp_tests": []}
    with tempfile.TemporaryDirectory() as cwd:
        # 1. per-step traces of the reference engine at the corrected L, from x0 = a^k mod N
        for k, n, steps in [(3, 2048, 300), (9999, 4096, 300), (77, 8300, 300), (5, 32700, 300), (3, 32768, 300),
                            (9999, 32752, 300), (4097, 65536, 200), (843, 120002, 100), (12345, 262144, 40),
                            (524287, 1048576, 30)]:
            N = k * (1 << n) + 1
            L = corrected_L(n, k)
            a = base_of(k, n) or 3
            x0 = _gmp.powmod(a, k, N)
            ref = ref_trace(k, n, L, x0, steps, cwd)
            chain = _gmp.square_chain(x0, steps, N)
            assert [c & M64 for c in chain] == ref, ("reference disagrees with GMP", k, n, L)
            g["traces"].append({"k": k, "n": n, "L": L, "a": a, "steps": steps, "x0": "a^k mod N",
                                "res64": [format(r, "016x") for r in ref], "final_sha256": digest(chain[-1])})
            print("trace", k, n, L, "ok", flush=True)
        # 2. the reference autotune length fails at these sizes (n + bitlen(k) > 16 L)
        for k, n, steps in [(3, 32768, 40), (4097, 65536, 20), (9999, 32752, 10)]:
            N = k * (1 << n) + 1
            L = autotune_start_L(n)
            a = base_of(k, n) or 3
            x0 = _gmp.powmod(a, k, N)
            ref = ref_trace(k, n, L, x0, steps, cwd)
            chain = [c & M64 for c in _gmp.square_chain(x0, steps, N)]
            first_bad = next((i for i in range(steps) if ref[i] != chain[i]), None)
            g["autotune_bug"].append({"k": k, "n": n, "a": a, "autotune_L": L, "corrected_L": corrected_L(n, k),
                                      "first_mismatch_step": first_bad,
                                      "ref_res64": [format(r, "016x") for r in ref]})
            print("autotune bug", k, n, L, first_bad, flush=True)
        # 3. full tests with the reference driver (execute_proth_test_fft) at the corrected L
        cands = workloads.single(count=4) + [(3, 2049), (5, 2500), (9, 3000), (27, 4096), (1275, 5000), (99, 6000)]
        for k, n in cands:
            N = k * (1 << n) + 1
            L = corrected_L(n, k)
            v, r, err = ref_test(k, n, L, cwd)
            a = base_of(k, n)
            gated = any(p % 2 and k % p and pow(2, n, p) == (-pow(k, -1, p)) % p
                        for p in [3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67])
            if not gated and a:
                y = _gmp.powmod(a, (N - 1) // 2, N)
                assert (y & M64) == r and v == (1 if y == N - 1 else 0), ("ref vs GMP", k, n)
            g["tests"].append({"k": k, "n": n, "L": L, "base": 0 if gated else a, "verdict": v,
                               "res64": format(r, "016x"), "gated": bool(gated)})
            print("test", k, n, v, format(r, "016x"), flush=True)
        # 4. known answers from the reference's console log ("Run test":41, 81, 88)
        for k, n, expect in [(843, 120002, 1), (853, 120002, 0), (895, 120002, 0)]:
            L = corrected_L(n, k)
            v, r, err = ref_test(k, n, L, cwd)
            assert v == expect
            g["known"].append({"k": k, "n": n, "L": L, "base": base_of(k, n), "verdict": v,
                               "res64": format(r, "016x"), "source": "Run test log"})
            print("known", k, n, v, flush=True)
    # 5. the large single-candidate configuration (GMP)
    g["large"] = large_section()
    # 6. full tests from the batched configurations, GMP only
    for k, n in workloads.uniform(count=3) + [c for c in workloads.uneven(count=40) if c[1] < 40000][:6]:
        N = k * (1 << n) + 1
        gated = any(p % 2 and k % p and pow(2, n, p) == (-pow(k, -1, p)) % p
                    for p in [3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67])
        a = 0 if gated else base_of(k, n)
        y = _gmp.powmod(a, (N - 1) // 2, N) if a else 0
        g["gmp_tests"].append({"k": k, "n": n, "base": a, "verdict": int(y == N - 1) if a else 0,
                               "res64": format(y & M64, "016x"), "gated": bool(gated)})
        print("gmp test", k, n, flush=True)
    # 7. a checkpoint file written by the reference's own save_checkpoint
    k, n = 9999, 32768
    N = k * (1 << n) + 1
    L = corrected_L(n, k)
    a = base_of(k, n)
    x = _gmp.square_chain(_gmp.powmod(a, k, N), 500, N, every=500)[0]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_checkpoint_k9999_n32768.bin")
    subprocess.run([REF] + _str_args(["ckpt_save", k, n, L, 499, path]), input=format(x, "x"), text=True,
                   check=True)
    g["ref_checkpoint"] = {"file": os.path.basename(path), "k": k, "n": n, "L": L, "a": a, "current_i": 499,
                           "squarings_from_a_pow_k": 500, "sha256": digest(x),
                           "res64_after_300_more": format(_gmp.square_chain(x, 300, N, every=300)[0] & M64, "016x")}
    print("ref checkpoint written", flush=True)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(out, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    if "--large-only" in sys.argv:
        update_large_only()
    else:
        main()
