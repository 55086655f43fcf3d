"""Host-side checks that need no GPU: the C-ABI library loads and exports every
symbol the header declares; host conversions and Proth-test decisions."""
import os
import random
import re

import pytest

import prothlogic_gb300 as pg
from prothlogic_gb300 import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "prothgpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(pg_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = pg.load()
    names = _declared()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
        assert name in pg.SIGNATURES, f"{name} missing from the Python binding"


def test_version_and_strerror():
    lib = pg.load()
    assert lib.pg_version() >= 100
    assert lib.pg_strerror(3).decode().startswith("roundoff")


@pytest.mark.parametrize("k,n,M", [(3, 2048, 256), (843, 120002, 8192), (524287, 1048576, 65536),
                                   (9999, 32768, 2048), (77, 8300, 1024), (999999, 65536, 4096)])
def test_host_representation_roundtrip(k, n, M):
    N = k * (1 << n) + 1
    rng = random.Random(n + k)
    for x in [0, 1, N - 1, N - 2, rng.randrange(N), rng.randrange(N), (1 << n) - 1, k << n]:
        assert pg.host_roundtrip(k, n, M, x) == x % N
    # values above N are reduced
    big = rng.randrange(N * N)
    assert pg.host_roundtrip(k, n, M, big) == big % N


def test_gate_and_base_match_oracle(oracle, gmp):
    rng = random.Random(3)
    L = oracle.lib()
    for _ in range(200):
        k = 2 * rng.randrange(1, 500000) + 1
        n = rng.randrange(2048, 300000)
        assert pg.gate_rejects(k, n) == bool(L.ora_gate_rejects(k, n))
        assert pg.choose_base(k, n) == L.ora_choose_base(k, n)
    assert pg.choose_base(843, 120002) == 5


def test_fft_length_choice():
    prev = 0
    for n in [2048, 4096, 8192, 32768, 65536, 131072, 262144, 524288, 1 << 20, 5435752]:
        L = pg.pick_fft_len(3, n)
        assert L >= prev and L & (L - 1) == 0
        assert n / L <= 19.5
        prev = L
    assert pg.pick_fft_len(3, 1 << 20) == 65536
    assert pg.pick_fft_len(3, 65536) == 4096
    assert pg.pick_fft_len(3, 100) == 0  # below the smallest supported residue
    assert pg.pick_fft_len(199971, 5435752) == 1 << 19  # the reference console's largest candidate
    assert pg.pick_fft_len(3, 9_000_000) == 0  # beyond 17 bits per digit at 2^19


def test_workloads_are_seeded():
    assert workloads.single(3) == workloads.single(3)
    k, n = workloads.large()
    assert n == 1 << 20 and k % 2 == 1 and 3 <= k < (1 << 20)
    u = workloads.uniform(50)
    assert all(n == 65536 and k % 2 == 1 and 3 <= k < 10 ** 6 for k, n in u)
    v = workloads.uneven(200)
    assert all(8192 <= n <= 262144 and k % 2 == 1 and k < 10 ** 5 for k, n in v)
    s = workloads.serving(20, rate=10.0)
    assert all(s[i][0] < s[i + 1][0] for i in range(19))


def test_engine_fails_loudly_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pg.ProthGpuError):
        pg.Engine(3, 4096)


@pytest.mark.parametrize("cname,pystruct", [("pg_result", pg.PgResult), ("pg_tune_result", pg.PgTuneResult)])
def test_abi_struct_layout_matches_binding(tmp_path, cname, pystruct):
    """The ctypes mirrors have the C header's size and field offsets (compiled
    with the host C compiler against include/prothgpu.h)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in pystruct._fields_]
    src = tmp_path / "layout.c"
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "prothgpu.h"', "int main(void) {",
             f'    printf("%zu\\n", sizeof({cname}));']
    lines += [f'    printf("%zu\\n", offsetof({cname}, {f}));' for f in fields]
    lines += ["    return 0;", "}"]
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert got[0] == __import__("ctypes").sizeof(pystruct)
    for f, off in zip(fields, got[1:]):
        assert getattr(pystruct, f).offset == off, f


def test_tune_set_validates_cluster_shapes():
    """Fused-middle shapes are accepted only where a cluster kernel is compiled:
    three passes with equal middle and inner radices (host logic, no device)."""
    base = {"lg": 16, "slots": 1, "passes": 3, "f0": 64, "f1": 32, "f2": 32, "g_mid": 2, "g_inner": 4, "tpb": 1}
    try:
        for cl in (0, 4, 8):
            pg.tune_set(pg.TUNE_ONE, dict(base, cluster=cl))
            assert pg.tune_get(16, pg.TUNE_ONE)["cluster"] == cl
        pg.tune_set(pg.TUNE_ONE, dict(base, f0=16, f1=64, f2=64, g_inner=2, cluster=16))
        for bad in (dict(base, cluster=16),                      # no 32-point cluster of 16 CTAs
                    dict(base, cluster=3),
                    dict(base, f0=16, f1=64, f2=64, g_inner=2, cluster=2),     # no cluster of 2
                    dict(base, f0=32, f1=32, f2=64, g_inner=2, cluster=8),    # middle and inner radices differ
                    {"lg": 12, "slots": 1, "passes": 2, "f0": 64, "f1": 64, "f2": 0, "g_mid": 2, "g_inner": 2,
                     "tpb": 1, "cluster": 8}):                  # two-pass plans have no middle
            with pytest.raises(pg.ProthGpuError):
                pg.tune_set(pg.TUNE_ONE, bad)
        # lanes per butterfly: 1, 2 or 4, separately for the first and last passes
        quad = {"lg": 12, "slots": 1, "passes": 2, "f0": 32, "f1": 128, "f2": 0, "g_mid": 2, "g_inner": 2,
                "tpb": 2, "tpb_outer": 4}
        pg.tune_set(pg.TUNE_ONE, quad)
        got = pg.tune_get(12, pg.TUNE_ONE)
        assert (got["tpb"], got["tpb_outer"]) == (2, 4)
        pg.tune_set(pg.TUNE_ONE, dict(quad, tpb=4, tpb_outer=0))
        assert pg.tune_get(12, pg.TUNE_ONE)["tpb_outer"] == 4  # 0: the same as tpb
        for bad in (dict(quad, tpb=3), dict(quad, tpb_outer=8), dict(quad, f1=128, g_inner=8, tpb=4)):
            with pytest.raises(pg.ProthGpuError):
                pg.tune_set(pg.TUNE_ONE, bad)
    finally:
        pg.tune_clear()


def test_bench_module_helpers():
    """bench.py imports without a GPU; its shape parser and shape label agree."""
    import importlib
    import sys
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    shape = bench.parse_shape("64x32x32,gm=2,gi=4,tpb=1,cl=8", 16)
    assert (shape["f0"], shape["f1"], shape["f2"], shape["g_inner"], shape["cluster"]) == (64, 32, 32, 4, 8)
    row = dict(shape, chosen=1, tpb_outer=2)
    label = bench._chosen([row, dict(row, chosen=0)])
    assert label.startswith("64x32x32 middle fused in clusters of 8 CTAs") and "fastest of 2" in label
    assert bench.dp_ops_per_point((16, 64, 64)) == 126


def test_autotune_engine_rejects_unsupported_sizes():
    """autotune_engine refuses a candidate with no FFT length before touching a device."""
    with pytest.raises(pg.ProthGpuError) as ei:
        pg.autotune_engine(3, 100)
    assert ei.value.status == pg.PG_EINVAL


def test_reference_callers_link_against_the_gpu_shim(tmp_path):
    """The reference's own callers (dcore.cpp, worker.cpp, pipeline_proth.cpp,
    proth_logic.cpp, checkpoint_manager.cpp, storage_core.cpp, progress_core.cpp),
    compiled unmodified, link against the shim and libprothgpu.so instead of the
    reference engine (oracle/ref/build_ref_callers.sh).  Needs the reference
    sources, named by PROTH_REF_SRC; nothing here runs them (no GPU)."""
    import shutil
    import subprocess
    from oracle.build_oracle import ref_src
    src = ref_src()
    if not src or not os.path.isdir(src):
        pytest.skip("reference sources not named (PROTH_REF_SRC)")
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    pg.load()  # libprothgpu.so built
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    subprocess.run(["bash", os.path.join(here, "oracle", "ref", "build_ref_callers.sh"), src], check=True,
                   capture_output=True)
    binary = os.path.join(here, "oracle", "_ref", "ref_callers")
    syms = subprocess.run(["nm", "-C", binary], capture_output=True, text=True, check=True).stdout
    defined = {ln.split(" ", 2)[2].split("(")[0].split("[")[0] for ln in syms.splitlines() if " T " in ln}
    undefined = {ln.split()[-1] for ln in syms.splitlines() if ln.strip().startswith("U ")}
    # the reference's callers, and the engine entry points from the shim
    for name in ["dispatch", "auto_tune_fft_len", "execute_proth_test_fft", "run_task_with_ctx",
                 "build_proth_ff_tasks_for_range", "save_checkpoint", "load_checkpoint",
                 "fft_init", "fft_destroy", "fft_square_karatsuba"]:
        assert name in defined, name
    # the squaring itself comes from libprothgpu.so
    assert {"pg_create", "pg_square", "pg_peek_residue", "pg_set_residue", "pg_get_residue"} <= undefined
    # and none of the reference engine's own code is linked in
    for name in ["fft_stockham_radix8", "fft_bailey_2d", "unpack_karatsuba_overlap_add", "pack_karatsuba_limbs"]:
        assert name not in syms, name
