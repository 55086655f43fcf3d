"""Host logic of the autotuner command line: shape names and kinds (no GPU)."""
from prothlogic_gb300 import tune


def _row(**kw):
    r = {"f0": 16, "f1": 64, "f2": 64, "g_mid": 2, "g_inner": 2, "tpb": 1, "tpb_outer": 1, "cluster": 0,
         "edge": 0, "resident": 0, "resident_threads": 0}
    r.update(kw)
    return r


def test_shape_names_and_kinds():
    assert tune.describe(_row(tpb=2, tpb_outer=2)) == "16x64x64 g2/2 t2/2"
    assert tune.describe(_row(cluster=8, edge=1)) == "16x64x64 g2/2 t1/1 cluster 8 fused edge"
    assert tune.describe(_row(f0=32, f1=128, f2=0, resident=16, resident_threads=128)) == \
        "32x128 resident 16 CTAs x 128"
    assert tune.kind(_row()) == "t1"
    assert tune.kind(_row(tpb_outer=2)) == "t2+"
    assert tune.kind(_row(resident=4, resident_threads=128)) == "resident"
