"""Launch-shape autotuner from the command line.

Times every compiled launch shape at each length class (pg_autotune: CUDA
events around graph replays of `iters` squarings, every shape checked to give
the same residues as the others) and prints, per length, the fastest shapes and
the fastest of each kind: `t1` (one thread per radix-4 butterfly everywhere),
`t2+` (two or four lanes per butterfly in some pass) and `resident` (the residue
held in a cluster's shared memory for the whole chain).  The fastest shape
becomes the one later engines (slots == 1) or batch classes (slots > 1) use at
that length in this process.

    python -m prothlogic_gb300.tune --lengths 12,14,16,17,18 --slots 1 --iters 400
"""
import argparse
import json

from . import autotune


def describe(r):
    """'16x64x64 g2/2 t2/2' style name of a tuner row."""
    radices = "x".join(str(x) for x in (r["f0"], r["f1"], r["f2"]) if x)
    if r["resident"]:
        return f"{radices} resident {r['resident']} CTAs x {r['resident_threads']}"
    s = f"{radices} g{r['g_mid']}/{r['g_inner']} t{r['tpb']}/{r['tpb_outer']}"
    if r["cluster"]:
        s += f" cluster {r['cluster']}"
    if r["edge"]:
        s += " fused edge"
    return s


def kind(r):
    if r["resident"]:
        return "resident"
    return "t1" if r["tpb"] == 1 and r["tpb_outer"] == 1 else "t2+"


def summary(lg, slots=1, iters=400, top=3):
    rows = sorted((r for r in autotune(lg, slots=slots, iters=iters) if r["valid"]), key=lambda r: r["us_per_step"])
    best = {}
    for r in rows:
        best.setdefault(kind(r), r)
    return {"lg": lg, "slots": slots, "shapes": len(rows),
            "fastest": [[describe(r), round(r["us_per_step"], 2)] for r in rows[:top]],
            "fastest_by_kind": {k: [describe(v), round(v["us_per_step"], 2)] for k, v in best.items()}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--lengths", default="12,14,16,17,18", help="log2 of the transform lengths")
    ap.add_argument("--slots", type=int, default=1, help="residues per launch (1: engines, > 1: batch classes)")
    ap.add_argument("--iters", type=int, default=400, help="squarings timed per shape")
    args = ap.parse_args()
    for lg in (int(x) for x in args.lengths.split(",")):
        print(json.dumps(summary(lg, args.slots, args.iters)), flush=True)


if __name__ == "__main__":
    main()
