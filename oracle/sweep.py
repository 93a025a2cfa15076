"""TEST INFRASTRUCTURE ONLY: a randomised parity sweep of the C restatement (kinc_oracle.c)
against KINC's own code compiled by build_ref.py (needs the KINC tree).

Each case draws a workload (synthetic.py 1, 2, 4 or 5), a matrix shape, and every argument
of the analytic (clustering none / GMM / K-means, Pearson / Spearman, BIC / ICL, pre and
post outliers, cluster range, minsamp, minexpr), runs the first pairs of the matrix
through both, and compares K, N, the labels of multi-cluster pairs and every
correlation bit for bit.  With --opencl the restatement runs in rand="lcg" mode against
KINC's OpenCL kernels (clustering none or GMM; minexpr integral, as that worker passes
it as an int; Pearson correlations only of pairs with no excluded sample, the others
reading the worker's stale slot contents).

    python -m oracle.sweep --cases 300 --seed 123
    python -m oracle.sweep --opencl --cases 200 --seed 5
"""
import argparse
import sys
import time

import numpy as np

from kinc_gb300 import synthetic

from . import pyoracle


def same_corr(a, b):
    return np.array_equal(np.nan_to_num(a, nan=9.0), np.nan_to_num(b, nan=9.0))


def random_case(rng):
    wl = int(rng.choice([1, 2, 4, 5]))
    G = int(rng.integers(20, 60))
    S = int(rng.integers(25, 420))
    clus = int(rng.integers(0, 3))
    kw = dict(clus_method=clus, corr_method=int(rng.integers(0, 2)), criterion=int(rng.integers(0, 2)),
              pre_out=int(rng.integers(0, 2)), post_out=int(rng.integers(0, 2)),
              min_clusters=int(rng.integers(1, 3)),
              max_clusters=int(rng.integers(2, 6)) if clus != 2 else int(rng.integers(2, 4)),
              min_samples=int(rng.integers(15, 40)), min_expr=float(rng.choice([-np.inf, 5.0, 6.5])))
    if kw["min_clusters"] > kw["max_clusters"]:
        kw["min_clusters"] = 1
    gem = synthetic.generate(wl, genes=G, samples=S, seed=int(rng.integers(1 << 30)))
    return wl, gem, kw


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--cases", type=int, default=40)
    ap.add_argument("--seed", type=int, default=123)
    ap.add_argument("--pairs", type=int, default=300, help="pairs per case (from the first)")
    ap.add_argument("--opencl", action="store_true", help="rand=lcg against KINC's OpenCL kernels")
    args = ap.parse_args(argv)
    if args.opencl:
        return sweep_opencl(args)
    if pyoracle.ref_lib(0) is None:
        print("KINC source tree not present: nothing to compare against", file=sys.stderr)
        return 2
    rng = np.random.default_rng(args.seed)
    t0 = time.time()
    pairs = bad = 0
    for _ in range(args.cases):
        wl, gem, kw = random_case(rng)
        G, S = gem.shape
        size = min(G * (G - 1) // 2, args.pairs)
        p = pyoracle.params(**kw)
        a = pyoracle.run_block(gem, p, 0, size)
        b = pyoracle.run_ref(gem, p, 0, size)
        ok = (np.array_equal(a[0], b[0]) and np.array_equal(a[3], b[3])
              and np.array_equal(a[1][a[0] > 1], b[1][b[0] > 1]) and same_corr(a[2], b[2]))
        pairs += size
        if not ok:
            bad += 1
            print(f"mismatch: workload {wl}, {G} x {S}, {kw}")
    print(f"{args.cases} cases, {pairs} pairs, {bad} mismatching cases, {time.time() - t0:.0f} s")
    return 1 if bad else 0


def sweep_opencl(args):
    if pyoracle.ocl_lib() is None:
        print("KINC source tree not present: nothing to compare against", file=sys.stderr)
        return 2
    rng = np.random.default_rng(args.seed)
    t0 = time.time()
    pairs = bad = 0
    for _ in range(args.cases):
        wl, gem, kw = random_case(rng)
        kw["clus_method"] = int(rng.integers(0, 2))                   # none or GMM
        kw["max_clusters"] = max(kw["max_clusters"], kw["min_clusters"])
        kw["min_expr"] = float(rng.choice([-np.inf, 5.0, 6.0]))       # integral, as the worker passes it
        G, S = gem.shape
        size = min(G * (G - 1) // 2, args.pairs)
        p = pyoracle.params(rand_mode=1, **kw)
        K1, L1, C1, N1 = pyoracle.run_block(gem, p, 0, size)
        K2, L2, C2 = pyoracle.run_ocl(gem, p, 0, size, ksize=int(rng.choice([32, 256, 4096])))
        rows = np.ones(size, bool) if p.corr_method == 1 else (N1 == S)
        mask = rows[:, None] & (np.arange(p.max_clusters)[None, :] < K1[:, None])
        ok = (np.array_equal(K1, K2) and np.array_equal(L1[K1 > 1], L2[K1 > 1])
              and same_corr(C1[mask], C2[mask]))
        pairs += size
        if not ok:
            bad += 1
            print(f"mismatch: workload {wl}, {G} x {S}, {kw}")
    print(f"{args.cases} cases, {pairs} pairs, {bad} mismatching cases (OpenCL kernels), {time.time() - t0:.0f} s")
    return 1 if bad else 0


if __name__ == "__main__":
    sys.exit(main())
