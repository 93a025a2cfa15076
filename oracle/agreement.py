"""Agreement of a run's results with KINC built against the C library's exp/log
(TEST INFRASTRUCTURE ONLY: used by tests/ and bench.py as a checker).

The fixtures in tests/golden/libm/ (made by tests/golden/make_libm_golden.py
from KINC's own Pairwise:: sources, src/core/pairwise_gmm.cpp et al.) hold,
for math mode 1 (glibc expf/logf) and mode 2 (glibc double exp/log), every
pair's K and correlations, a hash of every pair's label row, and the label
rows that differ from mode 0 (the portable exp/log the GPU and the oracle
use).  These builds are not expected to agree bit for bit with each other or
with mode 0: the EM trajectories depend on the last bit of every exp and log.
This module counts how far apart they are.
"""
import glob
import hashlib
import json
import os

import numpy as np

LIBM_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests", "golden", "libm")
MODES = {1: "glibc float expf/logf", 2: "glibc double exp/log (float sums partly in double)"}


def row_hashes(labels):
    """blake2b-64 of each int8 label row, as uint64 (the fixtures' hash)."""
    return np.array([int.from_bytes(hashlib.blake2b(r.tobytes(), digest_size=8).digest(), "little")
                     for r in np.ascontiguousarray(labels, np.int8)], dtype=np.uint64)


def cases():
    """{name: path} of the fixtures present."""
    return {os.path.basename(p)[:-4]: p for p in sorted(glob.glob(os.path.join(LIBM_DIR, "*.npz")))}


def load(path):
    z = np.load(path)
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    d["ncorr"] = int(d["ncorr"])
    return d


def compare(K, labels, corr, fx, mode):
    """Agreement of (K [P], labels [P][S], corr [P][maxk] or [P][maxk][2]) with fixture `fx`'s
    math mode `mode`: K agreement; of the pairs with the same K > 1, the share whose whole label
    row agrees and the share of their samples whose label agrees; max |dr| over the correlations
    of pairs whose K and labels both agree, and the share of those within 1e-5."""
    Kr, Cr, hr = fx[f"K{mode}"], fx[f"corr{mode}"], fx[f"hash{mode}"]
    diff_rows = {int(i): r for i, r in zip(fx[f"diff{mode}"], fx[f"labels{mode}"])}
    K = np.asarray(K)
    h = row_hashes(labels)
    same_k = K == Kr
    rows = same_k & (Kr > 1)
    same_lab = h == hr
    label_rows = int(rows.sum())
    label_eq = int((rows & same_lab).sum())
    # samples: rows with equal hashes agree everywhere; the others are compared with the stored row
    samples, differing, unknown = 0, 0, 0
    S = labels.shape[1]
    for i in np.nonzero(rows)[0]:
        samples += S
        if same_lab[i]:
            continue
        ref = diff_rows.get(int(i))
        if ref is None:
            unknown += 1
            differing += S
        else:
            differing += int((labels[i] != ref).sum())
    agree = same_k & (same_lab | (Kr <= 1))
    kk = np.arange(Cr.shape[1])[None, :] < Kr[:, None]
    m = kk & agree[:, None]
    a, b = np.asarray(corr)[m], Cr[m]
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    both = ~nan_a & ~nan_b
    dr = np.abs(a[both].astype(np.float64) - b[both].astype(np.float64))
    return {"mode": mode, "vs": "KINC's Pairwise:: sources built with " + MODES[mode],
            "pairs": int(len(K)), "k_agreement": float(same_k.mean()),
            "label_rows": label_rows,
            "label_agreement": float(label_eq / label_rows) if label_rows else 1.0,
            "sample_label_agreement": float(1.0 - differing / samples) if samples else 1.0,
            "rows_without_reference": unknown,
            "correlations_compared": int(both.sum()),
            "nan_mismatches": int((nan_a != nan_b).sum()),
            "max_abs_dr_same_labels": float(dr.max()) if len(dr) else 0.0,
            "within_1e-5": float((dr <= 1e-5).mean()) if len(dr) else 1.0}


def compare_modes(fx):
    """The two library builds against each other (mode 1 taken as the run, mode 2 as the reference)."""
    K1, C1, h1 = fx["K1"], fx["corr1"], fx["hash1"]
    K2, C2, h2 = fx["K2"], fx["corr2"], fx["hash2"]
    same_k = K1 == K2
    rows = same_k & (K2 > 1)
    return {"pairs": int(len(K1)), "k_agreement": float(same_k.mean()), "label_rows": int(rows.sum()),
            "label_agreement": float((rows & (h1 == h2)).sum() / rows.sum()) if rows.any() else 1.0}
