"""GPU parity on edge inputs: the generic fit for more than five clusters, Spearman
and outlier sorts longer than the shared-memory buffers hold, degenerate genes
(all missing, constant, duplicated, too few usable samples), the smallest
matrices and sample counts, single-K ranges.  Every case runs the whole pair
range through the worker and through the oracle and must agree bit for bit."""
import numpy as np
import pytest

from kinc_gb300 import Similarity, synthetic
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _degenerate(G, S, seed=3):
    rng = np.random.default_rng(seed)
    gem = (8.0 + 2.0 * rng.standard_normal((G, S))).astype(np.float32)
    gem[rng.random((G, S)) < 0.1] = np.nan
    gem[1, :] = np.nan                                # no usable sample
    gem[2, :] = 5.0                                   # constant: zero variance, det = 0 in the GMM
    gem[3, :] = gem[4, :]                             # duplicate: r = 1 where both are usable
    gem[5, rng.permutation(S)[: S - 10]] = np.nan     # fewer usable samples than minsamp
    gem[6, :] = np.where(np.arange(S) % 2 == 0, 7.0, 9.0).astype(np.float32)   # two exact values
    return gem


CASES = [
    # name, matrix, gpu args, oracle args
    ("gmm_maxclus7_generic_fit", lambda: synthetic.generate(2, genes=20, samples=150),
     dict(clusmethod="gmm", crit="BIC", postout=True, maxclus=7),
     dict(clus_method=1, criterion=0, post_out=1, max_clusters=7)),
    ("kmeans_maxclus6_generic_fit", lambda: synthetic.generate(4, genes=20, samples=120),
     dict(clusmethod="kmeans", crit="BIC", maxclus=6),
     dict(clus_method=2, criterion=0, max_clusters=6)),
    ("none_spearman_1100_samples_global_sort", lambda: synthetic.generate(1, genes=18, samples=1100),
     dict(corrmethod="spearman"), dict(corr_method=1)),
    ("gmm_spearman_1100_samples_outliers", lambda: synthetic.generate(2, genes=10, samples=1100),
     dict(clusmethod="gmm", corrmethod="spearman", crit="ICL", preout=True, postout=True, maxclus=3),
     dict(clus_method=1, corr_method=1, criterion=1, pre_out=1, post_out=1, max_clusters=3)),
    ("gmm_degenerate_genes", lambda: _degenerate(24, 90),
     dict(clusmethod="gmm", crit="BIC", preout=True, postout=True),
     dict(clus_method=1, criterion=0, pre_out=1, post_out=1)),
    ("kmeans_degenerate_genes", lambda: _degenerate(24, 90),
     dict(clusmethod="kmeans", corrmethod="spearman", crit="ICL", maxclus=3),
     dict(clus_method=2, corr_method=1, criterion=1, max_clusters=3)),
    ("none_pearson_degenerate_genes", lambda: _degenerate(40, 64), dict(), dict()),
    ("gmm_single_pair", lambda: synthetic.generate(2, genes=2, samples=200),
     dict(clusmethod="gmm", crit="ICL", postout=True), dict(clus_method=1, criterion=1, post_out=1)),
    ("gmm_tiny_samples_minsamp5", lambda: synthetic.generate(2, genes=30, samples=9),
     dict(clusmethod="gmm", crit="BIC", minsamp=5, maxclus=2),
     dict(clus_method=1, criterion=0, min_samples=5, max_clusters=2)),
    ("none_pearson_tiny_samples", lambda: synthetic.generate(1, genes=50, samples=7),
     dict(minsamp=3), dict(min_samples=3)),
    ("gmm_single_k3", lambda: synthetic.generate(5, genes=22, samples=140),
     dict(clusmethod="gmm", crit="BIC", minclus=3, maxclus=3, preout=True),
     dict(clus_method=1, criterion=0, min_clusters=3, max_clusters=3, pre_out=1)),
    ("kmeans_minclus2_minexpr", lambda: synthetic.generate(1, genes=26, samples=110),
     dict(clusmethod="kmeans", crit="BIC", minclus=2, maxclus=3, minexpr=7.0),
     dict(clus_method=2, criterion=0, min_clusters=2, max_clusters=3, min_expr=7.0)),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_edge_case_matches_oracle(case):
    name, make, gargs, oargs = case
    gem = make()
    sim = Similarity(gem, **gargs)
    sim.initialize()
    total = sim.total_pairs()
    res = sim.execute(None, start=0, size=total)
    sim.close()
    K, labels, corr, N = pyoracle.run_block(gem, pyoracle.params(**oargs), 0, total)
    assert np.array_equal(res.K, K), f"K differs on {(res.K != K).sum()} of {total} pairs"
    multi = K > 1
    assert np.array_equal(res.labels[multi], labels[multi])
    assert np.array_equal(np.nan_to_num(res.corr, nan=9.0), np.nan_to_num(corr, nan=9.0))
