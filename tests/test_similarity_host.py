"""Host-side mirror of the Similarity analytic: arguments, block split and
the ordered pairwise-matrix writer (no GPU)."""
import math

import numpy as np
import pytest

from kinc_gb300 import InvalidArgument, PairwiseMatrix, Similarity


def test_defaults_and_choices():
    s = Similarity(np.zeros((10, 5), np.float32))
    p = s.params
    assert (p.clus_method, p.corr_method, p.criterion, p.min_samples) == (0, 0, 1, 30)
    assert math.isinf(p.min_expr) and p.min_expr < 0
    s = Similarity(np.zeros((10, 5), np.float32), clusmethod="gmm", corrmethod="spearman", crit="BIC")
    assert (s.params.clus_method, s.params.corr_method, s.params.criterion) == (1, 1, 0)
    with pytest.raises(InvalidArgument):
        Similarity(np.zeros((10, 5), np.float32), clusmethod="dbscan")


def test_cluster_range_check():
    s = Similarity(np.zeros((10, 5), np.float32), minclus=4, maxclus=2)
    with pytest.raises(InvalidArgument, match="Minimum clusters"):
        s.initialize()


@pytest.mark.parametrize("genes", [2, 3, 257, 1000, 30000])
def test_block_split(genes):
    s = Similarity(np.zeros((genes, 1), np.float32))
    total = genes * (genes - 1) // 2
    assert s.size() == (total + 32767) // 32768
    blocks = [s.make_work(i) for i in range(s.size())]
    assert blocks[0].start == 0
    assert sum(b.size for b in blocks) == total
    assert all(b.size == 32768 for b in blocks[:-1])


def test_pairwise_matrix_order_is_enforced():
    m = PairwiseMatrix("cmx", 10, 5, 4)
    m.write_pair(1, 0, [0.9])
    m.write_pair(2, 1, [0.5, -0.7])
    with pytest.raises(ValueError, match="Attempting to write indent"):
        m.write_pair(2, 0, [0.8])
    with pytest.raises(ValueError, match="exceeding the max"):
        m.write_pair(9, 8, [0.1] * 6)
    x, y, c, r = m.arrays()
    assert list(c) == [0, 0, 1] and m.pairs == 2
