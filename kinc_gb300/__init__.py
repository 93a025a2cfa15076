"""kinc_gb300 -- GB300-native Similarity worker for KINC.

The per-pair work (fetch/mask, Tukey outliers, GMM / K-means with BIC/ICL
model selection, per-cluster Pearson / Spearman) runs in hand-written sm_103a
CUDA kernels behind the C ABI in include/kinc_sim.h; this package is the
host-side mirror of KINC's Similarity analytic over that ABI (Similarity),
of the CCM/CMX/EMX files and the analytics on either side of them
(pairwise_matrix: import/export of EMX and CMX text, network extraction;
rmt.RMT: RMT thresholding), plus sharding (shard) and seeded synthetic
workloads (synthetic).
"""
from .similarity import (CLUSTERING_NAMES, CORRELATION_NAMES, CRITERION_NAMES, InvalidArgument,  # noqa: F401
                         PairwiseMatrix, ResultBlock, Similarity, WorkBlock)
from . import pairwise_matrix, shard, synthetic  # noqa: F401

__all__ = ["Similarity", "WorkBlock", "ResultBlock", "PairwiseMatrix", "InvalidArgument", "pairwise_matrix",
           "shard", "synthetic"]
