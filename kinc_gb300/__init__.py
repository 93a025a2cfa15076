"""kinc_gb300 -- GB300-native Similarity worker for KINC.

The per-pair work (fetch/mask, Tukey outliers, GMM / K-means with BIC/ICL
model selection, per-cluster Pearson / Spearman) runs in hand-written sm_103a
CUDA kernels behind the C ABI in include/kinc_sim.h; this package is the
host-side mirror of KINC's Similarity analytic over that ABI.
"""
from .similarity import (CLUSTERING_NAMES, CORRELATION_NAMES, CRITERION_NAMES, InvalidArgument,  # noqa: F401
                         PairwiseMatrix, ResultBlock, Similarity, WorkBlock)
from . import synthetic  # noqa: F401

__all__ = ["Similarity", "WorkBlock", "ResultBlock", "PairwiseMatrix", "InvalidArgument", "synthetic"]
