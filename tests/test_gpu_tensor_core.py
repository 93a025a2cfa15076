"""Masked-contraction Pearson (precision TF32 / 3xBF16 / scaled FP16 on the tensor cores,
FP32 tiled on the CUDA cores; clusmethod none): maximum |r| error against the
FP64 pairwise-complete oracle, and agreement with the plain per-pair FP32
kernel on the same pairs (semantics fixed)."""
import numpy as np
import pytest

from kinc_gb300 import Similarity, synthetic
from oracle import pyoracle

pytestmark = pytest.mark.gpu

# max |r - r_fp64| allowed per precision
TOL = {"3xbf16": 1e-4, "tf32": 2e-3, "fp16": 2e-3, "fp32tiled": 1e-5}


def _dense(genes, samples, seed=5):
    return synthetic.generate(3, genes=genes, samples=samples, seed=seed)


@pytest.mark.parametrize("precision", ["tf32", "3xbf16", "fp16", "fp32tiled"])
@pytest.mark.parametrize("shape", [(300, 500), (257, 130), (65, 33)])
def test_tensor_core_pearson_vs_fp64(precision, shape):
    G, S = shape
    gem = _dense(G, S)
    sim = Similarity(gem, semantics="fixed", precision=precision)
    sim.initialize()
    total = sim.total_pairs()
    res = sim.execute(None, start=0, size=total)
    sim.close()
    assert np.all(res.K == 1)
    x, y = pyoracle.pair_xy(np.arange(total))
    ref = pyoracle.pearson_fp64_pairs(gem, x, y)
    got = res.corr[:, 0].astype(np.float64)
    both = ~np.isnan(ref)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    err = np.abs(got[both] - ref[both]).max()
    assert err <= TOL[precision], f"max |dr| {err}"


@pytest.mark.parametrize("precision", ["tf32", "3xbf16", "fp16", "fp32tiled"])
def test_tensor_core_partial_range_matches_full(precision):
    gem = _dense(200, 96, seed=9)
    sim = Similarity(gem, semantics="fixed", precision=precision)
    sim.initialize()
    full = sim.execute(None, start=0, size=sim.total_pairs())
    part = sim.execute(None, start=12345, size=4321)
    sim.close()
    assert np.array_equal(np.nan_to_num(part.corr[:, 0], nan=9), np.nan_to_num(full.corr[12345:16666, 0], nan=9))


def test_fp16_scaling_with_outliers_vs_fp64():
    """Scaled FP16: each gene is scaled by a power of two so that its largest centred |value| is
    below 1; genes with one sample a thousand times the spread push the others' squares into FP16's
    subnormal range, and r stays within the TF32 bound."""
    gem = _dense(160, 300, seed=21)
    rng = np.random.default_rng(22)
    for g in rng.choice(160, size=20, replace=False):
        s = rng.integers(300)
        if np.isfinite(gem[g, s]):
            gem[g, s] += 1000.0 * np.nanstd(gem[g])
    sim = Similarity(gem, semantics="fixed", precision="fp16")
    sim.initialize()
    total = sim.total_pairs()
    res = sim.execute(None, start=0, size=total)
    sim.close()
    x, y = pyoracle.pair_xy(np.arange(total))
    ref = pyoracle.pearson_fp64_pairs(gem, x, y)
    got = res.corr[:, 0].astype(np.float64)
    both = ~np.isnan(ref)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.abs(got[both] - ref[both]).max() <= TOL["fp16"]


@pytest.mark.parametrize("precision", ["tf32", "3xbf16", "fp16"])
def test_one_column_results(precision):
    """One correlation column (maxclus 1, the bench's dense form): every pair of a range starting
    mid-row, written into device arrays that held other values, gets K = 1 and the r of the
    five-column run."""
    import ctypes

    import torch

    from kinc_gb300 import _native
    gem = _dense(300, 500, seed=31)
    start, size = 1234, 40000
    full = Similarity(gem, semantics="fixed", precision=precision)
    full.initialize()
    want = full.execute(None, start=start, size=size)
    full.close()
    sim = Similarity(gem, semantics="fixed", precision=precision, maxclus=1)
    sim.initialize()
    L = _native.load()
    dK = torch.full((size,), 7, dtype=torch.int8, device="cuda")
    dC = torch.full((size, 1), 2.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()             # the worker runs on its own stream
    vp = ctypes.c_void_p
    _native.check(L.kinc_sim_execute_block_device(sim._ctx, start, size, vp(dK.data_ptr()), None,
                                                  vp(dC.data_ptr()), None), sim._ctx)
    _native.check(L.kinc_sim_synchronize(sim._ctx), sim._ctx)
    torch.cuda.synchronize()
    sim.close()
    assert torch.all(dK == 1).item()
    got = dC[:, 0].cpu().numpy()
    assert np.array_equal(np.nan_to_num(got, nan=9.0), np.nan_to_num(want.corr[:, 0], nan=9.0))


def test_plain_fp32_fixed_semantics_vs_fp64():
    gem = _dense(120, 300)
    sim = Similarity(gem, semantics="fixed")
    sim.initialize()
    res = sim.execute(None, start=0, size=sim.total_pairs())
    sim.close()
    x, y = pyoracle.pair_xy(np.arange(sim.total_pairs()))
    ref = pyoracle.pearson_fp64_pairs(gem, x, y)
    both = ~np.isnan(ref)
    assert np.abs(res.corr[both, 0] - ref[both]).max() < 1e-4


def test_tensor_peak_measures_both_operand_types():
    """kinc_sim_tensor_peak: the dense tcgen05 rate the tensor-core form is compared with; BF16
    (K = 16 per MMA) runs at about twice the TF32 rate (K = 8)."""
    import ctypes

    from kinc_gb300 import _native
    L = _native.load()
    rates = {}
    for prec in (1, 2):
        v = ctypes.c_double(0.0)
        assert L.kinc_sim_tensor_peak(prec, ctypes.byref(v)) == 0
        rates[prec] = v.value
    assert 100.0 < rates[1] < 10000.0
    assert 1.5 < rates[2] / rates[1] < 2.5
    assert L.kinc_sim_tensor_peak(3, ctypes.byref(ctypes.c_double(0.0))) == _native.EINVAL
