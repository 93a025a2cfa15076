"""Similarity benchmark: gene pairs/sec on the GMM(k<=5) + Spearman workload.

Workload (the headline configuration): expression matrix 5,000 genes x 1,000
samples float32, 10% NaN, 10 planted mixture modules (kinc_gb300.synthetic
workload 2); clusmethod gmm, minclus 1, maxclus 5, crit BIC, preout + postout,
minsamp 30, corrmethod spearman.  A "step" is one device block of pairs
(--block, default 1,048,576 = 32 of KINC's 32,768-pair work blocks) taken in
pair order; warm-up and timed steps walk consecutive blocks, so every timed
pair is distinct.  Under torchrun every rank takes its own disjoint range of
blocks (weak scaling, no collective on the data path); the ranges wrap around
the 12,497,500 pairs only when ranks x steps x block exceed them.

Lines printed by rank 0 (one JSON object):
  value    pairs/s with the matrix already resident in HBM, timed with CUDA
           events on the worker's stream (max over ranks);
  e2e      the same through the C ABI with host buffers: kinc_sim_create
           (host->device upload of the matrix) + kinc_sim_execute_block into
           pinned host arrays (device->host K, labels, correlations);
  roofline the similarity kernel's algorithmic FP32 rate, and its thread-
           instruction issue rate (roofline.issue);
  cpu_baseline  the oracle (C restatement of KINC's serial path) on the host
           cores over a bounded sample;
  parity   the same sampled pairs through the GPU, compared with the oracle;
  and one object per further leg: tensor_core (dense 20,000 x 2,000 masked
  Pearson, TF32 / 3xBF16 / per-pair FP32, errors against FP64), kmeans_uneven
  (10,000 x 4,000), streamed_30000x500 (GMM ICL, both correlations, to CCM/CMX
  files) and rmt (RMT thresholding); each can be skipped (--no-dense,
  --no-kmeans, --stream-blocks 0, --no-rmt).
--impl reference runs that CPU path as the timed arm instead.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOAD = dict(workload=2, clusmethod="gmm", corrmethod="spearman", minclus=1, maxclus=5, crit="BIC",
                preout=True, postout=True, minsamp=30)
ORACLE_ARGS = dict(clus_method=1, corr_method=1, min_clusters=1, max_clusters=5, criterion=0, pre_out=1,
                   post_out=1, min_samples=30)
# algorithmic cost of one GMM unit (sample, component, EM iteration): 40 FP32 flops
FLOPS_PER_UNIT = 40


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample(gem, threads, pairs_per_thread, seed, outputs=False):
    """Time the oracle on `threads` segments of consecutive pairs, each starting
    at a seeded random work-block boundary; returns (pairs/s, pairs, seconds),
    plus (starts, sizes, (K, labels, corr)) when `outputs` is set."""
    from oracle import pyoracle
    G = gem.shape[0]
    total = G * (G - 1) // 2
    nblocks = (total + 32767) // 32768
    rng = np.random.default_rng(seed)
    blocks = rng.choice(nblocks - 1, size=threads, replace=threads > nblocks - 1)
    starts = blocks.astype(np.int64) * 32768
    sizes = np.full(threads, pairs_per_thread, np.int64)
    p = pyoracle.params(**ORACLE_ARGS)
    if not outputs:
        done, secs = pyoracle.run_segments_parallel(gem, p, starts, sizes, threads)
        return done / secs, int(done), secs
    done, secs, res = pyoracle.run_segments_parallel(gem, p, starts, sizes, threads, outputs=True)
    return done / secs, int(done), secs, starts, sizes, res


def parity_block(gpu, cpu):
    """Agreement of the GPU results with the oracle's on the same pairs: K, the
    sample label strings of pairs with K > 1, and the correlations of k < K."""
    Kg, Lg, Cg = gpu
    Kc, Lc, Cc = cpu
    same_k = Kg == Kc
    rows = same_k & (Kc > 1)
    labels_eq = np.all(Lg[rows] == Lc[rows], axis=1) if rows.any() else np.ones(0, bool)
    mask = (np.arange(Cc.shape[1])[None, :] < Kc[:, None]) & same_k[:, None]
    if Cc.ndim == 3:                      # [pair][k][Pearson, Spearman]
        mask = np.broadcast_to(mask[:, :, None], Cc.shape)
    a, b = Cg[mask], Cc[mask]
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    both = ~nan_a & ~nan_b
    dr = float(np.max(np.abs(a[both] - b[both]))) if both.any() else 0.0
    return {"pairs": int(len(Kc)), "k_agreement": float(same_k.mean()),
            "label_agreement": float(labels_eq.mean()) if len(labels_eq) else 1.0,
            "label_rows": int(rows.sum()), "correlations": int(mask.sum()),
            "nan_mismatches": int((nan_a != nan_b).sum()), "max_abs_dr": dr,
            "k_histogram": np.bincount(np.asarray(Kc, np.int64)).tolist(),
            "bit_exact": bool(np.array_equal(Kg, Kc) and (not rows.any() or labels_eq.all())
                              and np.array_equal(a.view(np.uint32), b.view(np.uint32))),
            "vs": "oracle: C restatement of KINC's serial path, pinned bit-exact to KINC's compiled Pairwise code"}


def libm_leg():
    """The GPU on the clustering workloads' 64-gene matrices (tests/golden/libm: 2,016 pairs each, GMM
    k <= 5 + Spearman at 1,000 samples, K-means k <= 3 + Pearson at 4,000, GMM ICL + both correlations
    at 500): bit-exactness against KINC's own code with the portable exp/log (math mode 0), and the
    agreement with KINC built against glibc's float (mode 1) and double (mode 2) exp/log -- and of
    those two builds with each other, the spread that is the reference's own."""
    from kinc_gb300 import Similarity
    from oracle import agreement
    names = {0: "none", 1: "gmm", 2: "kmeans"}
    out = {}
    for name, path in agreement.cases().items():
        fx = agreement.load(path)
        a = fx["params"]
        sim = Similarity(fx["gem"], clusmethod=names[a["clus_method"]],
                         corrmethod=2 if fx["ncorr"] == 2 else a["corr_method"], minsamp=a.get("min_samples", 30),
                         minclus=a.get("min_clusters", 1), maxclus=a["max_clusters"], crit=a["criterion"],
                         preout=a.get("pre_out", 0), postout=a.get("post_out", 0))
        sim.initialize()
        res = sim.execute(None, start=0, size=len(fx["K0"]))
        sim.close()
        exact = bool(np.array_equal(res.K, fx["K0"])
                     and np.array_equal(agreement.row_hashes(res.labels), fx["hash0"])
                     and np.array_equal(np.nan_to_num(res.corr, nan=9.0).view(np.uint32),
                                        np.nan_to_num(fx["corr0"], nan=9.0).view(np.uint32)))
        entry = {"pairs": int(len(res.K)), "samples": int(fx["gem"].shape[1]),
                 "k_histogram": np.bincount(res.K.astype(np.int64)).tolist(), "bit_exact_vs_mode0": exact}
        for mode in (1, 2):
            entry[f"vs_mode{mode}"] = agreement.compare(res.K, res.labels, res.corr, fx, mode)
        entry["mode1_vs_mode2"] = agreement.compare_modes(fx)
        out[name] = entry
    return out


def run_reference(args, gem):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ppt = args.ref_pairs_per_thread
    for i in range(args.warmup):
        cpu_sample(gem, threads, ppt, seed=1000 + i)
    tot_pairs, tot_secs = 0, 0.0
    for i in range(args.steps):
        _, n, s = cpu_sample(gem, threads, ppt, seed=2000 + i)
        tot_pairs += n
        tot_secs += s
    value = tot_pairs / tot_secs
    line = {
        "impl": "reference", "metric": "gene pairs/sec", "value": value, "unit": "pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded; no public dataset)",
        "config": config_dict(args, gem),
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"{threads} threads x {ppt} consecutive pairs from seeded random work blocks "
                                   f"per step, oracle C restatement of KINC's serial path"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def dense_leg(L, vp, check_pairs=1000000):
    """Pearson without clustering on the dense 20,000 x 2,000 workload (kinc_gb300.synthetic workload 3:
    rank-50 factors + noise, per-gene NaN rate ~U(0,0.2)): all 199,990,000 pairs with the tcgen05 tensor-core
    form (TF32, 3xBF16 and scaled FP16), the same contraction tiled in FP32 on the CUDA cores (the comparator
    for the tensor-core forms), and a 1,048,576-pair block with the plain per-pair FP32 kernel, all
    device-resident and timed with CUDA events; max |r - r_fp64| over a seeded random subset."""
    import ctypes

    import torch

    from kinc_gb300 import Similarity, _native, synthetic
    from oracle import pyoracle
    gem = synthetic.generate(3)
    G, S = gem.shape
    total = G * (G - 1) // 2
    rng = np.random.default_rng(20260103)
    idx = np.sort(rng.choice(total, size=min(check_pairs, total), replace=False))
    x, y = pyoracle.pair_xy(idx)
    ref = pyoracle.pearson_fp64_pairs(gem, x, y)
    ok = ~np.isnan(ref)
    out = {"workload": "Pearson, no clustering, GEM 20000x2000 float32, rank-50 factors + N(0,0.5) noise, "
                       "per-gene NaN rate ~U(0,0.2), pairwise-complete (semantics fixed)",
           "pairs": total, "fp64_check_pairs": int(len(idx))}
    stream = torch.cuda.Stream()
    for prec in ("tf32", "3xbf16", "fp16", "fp32tiled", "fp32"):
        sim = Similarity(gem, semantics="fixed", precision=prec, maxclus=1)
        sim.initialize()
        ctx = sim._ctx
        mb = L.kinc_sim_max_device_block(ctx)
        n_run = total if prec != "fp32" else min(1 << 20, total)
        chunk = min(mb, n_run)
        dK = torch.empty(chunk, dtype=torch.int8, device="cuda")
        dC = torch.empty((chunk, 1), dtype=torch.float32, device="cuda")
        dL = torch.empty((chunk, S), dtype=torch.int8, device="cuda") if prec == "fp32" else None
        got = np.empty(n_run, np.float32)

        def run(keep):
            for s0 in range(0, n_run, chunk):
                n = min(chunk, n_run - s0)
                rc = L.kinc_sim_execute_block_device(ctx, s0, n, vp(dK.data_ptr()),
                                                     vp(dL.data_ptr()) if dL is not None else None,
                                                     vp(dC.data_ptr()), vp(stream.cuda_stream))
                _native.check(rc, ctx)
                if keep:
                    stream.synchronize()
                    got[s0:s0 + n] = dC[:n, 0].cpu().numpy()
        with torch.cuda.stream(stream):
            run(True)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            reps = 3 if prec in ("tf32", "3xbf16", "fp16") else 1
            e0.record(stream)
            for _ in range(reps):
                run(False)
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        _native.check(L.kinc_sim_synchronize(ctx), ctx)
        sim.close()
        entry = {"pairs_timed": int(n_run), "ms": ms, "pairs_per_s": n_run / (ms / 1e3)}
        sel = idx < n_run
        if sel.any():
            g = got[idx[sel]].astype(np.float64)
            m = ok[sel]
            entry["max_abs_err_vs_fp64"] = float(np.abs(g[m] - ref[sel][m]).max())
            entry["fp64_pairs_compared"] = int(m.sum())
        if prec != "fp32":
            useful = 12.0 * S * n_run / (ms / 1e3) / 1e12
            entry["useful_tflops"] = useful
        out[prec] = entry
    peaks = os.path.join(REPO, "MEASURED_PEAKS.json")
    bf16 = 1893.1
    if os.path.exists(peaks):
        with open(peaks) as fh:
            bf16 = float(json.load(fh).get("bf16_tflops", bf16))
    # the tcgen05 MMA rate itself, measured here on operands resident in shared memory
    mma = {}
    for prec, name in ((1, "tf32"), (2, "bf16")):
        v = ctypes.c_double(0.0)
        _native.check(L.kinc_sim_tensor_peak(prec, ctypes.byref(v)), None)
        mma[name] = v.value
    out["tf32"]["frac_of_tf32_peak"] = out["tf32"]["useful_tflops"] / (bf16 / 2)
    out["tf32"]["frac_of_tf32_mma_peak"] = out["tf32"]["useful_tflops"] / mma["tf32"]
    out["3xbf16"]["executed_tflops"] = 2 * out["3xbf16"]["useful_tflops"]
    out["3xbf16"]["frac_of_bf16_peak"] = out["3xbf16"]["executed_tflops"] / bf16
    out["3xbf16"]["frac_of_bf16_mma_peak"] = out["3xbf16"]["executed_tflops"] / mma["bf16"]
    out["fp16"]["frac_of_f16_peak"] = out["fp16"]["useful_tflops"] / bf16
    out["fp16"]["frac_of_f16_mma_peak"] = out["fp16"]["useful_tflops"] / mma["bf16"]
    out["mma_peak_tflops"] = mma
    out["peak_note"] = (f"frac_of_tf32_peak: half the measured bf16 library-GEMM burst ({bf16:.0f} TFLOP/s, "
                        "MEASURED_PEAKS.json); frac_of_*_mma_peak: the tcgen05 MMA rate measured in this run "
                        "(kinc_sim_tensor_peak, operands resident in shared memory: "
                        f"TF32 {mma['tf32']:.0f}, BF16 {mma['bf16']:.0f} TFLOP/s); 3xBF16 executes 2x the "
                        "useful flops of the TF32 form; FP16 (kind::f16, the BF16 rate) is compared with the "
                        "bf16 burst and the BF16 MMA rate")
    sm_max = 2070.0
    if os.path.exists(peaks):
        with open(peaks) as fh:
            sm_max = float(json.load(fh).get("sm_max_mhz", sm_max))
    fp32_peak = torch.cuda.get_device_properties(0).multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
    out["fp32tiled"]["frac_of_fp32_peak"] = out["fp32tiled"]["useful_tflops"] / fp32_peak
    out["fp32tiled"]["peak_note"] = (f"nominal FP32 FMA rate {fp32_peak:.1f} TFLOP/s; 12 useful flops per pair and "
                                     f"sample are 6 FFMA")
    out["speedup_tf32_vs_fp32_tiled"] = out["tf32"]["pairs_per_s"] / out["fp32tiled"]["pairs_per_s"]
    out["speedup_3xbf16_vs_fp32_tiled"] = out["3xbf16"]["pairs_per_s"] / out["fp32tiled"]["pairs_per_s"]
    out["speedup_fp16_vs_fp32_tiled"] = out["fp16"]["pairs_per_s"] / out["fp32tiled"]["pairs_per_s"]
    out["speedup_tf32_vs_fp32_per_pair"] = out["tf32"]["pairs_per_s"] / out["fp32"]["pairs_per_s"]
    out["speedup_3xbf16_vs_fp32_per_pair"] = out["3xbf16"]["pairs_per_s"] / out["fp32"]["pairs_per_s"]
    return out


def pearson_leg(L, vp, cpu=True):
    """Pearson without clustering on the 1,000 x 200 workload (kinc_gb300.synthetic workload 1: gene means
    ~U(4,12), N(mean, 2), 5% NaN; minsamp 30, mincorr 0.5), reference semantics -- KINC's packed-array
    reads, stale values of earlier pairs of the work block included: all 499,500 pairs as one device block
    timed with CUDA events, and end to end into CCM/CMX files; the oracle over all pairs on the host cores
    (one thread per 32,768-pair work block), its CMX/CCM items compared with the files bit for bit."""
    import shutil
    import tempfile

    import torch

    from kinc_gb300 import Similarity, _native, pairwise_matrix as pm, synthetic
    from oracle import pyoracle
    gem = synthetic.generate(1)
    G, S = gem.shape
    total = G * (G - 1) // 2
    args = dict(clusmethod="none", corrmethod="pearson", minsamp=30, mincorr=0.5, maxcorr=1.0, maxclus=1)
    sim = Similarity(gem, **args)
    sim.initialize()
    ctx = sim._ctx
    dK = torch.empty(total, dtype=torch.int8, device="cuda")
    dL = torch.empty((total, S), dtype=torch.int8, device="cuda")
    dC = torch.empty((total, 1), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    reps = 5
    with torch.cuda.stream(stream):
        def once():
            _native.check(L.kinc_sim_execute_block_device(ctx, 0, total, vp(dK.data_ptr()), vp(dL.data_ptr()),
                                                          vp(dC.data_ptr()), vp(stream.cuda_stream)), ctx)
        once()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            once()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    _native.check(L.kinc_sim_synchronize(ctx), ctx)
    tmp = tempfile.mkdtemp(prefix="kinc_cfg1_")
    try:
        ccm, cmx = os.path.join(tmp, "a.ccm"), os.path.join(tmp, "a.cmx")
        t0 = time.perf_counter()
        sim.run(ccm_path=ccm, cmx_path=cmx)
        e2e_s = time.perf_counter() - t0
        got_cmx, got_ccm = pm.read(cmx, pm.CMX), pm.read(ccm, pm.CCM)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
        sim.close()
    # per (pair, sample) 8 flops: n, sums of x, y, x^2, y^2, xy
    out = {"workload": "Pearson only, GEM 1000x200 float32, gene means ~U(4,12), 5% NaN, minsamp 30, mincorr 0.5, "
                       "reference semantics (stale packed-array reads), all pairs",
           "pairs": total, "ms": ms, "pairs_per_s": total / (ms / 1e3),
           "e2e": {"seconds": e2e_s, "pairs_per_s": total / e2e_s,
                   "includes": "kinc_sim_run_to_files: compute, device process(), items to CCM/CMX files"},
           "achieved_tflops": 8.0 * S * total / (ms / 1e3) / 1e12, "cmx_items": int(len(got_cmx["x"]))}
    if cpu:
        threads = os.cpu_count() or 1
        nblk = (total + 32767) // 32768
        starts = np.arange(nblk, dtype=np.int64) * 32768
        sizes = np.minimum(32768, total - starts).astype(np.int64)
        p = pyoracle.params(clus_method=0, corr_method=0, min_samples=30, max_clusters=1, min_corr=0.5,
                            max_corr=1.0)
        done, secs, ref = pyoracle.run_segments_parallel(gem, p, starts, sizes, threads, outputs=True)
        # one pass over all pairs takes a few tens of ms: repeat it for a stable rate (~10 s)
        reps, rsecs = 1, secs
        while rsecs < 10.0 and reps < 2000:
            d, t = pyoracle.run_segments_parallel(gem, p, starts, sizes, threads)
            done += d
            rsecs += t
            reps += 1
        out["cpu_baseline"] = {"value": done / rsecs, "unit": "pairs/s", "cores": min(threads, nblk), "kind": "port",
                               "sample": f"all {total} pairs x {reps} passes, one thread per work block, "
                                         f"{rsecs:.1f} s"}
        out["gpu_over_cpu"] = out["pairs_per_s"] / out["cpu_baseline"]["value"]
        want_cmx, want_ccm = pyoracle.process_block(S, p, 0, *ref)
        same_cmx = (np.array_equal(got_cmx["x"], want_cmx["x"]) and np.array_equal(got_cmx["y"], want_cmx["y"])
                    and np.array_equal(got_cmx["c"], want_cmx["c"])
                    and np.array_equal(got_cmx["payload"][:, 0].view(np.uint32), want_cmx["r"].view(np.uint32)))
        same_ccm = len(got_ccm["x"]) == len(want_ccm["x"]) and np.array_equal(got_ccm["x"], want_ccm["x"]) \
            and np.array_equal(got_ccm["y"], want_ccm["y"])
        out["parity"] = {"cmx_items_gpu": int(len(got_cmx["x"])), "cmx_items_oracle": int(len(want_cmx["x"])),
                         "cmx_bit_exact": bool(same_cmx), "ccm_pairs_equal": bool(same_ccm),
                         "vs": "oracle: C restatement of KINC's serial path and Similarity::process"}
    return out


def kmeans_leg(L, vp, cpu=True):
    """K-means (k <= 3, BIC) + Pearson on the uneven 10,000 x 4,000 workload (kinc_gb300.synthetic workload 4:
    per-gene NaN rate ~U(0,0.6), so usable-sample counts span ~600-4,000; 5% planted 2-cluster pairs):
    two device blocks of 262,144 pairs timed with CUDA events (after a 32,768-pair warm-up block), and the
    oracle on the host cores over a bounded sample of the same workload."""
    import ctypes

    import torch

    from kinc_gb300 import Similarity, _native, synthetic
    from oracle import pyoracle
    gem = synthetic.generate(4)
    G, S = gem.shape
    args = dict(clusmethod="kmeans", corrmethod="pearson", minclus=1, maxclus=3, crit="BIC", minsamp=30)
    sim = Similarity(gem, **args)
    sim.initialize()
    chosen, _ = sim.autotune()      # launch shape for this workload (kinc_sim_autotune, cached)
    ctx = sim._ctx
    n = 262144
    dK = torch.empty(n, dtype=torch.int8, device="cuda")
    dL = torch.empty((n, S), dtype=torch.int8, device="cuda")
    dC = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        def once(s0, size=n):
            _native.check(L.kinc_sim_execute_block_device(ctx, s0, size, vp(dK.data_ptr()), vp(dL.data_ptr()),
                                                          vp(dC.data_ptr()), vp(stream.cuda_stream)), ctx)
        once(0, 32768)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        once(32768)
        once(32768 + n)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 2
    _native.check(L.kinc_sim_synchronize(ctx), ctx)
    sim.close()
    out = {"workload": "K-means k<=3 (BIC) + Pearson, GEM 10000x4000 float32, per-gene NaN rate ~U(0,0.6), "
                       "5% planted 2-cluster pairs, minsamp 30", "pairs_per_step": n, "ms_per_step": ms,
           "pairs_per_s": n / (ms / 1e3), "launch": chosen}
    if cpu:
        threads = os.cpu_count() or 1
        total = G * (G - 1) // 2
        rng = np.random.default_rng(11)
        starts = rng.choice((total - 1) // 32768, size=threads, replace=False).astype(np.int64) * 32768
        p = pyoracle.params(clus_method=2, corr_method=0, min_clusters=1, max_clusters=3, criterion=0, min_samples=30)
        sizes = np.full(threads, max(1, 16384 // threads), np.int64)      # ~20 s on 16 cores
        done, secs, ref = pyoracle.run_segments_parallel(gem, p, starts, sizes, threads, outputs=True)
        out["cpu_baseline"] = {"value": done / secs, "unit": "pairs/s", "cores": threads, "kind": "port",
                               "sample": f"{done} pairs: {threads} threads x {int(sizes[0])} consecutive pairs "
                                         f"from seeded random work blocks, {secs:.1f} s"}
        out["gpu_over_cpu"] = out["pairs_per_s"] / out["cpu_baseline"]["value"]
        chk = Similarity(gem, **args)
        parts = [chk.execute(None, int(a), int(b)) for a, b in zip(starts, sizes)]
        chk.close()
        out["parity"] = parity_block((np.concatenate([r.K for r in parts]), np.concatenate([r.labels for r in parts]),
                                      np.concatenate([r.corr for r in parts])), ref)
    return out


def stream_leg(device_block, nblk, cpu=True):
    """The large streamed run (kinc_gb300.synthetic workload 5: GEM 30,000 x 500, 8% NaN, 5% planted
    2-4 component mixture pairs; GMM k <= 5, ICL, pre+post outliers, Pearson and Spearman per cluster)
    end to end through kinc_sim_run_to_files_ex: `nblk` device blocks of `device_block` pairs from the
    middle of the 449,985,000 pairs, computed, filtered and compacted on the GPU, kept items streamed
    back through pinned buffers and written as CCM/CMX files.  Wall clock of the whole call."""
    import shutil
    import tempfile

    from kinc_gb300 import Similarity, synthetic
    gem = synthetic.generate(5)
    G, S = gem.shape
    sim = Similarity(gem, clusmethod="gmm", corrmethod="both", minclus=1, maxclus=5, crit="ICL", preout=True,
                     postout=True, minsamp=30, mincorr=0.5, maxcorr=1.0)
    sim.initialize()
    chosen, _ = sim.autotune()      # launch shape for this workload (kinc_sim_autotune, cached)
    wb_per_dev = device_block // 32768
    first = (sim.size() // 2) // wb_per_dev * wb_per_dev
    pairs = min(sim.total_pairs(), (first + nblk * wb_per_dev) * 32768) - first * 32768
    tmp = tempfile.mkdtemp(prefix="kinc_stream_")
    try:
        ccm, cmx = os.path.join(tmp, "out.ccm"), os.path.join(tmp, "out.cmx")
        t0 = time.perf_counter()
        sim.run(ccm_path=ccm, cmx_path=cmx, first_block=first, nblocks=nblk * wb_per_dev, device_block=device_block)
        secs = time.perf_counter() - t0
        ccm_bytes, cmx_bytes = os.path.getsize(ccm), os.path.getsize(cmx)
        items_cmx = (cmx_bytes - 31) // (9 + 8)
        items_ccm = (ccm_bytes - 34) // (9 + (S + 1) // 2)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
        sim.close()
    rate = pairs / secs
    extra = {}
    if cpu:
        # the oracle on the host cores over seeded random work blocks of the same workload, and the GPU on the
        # same pairs through the host-buffer entry point
        from oracle import pyoracle
        threads = os.cpu_count() or 1
        total = sim.total_pairs()
        rng = np.random.default_rng(55)
        starts = rng.choice((total - 1) // 32768, size=threads, replace=False).astype(np.int64) * 32768
        sizes = np.full(threads, max(1, 24576 // threads), np.int64)      # ~15 s on 16 cores
        p = pyoracle.params(clus_method=1, corr_method=2, min_clusters=1, max_clusters=5, criterion=1, pre_out=1,
                            post_out=1, min_samples=30)
        done, csecs, ref = pyoracle.run_segments_parallel(gem, p, starts, sizes, threads, outputs=True)
        chk = Similarity(gem, clusmethod="gmm", corrmethod="both", minclus=1, maxclus=5, crit="ICL", preout=True,
                         postout=True, minsamp=30)
        parts = [chk.execute(None, int(a), int(b)) for a, b in zip(starts, sizes)]
        chk.close()
        gpu = (np.concatenate([r.K for r in parts]), np.concatenate([r.labels for r in parts]),
               np.concatenate([r.corr for r in parts]))
        extra["cpu_baseline"] = {"value": done / csecs, "unit": "pairs/s", "cores": threads, "kind": "port",
                                 "sample": f"{done} pairs: {threads} threads x {int(sizes[0])} consecutive pairs "
                                           f"from seeded random work blocks, both correlations, {csecs:.1f} s"}
        extra["gpu_over_cpu"] = rate / extra["cpu_baseline"]["value"]
        extra["parity"] = parity_block(gpu, ref)
    return {**extra,
            "workload": "GMM k<=5 (ICL) + pre/post outliers + Pearson and Spearman per cluster, GEM 30000x500 "
                        "float32, 8% NaN, 5% planted 2-4 component mixture pairs, minsamp 30, mincorr 0.5",
            "pairs": int(pairs), "first_pair": int(first * 32768), "device_block": device_block,
            "device_blocks": nblk, "seconds": secs, "pairs_per_s": rate, "launch": chosen,
            "cmx_items": int(items_cmx), "ccm_items": int(items_ccm), "bytes_written": int(ccm_bytes + cmx_bytes),
            "projected_full_run_s": sim.total_pairs() / rate,
            "includes": "kinc_sim_run_to_files_ex: compute, device-side process(), pinned D2H of kept items "
                        "overlapped with the next block, CCM/CMX file writes"}


def rmt_leg(blocks=1000, size=5, cpu=True):
    """RMT thresholding (include/kinc_rmt.h) with the reference's defaults except a 0.01 threshold step,
    on a clique network of blocks x size genes (kinc_gb300.synthetic.clique_network): pruned matrices
    grow to a few thousand rows before the spacing test finds the threshold.  GPU wall clock of the
    whole analytic (pruned matrices in HBM, cuSOLVER eigenvalues, host unfolding) beside the oracle
    (numpy eigensolver, scipy spline) on the host cores, with the step sequences compared."""
    from kinc_gb300 import synthetic
    from kinc_gb300.rmt import RMT
    G, x, y, c, r = synthetic.clique_network(blocks, size)
    rmt = RMT(tstep=0.01)
    rmt.run(items=(x, y, c, r), genes=G, max_clusters=1, strict=False)      # warm-up (solver, allocations)
    t0 = time.perf_counter()
    thr, steps = rmt.run(items=(x, y, c, r), genes=G, max_clusters=1, strict=False)
    secs = time.perf_counter() - t0
    out = {"workload": f"RMT, clique network of {G} genes ({blocks} cliques of {size}), {len(r)} CMX items, "
                       "tstep 0.01, other arguments at the reference's defaults",
           "seconds": secs, "steps": int(len(steps)), "largest_pruned_matrix": int(steps[:, 1].max()),
           "threshold": thr}
    if cpu:
        from oracle import pyoracle
        t0 = time.perf_counter()
        want_t, want_steps = pyoracle.rmt_run(G, 1, x, y, c, r, threshold_step=0.01)
        csecs = time.perf_counter() - t0
        dchi = max((abs(float(a[2]) - b[2]) for a, b in zip(steps, want_steps)), default=0.0)
        out["cpu_baseline"] = {"seconds": csecs, "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": "the whole analytic: numpy (LAPACK) eigensolver, scipy Akima unfolding"}
        out["gpu_over_cpu"] = csecs / secs
        out["parity"] = {"same_threshold": bool((want_t is None and thr is None)
                                                or (want_t is not None and thr is not None
                                                    and np.float32(want_t) == np.float32(thr))),
                         "same_sizes": [int(a[1]) for a in steps] == [b[1] for b in want_steps],
                         "max_abs_dchi": dchi}
    return out


def config_dict(args, gem):
    G, S = gem.shape
    return {"workload": "GMM k<=5 + Spearman, GEM 5000x1000 float32, 10% NaN, 10 planted modules; "
                        "BIC, preout+postout, minsamp 30",
            "genes": G, "samples": S, "pairs_per_step": args.block, "global_batch": args.block,
            "clusmethod": "gmm", "corrmethod": "spearman", "minclus": 1, "maxclus": 5, "crit": "BIC",
            "semantics": "reference CPU path (bit-exact)", "l2": "256 MiB memset between steps"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--block", type=int, default=1048576)
    ap.add_argument("--ref-pairs-per-thread", type=int, default=128)
    ap.add_argument("--cpu-pairs-per-thread", type=int, default=3072, help="headline CPU sample (~60 s on 16 cores)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-dense", action="store_true")
    ap.add_argument("--no-kmeans", action="store_true")
    ap.add_argument("--no-rmt", action="store_true")
    ap.add_argument("--no-libm", action="store_true")
    ap.add_argument("--no-pearson", action="store_true")
    ap.add_argument("--no-tune-cache", action="store_true", help="time the launch shapes even if cached")
    ap.add_argument("--dense-check-pairs", type=int, default=1000000)
    ap.add_argument("--stream-blocks", type=int, default=2,
                    help="device blocks of 2^22 pairs in the streamed 30000x500 leg (0 = skip)")
    args = ap.parse_args()

    from kinc_gb300 import synthetic
    gem = synthetic.generate(WORKLOAD["workload"])

    if args.impl == "reference":
        if int(os.environ.get("WORLD_SIZE", "1")) > 1 and int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args, gem)
        return

    import ctypes

    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from kinc_gb300 import Similarity, _native
    L = _native.load()
    sim_args = {k: v for k, v in WORKLOAD.items() if k != "workload"}
    G, S = gem.shape
    total = G * (G - 1) // 2
    B = args.block
    nsteps = args.warmup + args.steps
    nfull = total // B
    if nfull < 1:
        raise SystemExit(f"--block {B} exceeds the {total} pairs of the workload")

    def block_start(i):
        """Rank-disjoint consecutive device blocks; ranges wrap around the workload
        only when ranks x steps x block exceed its pairs."""
        return ((rank * nsteps + i) % nfull) * B

    sim = Similarity(gem, **sim_args)
    sim.initialize()
    ctx = sim._ctx
    maxk = sim.params.max_clusters
    # launch shape picked by the autotuner (kinc_sim_autotune, cached per shape and GPU) before any timing
    t0 = time.perf_counter()
    chosen, timed = sim.autotune(use_cache=not args.no_tune_cache)
    autotune = {"chosen": chosen, "candidates": timed, "seconds": time.perf_counter() - t0,
                "sample_pairs": 4 * 32 * 16 * 152, "from_cache": len(timed) == 0}
    dK = torch.empty(B, dtype=torch.int8, device="cuda")
    dL = torch.empty((B, S), dtype=torch.int8, device="cuda")
    dC = torch.empty((B, maxk), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    vp = ctypes.c_void_p

    def step(i):
        flush.zero_()
        rc = L.kinc_sim_execute_block_device(ctx, block_start(i), B, vp(dK.data_ptr()), vp(dL.data_ptr()),
                                             vp(dC.data_ptr()), vp(stream.cuda_stream))
        _native.check(rc, ctx)
        return L.kinc_sim_last_launch_count(ctx)

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step(i)
        torch.cuda.synchronize()
        counters = (ctypes.c_uint64 * 4)()
        _native.check(L.kinc_sim_work_counters(ctx, counters, 1), ctx)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        launches = 0
        for i in range(args.warmup, nsteps):
            launches += step(i)
        ev1.record(stream)
        torch.cuda.synchronize()
        clk = clocks.stop()
        ms = ev0.elapsed_time(ev1)
        _native.check(L.kinc_sim_synchronize(ctx), ctx)
        _native.check(L.kinc_sim_work_counters(ctx, counters, 1), ctx)
    units, fits = int(counters[0]), int(counters[1])
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.barrier()
    ms_max = float(t.item())
    value = world * args.steps * B / (ms_max / 1e3)
    sim.close()

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        hK = torch.empty(B, dtype=torch.int8, pin_memory=True)
        hL = torch.empty((B, S), dtype=torch.int8, pin_memory=True)
        hC = torch.empty((B, maxk), dtype=torch.float32, pin_memory=True)
        gem_pinned = torch.from_numpy(gem).pin_memory()
        e2e_steps = max(1, min(args.steps, 3))
        params = _native.SimParams()
        params_src = Similarity(gem, **sim_args).params
        ctypes.memmove(ctypes.byref(params), ctypes.byref(params_src), ctypes.sizeof(params))
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c2 = ctypes.c_void_p()
        _native.check(L.kinc_sim_create(vp(gem_pinned.data_ptr()), G, S, ctypes.byref(params), ctypes.byref(c2)))
        for i in range(e2e_steps):
            rc = L.kinc_sim_execute_block(c2, block_start(args.warmup + i), B, vp(hK.data_ptr()), vp(hL.data_ptr()),
                                          vp(hC.data_ptr()))
            _native.check(rc, c2)
        L.kinc_sim_destroy(c2)
        secs = time.perf_counter() - t0
        tt = torch.tensor([secs], dtype=torch.float64, device="cuda")
        if world > 1:
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        secs = float(tt.item())
        e2e = {"value": world * e2e_steps * B / secs, "unit": "pairs/s",
               "h2d_bytes_per_step": int(gem.nbytes // e2e_steps),
               "d2h_bytes_per_step": int(B * (1 + S + 4 * maxk)),
               "steps": e2e_steps,
               "includes": "kinc_sim_create (matrix upload) + execute_block into pinned host arrays + destroy"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- roofline of the similarity kernel (algorithmic FP32 flops of the EM units)
    peaks_path = os.path.join(REPO, "MEASURED_PEAKS.json")
    sm_max = 2070.0
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            sm_max = float(json.load(fh).get("sm_max_mhz", sm_max))
    props = torch.cuda.get_device_properties(local)
    fp32_peak = props.multi_processor_count * 128 * 2 * sm_max * 1e6 / 1e12
    achieved = units * FLOPS_PER_UNIT / (ms / 1e3) / 1e12
    traffic = None
    issue = None
    tpath = os.path.join(REPO, "profiles", "k_similarity_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tj = json.load(fh)
        traffic = tj.get("bytes_per_pair", 0) * B   # DRAM bytes of one launch (one step), scaled from the capture
        tpu = tj.get("thread_inst_per_unit")
        if tpu:
            # the bound that binds: instruction issue (exp/log are polynomials, sums are ordered float adds)
            lane_peak = props.multi_processor_count * 4 * 32 * sm_max * 1e6
            rate = units * tpu / (ms / 1e3)
            issue = {"thread_inst_per_unit": tpu, "achieved_thread_inst_per_s": rate,
                     "peak_thread_inst_per_s": lane_peak, "frac": rate / lane_peak,
                     "source": "thread instructions per unit from the ncu capture in profiles/"}
    roofline = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak, "traffic": traffic,
                "peak_source": f"nominal FP32 FMA rate: {props.multi_processor_count} SMs x 128 lanes x 2 flops x "
                               f"{sm_max:.0f} MHz (MEASURED_PEAKS.json holds no FP32 figure)",
                "kernel": "k_similarity", "units": units, "flops_per_unit": FLOPS_PER_UNIT, "fits": fits,
                "issue_frac": issue["frac"] if issue else None, "issue": issue}

    tensor_core = None if args.no_dense else dense_leg(L, vp, args.dense_check_pairs)
    kmeans = None if args.no_kmeans else kmeans_leg(L, vp, cpu=not args.no_cpu)
    pearson = None if args.no_pearson else pearson_leg(L, vp, cpu=not args.no_cpu)
    streamed = None if args.stream_blocks <= 0 else stream_leg(1 << 22, args.stream_blocks, cpu=not args.no_cpu)
    rmt = None if args.no_rmt else rmt_leg(cpu=not args.no_cpu)
    libm = None if args.no_libm else libm_leg()

    cpu = None
    parity = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        v, n, s, starts, sizes, ref = cpu_sample(gem, threads, args.cpu_pairs_per_thread, seed=7, outputs=True)
        cpu = {"value": v, "unit": "pairs/s", "cores": threads, "kind": "port",
               "sample": f"{n} pairs: {threads} threads x {args.cpu_pairs_per_thread} consecutive pairs from "
                         f"seeded random work blocks, {s:.1f} s"}
        # the same pairs on the GPU, through the host-buffer entry point
        chk = Similarity(gem, **sim_args)
        parts = [chk.execute(None, int(a), int(b)) for a, b in zip(starts, sizes)]
        chk.close()
        gpu = (np.concatenate([r.K for r in parts]), np.concatenate([r.labels for r in parts]),
               np.concatenate([r.corr for r in parts]))
        parity = parity_block(gpu, ref)

    line = {"metric": "gene pairs/sec", "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded; no public dataset)",
            "config": config_dict(args, gem), "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
            "cpu_baseline": cpu, "parity": parity, "clocks": clk, "tensor_core": tensor_core, "kmeans_uneven": kmeans,
            "streamed_30000x500": streamed, "rmt": rmt, "libm_agreement": libm, "autotune": autotune,
            "pearson_1000x200": pearson}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
