"""Run and time device blocks of one synthetic workload through the worker.

    python -m kinc_gb300.blockrun --workload 2 --clusmethod gmm --corrmethod spearman \\
        --crit BIC --preout --postout --blocks 32768,262144

Each entry of --blocks is one kinc_sim_execute_block_device call of that many
pairs, taken consecutively from --start (default: pair 0; "mid" = the work
block in the middle of the workload), timed with CUDA events on a stream of
its own.  Prints one line per block with the time, pairs/s and the clustering
work counters (model units = iterations x N x K summed over fits), so a single
kernel launch can be captured by a profiler with -s/-c on k_similarity.
"""
import argparse
import ctypes
import json

from . import Similarity, _native, synthetic


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", type=int, default=2, help="kinc_gb300.synthetic workload (1-5)")
    ap.add_argument("--clusmethod", default="gmm")
    ap.add_argument("--corrmethod", default="spearman")
    ap.add_argument("--crit", default="BIC")
    ap.add_argument("--minclus", type=int, default=1)
    ap.add_argument("--maxclus", type=int, default=5)
    ap.add_argument("--minsamp", type=int, default=30)
    ap.add_argument("--preout", action="store_true")
    ap.add_argument("--postout", action="store_true")
    ap.add_argument("--semantics", default="reference")
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--start", default="0", help="first pair, or 'mid'")
    ap.add_argument("--blocks", default="32768,262144", help="comma-separated device block sizes")
    ap.add_argument("--repeat", type=int, default=1, help="run each block this many times from the same pair")
    ap.add_argument("--launch", default="", help="launch shape warps_per_cta,rounds,prefetch (default: the "
                                                 "worker's); 'tune' = kinc_sim_autotune with its cache")
    ap.add_argument("--tune-grid", action="store_true",
                    help="run kinc_sim_autotune (no cache) on its default sample block, then time every launch "
                         "shape on that block and print the pick beside the best of the grid")
    ap.add_argument("--genes", type=int, default=0, help="override the workload's gene count")
    ap.add_argument("--samples", type=int, default=0, help="override the workload's sample count")
    args = ap.parse_args(argv)

    import torch

    over = {k: v for k, v in (("genes", args.genes), ("samples", args.samples)) if v}
    gem = synthetic.generate(args.workload, **over)
    G, S = gem.shape
    sim = Similarity(gem, clusmethod=args.clusmethod, corrmethod=args.corrmethod, crit=args.crit,
                     minclus=args.minclus, maxclus=args.maxclus, minsamp=args.minsamp, preout=args.preout,
                     postout=args.postout, semantics=args.semantics, precision=args.precision)
    sim.initialize()
    if args.tune_grid:
        tune_grid(sim, args)
        sim.close()
        return
    if args.launch == "tune":
        sim.autotune()
    elif args.launch:
        sim.set_launch(*[int(v) for v in args.launch.split(",")])
    L = _native.load()
    ctx = sim._ctx
    vp = ctypes.c_void_p
    sizes = [int(b) for b in args.blocks.split(",") if b]
    pos = (sim.total_pairs() // 2) // 32768 * 32768 if args.start == "mid" else int(args.start)
    n = max(sizes)
    nc = 2 if sim.params.corr_method == 2 else 1
    dK = torch.empty(n, dtype=torch.int8, device="cuda")
    dL = torch.empty((n, S), dtype=torch.int8, device="cuda") if args.precision == "fp32" else None
    dC = torch.empty((n, sim.params.max_clusters * nc), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()   # the worker's stream argument 0 would mean its own stream
    counters = (ctypes.c_uint64 * 4)()
    for size in [b for b in sizes for _ in range(max(1, args.repeat))]:
        _native.check(L.kinc_sim_work_counters(ctx, counters, 1), ctx)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        labels = vp(dL.data_ptr()) if dL is not None else None   # the tensor-core form writes no labels
        rc = L.kinc_sim_execute_block_device(ctx, pos, size, vp(dK.data_ptr()), labels, vp(dC.data_ptr()),
                                             vp(stream.cuda_stream))
        _native.check(rc, ctx)
        e1.record(stream)
        torch.cuda.synchronize()
        _native.check(L.kinc_sim_synchronize(ctx), ctx)
        _native.check(L.kinc_sim_work_counters(ctx, counters, 1), ctx)
        ms = e0.elapsed_time(e1)
        print(json.dumps({"workload": args.workload, "launch": sim.launch() if args.precision == "fp32" else None,
                          "start": pos, "pairs": size, "ms": ms,
                          "pairs_per_s": size / (ms / 1e3), "units": int(counters[0]), "fits": int(counters[1]),
                          "launches": int(L.kinc_sim_last_launch_count(ctx))}), flush=True)
        if args.repeat <= 1:
            pos += size
    sim.close()


def tune_grid(sim, args):
    """The autotuner's pick against every launch shape, on the sample block it times."""
    import time

    import torch
    L = _native.load()
    vp = ctypes.c_void_p
    wpb = sim.launch()["warps_per_cta"]             # the default shape: the kernel's full warp count
    warps = [w for w in (4, 8, 10, 16, 20) if w <= wpb and wpb % w == 0]
    t0 = time.perf_counter()
    chosen, cands = sim.autotune(use_cache=False)
    tune_s = time.perf_counter() - t0
    total = sim.total_pairs()
    size = int(min(4 * 32 * 16 * 152, total, L.kinc_sim_max_device_block(sim._ctx)))
    start = max(0, total // 2 - size // 2)          # Similarity.autotune's default block
    G, S = sim.expressions.shape
    nc = 2 if sim.params.corr_method == 2 else 1
    dK = torch.empty(size, dtype=torch.int8, device="cuda")
    dL = torch.empty((size, S), dtype=torch.int8, device="cuda")
    dC = torch.empty((size, sim.params.max_clusters * nc), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    grid = {}
    for w in warps:
        for r in (0, 1):
            for pf in (0, 4, 8, 16):
                sim.set_launch(w, r, pf)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                _native.check(L.kinc_sim_execute_block_device(sim._ctx, start, size, vp(dK.data_ptr()),
                                                              vp(dL.data_ptr()), vp(dC.data_ptr()),
                                                              vp(stream.cuda_stream)), sim._ctx)
                e1.record(stream)
                torch.cuda.synchronize()
                grid[f"{w},{r},{pf}"] = e0.elapsed_time(e1)
    best = min(grid, key=grid.get)
    pick = f"{chosen['warps_per_cta']},{chosen['rounds']},{chosen['prefetch']}"
    print(json.dumps({"workload": args.workload, "genes": int(G), "samples": int(S),
                      "sample_pairs": size, "autotune_s": tune_s, "autotune_candidates": len(cands),
                      "picked": pick, "picked_ms": grid[pick], "best": best, "best_ms": grid[best],
                      "picked_over_best": grid[pick] / grid[best], "grid_ms": grid}), flush=True)


if __name__ == "__main__":
    main()
