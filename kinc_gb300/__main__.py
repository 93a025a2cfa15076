"""Command line with KINC's analytic and argument names.

    python -m kinc_gb300 run similarity --input a.emx --ccm a.ccm --cmx a.cmx \\
        --clusmethod gmm --corrmethod spearman --minsamp 30 --maxclus 5 --crit BIC --preout --postout
    python -m kinc_gb300 run export-cmx --ccm a.ccm --cmx a.cmx --output a.txt
    python -m kinc_gb300 run extract --emx a.emx --ccm a.ccm --cmx a.cmx --output net.txt --graphml net.graphml
    python -m kinc_gb300 run rmt --input a.cmx --log rmt.log
    python -m kinc_gb300 run import-emx --input a.txt --output a.emx --nan NA --names a.genes
    python -m kinc_gb300 run export-emx --input a.emx --output b.txt --nan NA --names a.genes
    python -m kinc_gb300 run import-cmx --input a.txt --ccm a.ccm --cmx a.cmx --genes 100 --maxclusters 5 \\
        --samples 40 --corrname pearson
    python -m kinc_gb300 run merge --output a.cmx --inputs rank0.cmx rank1.cmx

Analytic names follow src/core/analyticfactory.cpp:49-55; arguments follow each
analytic's input class (src/core/similarity_input.cpp, exportcorrelationmatrix_input.cpp,
extract_input.cpp, rmt_input.cpp, importexpressionmatrix_input.cpp,
exportexpressionmatrix_input.cpp, importcorrelationmatrix_input.cpp), with the
reference's defaults.  Boolean arguments take no value or an explicit true/false.
Expression matrices are the EMX data section (include/kinc_pairwise_matrix.h);
gene and sample names, metadata in KINC, are text files with one name per line
(--names, --sample-names): written by import-emx, read by export-emx and
extract.  Files use the big-endian byte order unless --little-endian is given.
"""
import argparse
import math
import sys


def _bool(v):
    if isinstance(v, bool):
        return v
    if str(v).lower() in ("1", "true", "yes", "on"):
        return True
    if str(v).lower() in ("0", "false", "no", "off"):
        return False
    raise argparse.ArgumentTypeError(f"expected true or false, got {v!r}")


def _parser():
    ap = argparse.ArgumentParser(prog="python -m kinc_gb300", description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="command", required=True)
    run = sub.add_parser("run", help="run an analytic")
    an = run.add_subparsers(dest="analytic", required=True)

    def common(p):
        p.add_argument("--little-endian", action="store_true", help="little-endian files")

    sim = an.add_parser("similarity", help="expression matrix -> cluster matrix (CCM) + correlation matrix (CMX)")
    sim.add_argument("--input", required=True, help="expression matrix (EMX data section)")
    sim.add_argument("--ccm", help="output cluster matrix")
    sim.add_argument("--cmx", help="output correlation matrix")
    sim.add_argument("--clusmethod", default="none", choices=["none", "gmm", "kmeans"])
    sim.add_argument("--corrmethod", default="pearson", choices=["pearson", "spearman", "both"])
    sim.add_argument("--minexpr", type=float, default=-math.inf)
    sim.add_argument("--minsamp", type=int, default=30)
    sim.add_argument("--minclus", type=int, default=1)
    sim.add_argument("--maxclus", type=int, default=5)
    sim.add_argument("--crit", default="ICL", choices=["BIC", "ICL"])
    sim.add_argument("--preout", nargs="?", const=True, default=False, type=_bool)
    sim.add_argument("--postout", nargs="?", const=True, default=False, type=_bool)
    sim.add_argument("--mincorr", type=float, default=0.5)
    sim.add_argument("--maxcorr", type=float, default=1.0)
    sim.add_argument("--ksize", type=int, default=4096)
    sim.add_argument("--semantics", default="reference", choices=["reference", "fixed"])
    sim.add_argument("--precision", default="fp32", choices=["fp32", "tf32", "3xbf16", "fp32tiled", "fp16"])
    sim.add_argument("--autotune", action="store_true", help="pick the kernel launch shape by timing (cached)")
    sim.add_argument("--rand", default="glibc", choices=["glibc", "lcg"],
                     help="glibc: KINC's serial path; lcg: KINC's OpenCL worker (per-fit LCG GMM)")
    sim.add_argument("--first-block", type=int, default=0, help="first work block (for a shard)")
    sim.add_argument("--blocks", type=int, default=-1, help="work blocks to run (-1: to the end)")
    sim.add_argument("--world", type=int, help="ranks of a sharded run (with --rank): this rank's work blocks")
    sim.add_argument("--rank", type=int, default=0)
    sim.add_argument("--by-cost", nargs="?", const=True, default=False, type=_bool,
                     help="cut the ranks' ranges by estimated cost instead of block count")
    sim.add_argument("--resume", nargs="?", const=True, default=False, type=_bool,
                     help="continue an interrupted run: keep the files' whole work blocks, run the rest")
    common(sim)

    exp = an.add_parser("export-cmx", help="CMX + CCM -> text")
    exp.add_argument("--ccm", required=True)
    exp.add_argument("--cmx", required=True)
    exp.add_argument("--output", required=True)
    common(exp)

    ext = an.add_parser("extract", help="CMX + CCM + EMX -> network edge list and GraphML")
    ext.add_argument("--emx", required=True)
    ext.add_argument("--ccm", required=True)
    ext.add_argument("--cmx", required=True)
    ext.add_argument("--output", help="edge list (text)")
    ext.add_argument("--graphml", help="GraphML network")
    ext.add_argument("--mincorr", type=float, default=0.85)
    ext.add_argument("--maxcorr", type=float, default=1.0)
    ext.add_argument("--names", help="gene names, one per line")
    common(ext)

    rmt = an.add_parser("rmt", help="correlation threshold by random matrix theory")
    rmt.add_argument("--input", required=True, help="correlation matrix (CMX)")
    rmt.add_argument("--log", required=True)
    rmt.add_argument("--tstart", type=float, default=0.99)
    rmt.add_argument("--tstep", type=float, default=0.001)
    rmt.add_argument("--tstop", type=float, default=0.5)
    rmt.add_argument("--minpace", type=int, default=10)
    rmt.add_argument("--maxpace", type=int, default=40)
    rmt.add_argument("--bins", type=int, default=60)
    common(rmt)

    from .pairwise_matrix import TRANSFORMS
    iem = an.add_parser("import-emx", help="text -> expression matrix (EMX)")
    iem.add_argument("--input", required=True, help="text: one gene per line, name then one value per sample")
    iem.add_argument("--output", required=True, help="expression matrix (EMX data section)")
    iem.add_argument("--nan", help="token of a missing value")
    iem.add_argument("--samples", type=int, default=0, help="sample count; 0: the first line names the samples")
    iem.add_argument("--transform", default=TRANSFORMS[0], choices=TRANSFORMS)
    iem.add_argument("--names", help="gene names written here, one per line")
    iem.add_argument("--sample-names", help="sample names written here, one per line")
    common(iem)

    eem = an.add_parser("export-emx", help="expression matrix (EMX) -> text")
    eem.add_argument("--input", required=True)
    eem.add_argument("--output", required=True)
    eem.add_argument("--nan", help="token written for a missing value")
    eem.add_argument("--transform", default=TRANSFORMS[0], choices=TRANSFORMS,
                     help="the transform the matrix was imported with (undone on export)")
    eem.add_argument("--names", help="gene names, one per line")
    eem.add_argument("--sample-names", help="sample names, one per line")
    common(eem)

    icm = an.add_parser("import-cmx", help="text (as export-cmx writes it) -> CCM + CMX")
    icm.add_argument("--input", required=True)
    icm.add_argument("--ccm", required=True)
    icm.add_argument("--cmx", required=True)
    icm.add_argument("--genes", type=int, required=True)
    icm.add_argument("--maxclusters", type=int, required=True)
    icm.add_argument("--samples", type=int, required=True)
    icm.add_argument("--corrname", required=True, help="correlation name (KINC metadata; not stored in the files)")
    common(icm)

    mrg = an.add_parser("merge", help="the CCM or CMX files of a sharded run -> one file, in rank order")
    mrg.add_argument("--output", required=True)
    mrg.add_argument("--inputs", required=True, nargs="+", help="the ranks' files, in rank order")
    common(mrg)
    return ap


def main(argv=None):
    args = _parser().parse_args(argv)
    from . import _native
    from . import pairwise_matrix as pm
    try:
        if args.analytic == "similarity":
            import numpy as np

            from .similarity import Similarity
            if not args.ccm and not args.cmx:
                raise SystemExit("similarity: give --ccm and/or --cmx")
            gem = pm.read_emx(args.input, little_endian=args.little_endian)
            sim = Similarity(np.ascontiguousarray(gem), clusmethod=args.clusmethod, corrmethod=args.corrmethod,
                             minexpr=args.minexpr, minsamp=args.minsamp, minclus=args.minclus, maxclus=args.maxclus,
                             crit=args.crit, preout=args.preout, postout=args.postout, mincorr=args.mincorr,
                             maxcorr=args.maxcorr, ksize=args.ksize, semantics=args.semantics,
                             precision=args.precision, rand=args.rand)
            if args.autotune and args.precision == "fp32":
                sim.autotune()
            sim.run(ccm_path=args.ccm, cmx_path=args.cmx, little_endian=args.little_endian,
                    first_block=args.first_block, nblocks=args.blocks, world=args.world, rank=args.rank,
                    by_cost=args.by_cost, resume=args.resume)
            sim.close()
        elif args.analytic == "export-cmx":
            pm.export_text(args.ccm, args.cmx, args.output, little_endian=args.little_endian)
        elif args.analytic == "extract":
            if not args.output and not args.graphml:
                raise SystemExit("extract: give --output and/or --graphml")
            pm.extract(args.emx, args.ccm, args.cmx, tsv_path=args.output, graphml_path=args.graphml,
                       names_path=args.names, min_corr=args.mincorr, max_corr=args.maxcorr,
                       little_endian=args.little_endian)
        elif args.analytic == "rmt":
            from .rmt import RMT
            t, _ = RMT(tstart=args.tstart, tstep=args.tstep, tstop=args.tstop, minpace=args.minpace,
                       maxpace=args.maxpace, bins=args.bins).run(input=args.input, log=args.log,
                                                                 little_endian=args.little_endian)
            print(f"threshold: {t:g}")
        elif args.analytic == "import-emx":
            pm.import_emx_text(args.input, args.output, nan=args.nan, samples=args.samples, transform=args.transform,
                               gene_names_path=args.names, sample_names_path=args.sample_names,
                               little_endian=args.little_endian)
        elif args.analytic == "export-emx":
            pm.export_emx_text(args.input, args.output, nan=args.nan, transform=args.transform,
                               gene_names_path=args.names, sample_names_path=args.sample_names,
                               little_endian=args.little_endian)
        elif args.analytic == "merge":
            pm.concat(args.output, args.inputs, little_endian=args.little_endian)
        elif args.analytic == "import-cmx":
            pm.import_text(args.input, args.ccm, args.cmx, args.genes, args.maxclusters, args.samples,
                           little_endian=args.little_endian)
    except (_native.SimError, ValueError) as e:
        print(f"{args.analytic}: {e}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
