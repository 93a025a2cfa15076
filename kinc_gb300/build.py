"""Build the native library of the package in-tree.

``libkinc_gb300.so`` holds the CUDA Similarity worker and its C ABI
(include/kinc_sim.h).  It is compiled for sm_103a only, with --fmad=false:
the worker reproduces the reference's floating-point operation sequence and
must not let the compiler contract a*b+c (kinc_fmath.h uses explicit fmaf).
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libkinc_gb300.so")
CLI = os.path.join(OUT_DIR, "kinc-gb300")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", os.path.join(REPO, "include"), "-I", CSRC]
# extra nvcc flags for the CUDA units, e.g. KINC_BUILD_FLAGS="-DKINC_GMM_PACKED=0" to time a compile-time
# variant (every variant gives the same results); pass force=True after changing it
EXTRA = os.environ.get("KINC_BUILD_FLAGS", "").split()

# (source, extra flags); kinc_cli.cpp is the command-line program, linked against the library
CLI_SRC = "kinc_cli.cpp"
UNITS = [
    ("kinc_sim.cu", ["--fmad=false"]),
    ("sim_none.cu", ["--fmad=false"]),
    ("sim_gmm.cu", ["--fmad=false"]),
    ("sim_kmeans.cu", ["--fmad=false"]),
    ("pearson_gemm.cu", []),
    ("compact.cu", []),
    ("pairwise_file.cpp", []),
    ("text_io.cpp", []),
    ("shard.cpp", []),
    ("rmt.cu", []),
]


def _sources():
    return [os.path.join(CSRC, s) for s, _ in UNITS if os.path.exists(os.path.join(CSRC, s))]


def _deps():
    out = []
    for d in (CSRC, os.path.join(REPO, "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def up_to_date():
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False):
    """Compile every CUDA unit in parallel and link the shared library."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs = []
    for src, flags in UNITS:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [NVCC, *ARCH, *COMMON, *flags, *EXTRA, "-c", path, "-o", obj]
        jobs.append((cmd, obj))

    def run(job):
        cmd, obj = job
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    subprocess.check_call([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lcusolver"])
    os.replace(tmp, LIB)
    # the command-line program finds the library next to itself
    tmp = CLI + ".tmp"
    subprocess.check_call([NVCC, *COMMON, os.path.join(CSRC, CLI_SRC), "-o", tmp, "-L", OUT_DIR, "-lkinc_gb300",
                           "-Xlinker", "-rpath=$ORIGIN"])
    os.replace(tmp, CLI)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
