"""Build recipe for the checkers under oracle/ (TEST INFRASTRUCTURE ONLY).

* ``oracle/_build/libkinc_oracle.so`` -- the plain-C restatement
  (kinc_oracle.c).  Builds on any host (x86-64 or aarch64).
* ``oracle/_ref/libkinc_ocl.so`` -- KINC's OpenCL kernels compiled as C++ for
  the host (ref_shim/ocl_shim.h) and driven as the OpenCL worker drives them
  (ocl_driver.cpp); also only with the KINC tree.
* ``oracle/_ref/libkinc_ref{0,1,2}.so`` -- KINC's own CPU Pairwise:: sources,
  compiled unmodified from the KINC source tree with the stand-in ACE header
  in ref_shim/ and the restated serial driver ref_driver.cpp.  Only built when
  ``KINC_REFERENCE_DIR`` names a KINC tree; without it, libraries built earlier
  are used as they are, and none is built.
  The suffix is the math resolution (ref_shim/ace/core/core.h): 0 = the
  portable kinc_expf/kinc_logf the GPU uses, 1 = glibc float expf/logf,
  2 = the C library's double functions.

Everything is compiled with -ffp-contract=off so that x86 and Arm hosts give
identical results (GCC contracts a*b+c into FMA on Arm by default).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REF_SOURCES = ["pairwise_linalg.cpp", "pairwise_clustering.cpp", "pairwise_gmm.cpp",
               "pairwise_kmeans.cpp", "pairwise_correlation.cpp", "pairwise_pearson.cpp",
               "pairwise_spearman.cpp"]
FP_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC"]


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle():
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libkinc_oracle.so")
    srcs = [os.path.join(HERE, "kinc_oracle.c"), os.path.join(HERE, "kinc_oracle.h"),
            os.path.join(REPO, "kinc_gb300", "csrc", "kinc_fmath.h")]
    if _newer(out, srcs):
        return out
    cmd = ["gcc", "-std=c99", "-shared", *FP_FLAGS, "-o", out, srcs[0], "-lm", "-lpthread"]
    subprocess.check_call(cmd)
    return out


def ref_dir():
    """The KINC source tree named by KINC_REFERENCE_DIR, or None."""
    return os.environ.get("KINC_REFERENCE_DIR") or None


def reference_available():
    d = ref_dir()
    return d is not None and os.path.isfile(os.path.join(d, "src", "core", "pairwise_gmm.cpp"))


def _prebuilt(name, own_deps):
    """A library built earlier from the KINC tree, when the tree is not named now; None when it is
    missing or older than this repository's files it was built from."""
    path = os.path.join(HERE, "_ref", name)
    return path if _newer(path, own_deps) else None


def build_ref(math_mode=0):
    """Compile the KINC Pairwise:: sources where they lie; returns the .so path or None."""
    own = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "ref_shim", "ace", "core", "core.h"),
           os.path.join(HERE, "ref_shim", "pre.h"), os.path.join(REPO, "kinc_gb300", "csrc", "kinc_fmath.h")]
    if not reference_available():
        return _prebuilt(f"libkinc_ref{math_mode}.so", own)
    core = os.path.join(ref_dir(), "src", "core")
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, f"libkinc_ref{math_mode}.so")
    srcs = [os.path.join(core, s) for s in REF_SOURCES] + [os.path.join(HERE, "ref_driver.cpp")]
    deps = srcs + own
    if _newer(out, deps):
        return out
    cmd = ["g++", "-std=c++14", "-shared", *FP_FLAGS, "-w",
           f"-DKINC_REF_MATH={math_mode}",
           "-DCCMATRIX_H", "-DCORRELATIONMATRIX_H", "-DEXPRESSIONMATRIX_H",
           "-include", os.path.join(HERE, "ref_shim", "pre.h"),
           "-I", os.path.join(HERE, "ref_shim"), "-I", core,
           "-I", os.path.join(REPO, "kinc_gb300", "csrc"),
           "-o", out, *srcs]
    subprocess.check_call(cmd)
    return out


# KINC's OpenCL kernels in the order the OpenCL analytic concatenates them
# (src/core/similarity_opencl.cpp:37-46)
OCL_SOURCES = ["linalg.cl", "fetchpair.cl", "sort.cl", "outlier.cl", "gmm.cl", "kmeans.cl", "pearson.cl",
               "spearman.cl"]


def build_ocl():
    """Compile KINC's OpenCL kernels as C++ for the host, with ref_shim/ocl_shim.h and the
    worker restated in ocl_driver.cpp, into oracle/_ref/libkinc_ocl.so; None without the
    KINC tree.  The kernels are read where they lie and piped to the compiler; the one
    OpenCL-only construct in them, the vector literal "(float2) (a, b)"
    (src/opencl/fetchpair.cl:62), is rewritten to a constructor call on the way."""
    own = [os.path.join(HERE, "ocl_driver.cpp"), os.path.join(HERE, "ref_shim", "ocl_shim.h"),
           os.path.join(REPO, "kinc_gb300", "csrc", "kinc_fmath.h")]
    if not reference_available():
        return _prebuilt("libkinc_ocl.so", own)
    cl_dir = os.path.join(ref_dir(), "src", "opencl")
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "libkinc_ocl.so")
    srcs = [os.path.join(cl_dir, s) for s in OCL_SOURCES]
    deps = srcs + own
    if _newer(out, deps):
        return out
    import re
    text = ""
    for path in srcs:
        with open(path) as fh:
            text += f'#line 1 "{path}"\n' + fh.read() + "\n"
    text = re.sub(r"\(float2\)\s*\(", "float2(", text)
    text += '#include "ocl_driver.cpp"\n'
    cmd = ["g++", "-std=c++14", "-shared", *FP_FLAGS, "-w", "-fsigned-char", "-x", "c++",
           "-include", os.path.join(HERE, "ref_shim", "ocl_shim.h"),
           "-I", HERE, "-I", os.path.join(REPO, "kinc_gb300", "csrc"), "-o", out, "-"]
    subprocess.run(cmd, input=text.encode(), check=True)
    return out


def build_all():
    paths = [build_oracle()]
    for m in (0, 1, 2):
        paths.append(build_ref(m))
    paths.append(build_ocl())
    return paths


if __name__ == "__main__":
    for p in build_all():
        print(p if p else "reference tree not present: oracle/_ref not built", file=sys.stdout)
