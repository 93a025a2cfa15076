"""Run the host-only tests against AddressSanitizer + UndefinedBehaviorSanitizer builds of the
library's host units (pairwise_file.cpp, text_io.cpp, shard.cpp) and of the oracle's C
restatement.  CPU only; not collected by pytest (run it directly):

    python tests/sanitize_host.py

The sanitizer builds go to a temporary folder.  The file runner's calls into the worker are
linked to stand-ins that are never reached by these tests.  Exit status: pytest's.
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "kinc_gb300", "csrc")
CUDA = "/usr/local/cuda"
SAN = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-g", "-O1", "-fPIC"]

STUBS = r"""
#include <stdint.h>
struct kinc_sim_ctx;
struct CUstream_st;
extern "C" {
int kinc_sim_compact_block_device() { return 2; }
int kinc_sim_execute_block_device() { return 2; }
int kinc_sim_get_params() { return 1; }
const char* kinc_sim_last_error() { return "worker not linked in the sanitizer build"; }
int64_t kinc_sim_max_device_block() { return 0; }
int64_t kinc_sim_num_work_blocks() { return 0; }
int kinc_sim_synchronize() { return 2; }
int64_t kinc_sim_total_pairs() { return 0; }
}
int kinc_sim_status_copy_async(kinc_sim_ctx*, uint64_t*, CUstream_st*) { return 2; }
"""

PLUGIN = r"""
import ctypes
from kinc_gb300 import _native
from oracle import pyoracle

REAL = _native.load()
L = ctypes.CDLL({pm!r})


class _Lib:
    # the sanitizer build's functions where it has them (the host file/text units), the
    # normal library's for the rest (the worker's)
    def __getattr__(self, name):
        fn = getattr(L, name, None) if name.startswith(("kinc_pm_", "kinc_emx_", "kinc_shard_")) else None
        return fn if fn is not None else getattr(REAL, name)


for name, (res, args) in _native.SIGNATURES.items():
    fn = getattr(L, name, None)
    if fn is not None:
        fn.restype, fn.argtypes = res, args
_native._lib = _Lib()

O = ctypes.CDLL({ko!r})
ref = pyoracle.lib()
for name in ("ko_rand_seed", "ko_rand_next", "ko_rand_skip", "ko_libc_rand", "ko_draws_per_pair",
             "ko_count_qualifying", "ko_run_block", "ko_run_segments_parallel", "ko_run_segments_parallel_out",
             "ko_process_block", "ko_pearson_fp64", "ko_pearson_fp64_batch"):
    f, g = getattr(O, name), getattr(ref, name)
    f.argtypes, f.restype = g.argtypes, g.restype
pyoracle._lib = O
"""

TESTS = ["tests/test_pairwise_files.py", "tests/test_text_io.py", "tests/test_oracle.py",
         "tests/test_similarity_host.py", "tests/test_shard_gloo.py", "tests/test_native_abi.py"]


def main():
    sys.path.insert(0, REPO)
    from kinc_gb300 import build
    build.build()                               # the normal library, so the tests' fixture finds it current
    tmp = tempfile.mkdtemp(prefix="kinc_san_")
    inc = ["-I", os.path.join(REPO, "include"), "-I", CSRC, "-I", os.path.join(CUDA, "include")]
    objs = []
    for src in ("pairwise_file.cpp", "text_io.cpp", "shard.cpp"):
        o = os.path.join(tmp, src + ".o")
        subprocess.check_call(["g++", "-std=c++17", *SAN, *inc, "-c", os.path.join(CSRC, src), "-o", o])
        objs.append(o)
    stubs = os.path.join(tmp, "stubs.cpp")
    with open(stubs, "w") as fh:
        fh.write(STUBS)
    subprocess.check_call(["g++", "-std=c++17", *SAN, "-c", stubs, "-o", stubs + ".o"])
    pm = os.path.join(tmp, "libpm_san.so")
    subprocess.check_call(["g++", "-shared", *SAN, "-o", pm, *objs, stubs + ".o", "-L", os.path.join(CUDA, "lib64"),
                           "-lcudart", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"])
    ko = os.path.join(tmp, "libkinc_oracle_san.so")
    subprocess.check_call(["gcc", "-std=c99", *SAN, "-ffp-contract=off", "-shared", "-o", ko,
                           os.path.join(REPO, "oracle", "kinc_oracle.c"), "-lm", "-lpthread"])
    with open(os.path.join(tmp, "san_plugin.py"), "w") as fh:
        fh.write(PLUGIN.format(pm=pm, ko=ko))
    libs = [subprocess.check_output(["gcc", f"-print-file-name={n}"], text=True).strip()
            for n in ("libasan.so", "libubsan.so")]
    env = dict(os.environ, LD_PRELOAD=":".join(libs), PYTHONPATH=tmp + os.pathsep + REPO,
               ASAN_OPTIONS="detect_leaks=0:protect_shadow_gap=0", UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    # multi-process cases start fresh interpreters that would not load the plugin: left out
    cmd = [sys.executable, "-m", "pytest", "-p", "san_plugin", "-p", "no:cacheprovider", "-q", "-x", "-s",
           "-m", "not gpu", "-k", "not two_ranks and not rank_files", *TESTS]
    return subprocess.call(cmd, cwd=REPO, env=env)


if __name__ == "__main__":
    sys.exit(main())
