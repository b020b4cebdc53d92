"""Build the CUDA engine library in-tree: contrafold_gpu_gb300/libcontrafold_gb300.so.

Every translation unit in csrc/ is compiled for sm_103a only, in parallel,
then linked into one shared library that exports the C-ABI of
include/contrafold_gb300.h.  `-fmad=false` keeps every float add and multiply
separately rounded (the FP32 paths are bitwise parity targets).

Extra nvcc flags (for example -DCF_FLAT_WALK=0 to compare a kernel variant)
come from the environment variable CONTRAFOLD_GB300_NVCC_FLAGS; the flags of
the last build are recorded next to the library, and a change rebuilds it.

`--check` (build(check=True)) builds the same sources with -DCF_CHECK into
libcontrafold_gb300_check.so: every DP-table subscript of the fold kernels is
checked against its table's size and reported with printf instead of being
performed out of range.  Point the package at it with the environment
variable CONTRAFOLD_GB300_LIB to run the test suite against it.
"""
from __future__ import annotations

import concurrent.futures as cfut
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libcontrafold_gb300.so")
LIB_CHECK = os.path.join(HERE, "libcontrafold_gb300_check.so")
BUILD_DIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        [os.path.join(os.path.dirname(HERE), "include", "contrafold_gb300.h")]


def _extra_flags():
    return os.environ.get("CONTRAFOLD_GB300_NVCC_FLAGS", "").split()


def _stamp(lib: str) -> str:
    return lib + ".flags"


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return False
    try:
        with open(_stamp(lib)) as fh:
            if fh.read() != " ".join(_extra_flags()):
                return False
    except OSError:
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False, check: bool = False) -> str:
    """Compile and link the library (the checked variant with check=True);
    returns its path.  Skips the work when the library is newer than every
    source."""
    lib = LIB_CHECK if check else LIB
    if not force and up_to_date(lib):
        return lib
    bdir = BUILD_DIR + ("_check" if check else "")
    os.makedirs(bdir, exist_ok=True)
    cc = nvcc()
    srcs = _sources()
    flags = NVCC_FLAGS + (["-DCF_CHECK"] if check else []) + _extra_flags()

    def compile_one(src):
        obj = os.path.join(bdir, os.path.basename(src).replace(".cu", ".o"))
        cmd = [cc, *ARCH, *flags, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with cfut.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    with open(_stamp(lib), "w") as fh:
        fh.write(" ".join(_extra_flags()))
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, check="--check" in sys.argv))
