"""Compile the CUDA sources in ../csrc into the in-tree shared library libstonewall.so.

    python -m stonewall.build            (from jeju-stonewall-lbm_gb300/)
    python -m stonewall.build --check    the bounds-checked build, libstonewall_check.so

The bounds-checked build compiles the same sources with -DSW_CHECK: every
computed element offset of the step kernels is tested against its plane and an
offset outside it is reported in the lattice's status word (SW_STATUS_BOUNDS)
instead of being used.  It is for tests; the product loads libstonewall.so.

One nvcc process per translation unit, run in parallel, then one link.  Only
sm_103a (GB300) code is generated.  The object files go to _build/ beside this
file; the library lands next to this file so that the package loads it without
any search path.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG_ROOT), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libstonewall.so")
LIB_CHECK = os.path.join(HERE, "libstonewall_check.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", CSRC, "-I", INCLUDE]
# translation units that must evaluate float expressions in source order
NO_FMAD = {"sw_aux.cu", "sw_geometry.cu"}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libstonewall.so")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(f) for f in files)


def _compile(src, verbose, check=False):
    obj = os.path.join(BUILD, ("check_" if check else "") + src[:-3] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + (["--fmad=false"] if src in NO_FMAD else []) + (["-DSW_CHECK"] if check else [])
    if verbose:
        cmd += ["-Xptxas", "-v"]
    cmd += ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False, check=False):
    """Build libstonewall.so (check: libstonewall_check.so) if any source is newer than it; returns its path."""
    lib = LIB_CHECK if check else LIB
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= _deps():
        return lib
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, check), srcs))
    if verbose:
        for (_, log), s in zip(results, srcs):
            print(f"== {s}\n{log}")
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lcudart"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, check="--check" in sys.argv))
