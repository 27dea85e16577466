"""In-tree build of the CUDA library ``libvivsim_gb300.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel and linked into
one shared library next to this file (``_build/``).  The per-operator translation units
are compiled with ``-fmad=false`` so that their arithmetic is the reference's
operation by operation; the fused step kernels keep FMA contraction.
"""

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
LIB_NAME = "libvivsim_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra flags
UNITS = {
    "vs_status.cu": [],
    "vs_ops_lbm.cu": ["-fmad=false"],
    "vs_ops_ib.cu": ["-fmad=false"],
    "vs_step.cu": [],
    "vs_adjoint.cu": [],
    "vs_post.cu": [],
    "vs_refine.cu": [],
    "vs_grad.cu": [],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build vivsim_gb300")


CHECKED_LIB_NAME = "libvivsim_gb300_checked.so"


def lib_path(checked=False):
    return os.path.join(OUT, CHECKED_LIB_NAME if checked else LIB_NAME)


def _common_flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                   "-I", os.path.join(ROOT, "include"), "-I", SRC]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, checked=False):
    """Compile and link; returns the library path.  Rebuilds only what changed.

    checked=True builds libvivsim_gb300_checked.so with -DVIVSIM_BOUNDS_CHECK: the grid
    kernels test every gather and scatter index and report VS_ERR_RANGE instead of
    touching memory outside their arrays (a slower library for debugging and the tests)."""
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cuh")]
    headers.append(os.path.join(ROOT, "include", "vivsim_gb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for unit, extra in UNITS.items():
        src = os.path.join(SRC, unit)
        obj = os.path.join(OUT, unit.replace(".cu", "_chk.o" if checked else ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers + [__file__]):
            jobs.append([cc, "-c", src, "-o", obj] + _common_flags() + extra +
                        (["-DVIVSIM_BOUNDS_CHECK"] if checked else []))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg)
    lib = lib_path(checked)
    if force or jobs or _stale(lib, objs):
        tmp = lib + ".tmp"
        run([cc, "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
