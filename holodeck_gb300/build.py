"""Build the CUDA extension ``_build/libholodeck_gb300.so`` for sm_103a with nvcc.

Each translation unit under ``csrc/`` compiles in parallel to an object file and the objects are
linked into one shared library exposing the C ABI of ``include/holodeck_gb300.h``.  The grid
stages (density, hardening, strain) are compiled with ``-fmad=false`` so their FP64 arithmetic
rounds like the numpy / Cython code they replace.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
CHECKED_DIR = os.path.join(HERE, "_build_checked")   # the -DHGB_BOUNDS_CHECK variant
LIB_NAME = "libholodeck_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NO_FMA = {"hgb_density.cu", "hgb_hardening.cu", "hgb_strain.cu", "hgb_scatter.cu", "hgb_details.cu"}


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the holodeck_gb300 CUDA extension cannot be built")
    return path


def _sources():
    return sorted(fn for fn in os.listdir(CSRC) if fn.endswith((".cu", ".cpp")))


def _stale(lib_path):
    if not os.path.exists(lib_path):
        return True
    t_lib = os.path.getmtime(lib_path)
    deps = [os.path.join(CSRC, fn) for fn in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "holodeck_gb300.h")]
    return any(os.path.getmtime(d) > t_lib for d in deps)


def build(force=False, verbose=False, checked=False):
    """Compile every ``csrc/*.cu`` and link the shared library; returns its path.  ``checked``: the
    variant with the kernels' bounds checks compiled in (-DHGB_BOUNDS_CHECK: an index outside its
    array is skipped and flagged as HGB_STATUS_BOUNDS), built into ``_build_checked/`` and loaded
    when HOLODECK_GB300_CHECKED=1."""
    out_dir = CHECKED_DIR if checked else OUT_DIR
    lib_path = os.path.join(out_dir, LIB_NAME)
    os.makedirs(out_dir, exist_ok=True)
    srcs = _sources()
    objs = [os.path.join(out_dir, os.path.splitext(fn)[0] + ".o") for fn in srcs]
    if not force and not _stale(lib_path):
        return lib_path
    exe = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                     "-I", os.path.join(ROOT, "include"), "-I", CSRC] + (["-DHGB_BOUNDS_CHECK"] if checked else [])

    def one(fn):
        cmd = [exe, "-c", os.path.join(CSRC, fn), "-o", os.path.join(out_dir, os.path.splitext(fn)[0] + ".o")] + common
        if fn in NO_FMA:
            cmd.append("-fmad=false")
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {fn}:\n{res.stdout}\n{res.stderr}")
        return res.stdout + res.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(one, srcs))
    if verbose:
        for fn, log in zip(srcs, logs):
            sys.stderr.write(f"---- {fn}\n{log}")
    tmp = lib_path + ".tmp"
    res = subprocess.run([exe] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
