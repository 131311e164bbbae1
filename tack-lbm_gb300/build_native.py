"""Build liblbm_gb300.so (the C ABI in include/lbm_gb300.h) for sm_103a.

    python tack-lbm_gb300/build_native.py [--force]

Each translation unit is compiled by its own nvcc process (in parallel) and
the objects are linked into ``tack-lbm_gb300/liblbm_gb300.so``. A stamp file
records a hash of the sources and flags, so an up-to-date library is not
rebuilt.
"""

import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblbm_gb300.so")
UNITS = ["lbm_api.cu", "lbm_kernels_f32.cu", "lbm_kernels_f16.cu", "lbm_kernels_bf16.cu",
         "lbm_kernels_f64.cu", "lbm_static_sums.cu", "lbm_adjoint.cu",
         "lbm_heat.cu", "lbm_derived.cu", "lbm_wing.cu", "lbm_fsi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-diag-suppress", "128", "-I", os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")
    return exe


def _digest():
    h = hashlib.sha256()
    h.update(" ".join(ARCH + FLAGS).encode())
    names = sorted(os.listdir(CSRC)) + ["../../include/lbm_gb300.h"]
    for name in names:
        path = os.path.normpath(os.path.join(CSRC, name))
        if os.path.isfile(path):
            h.update(name.encode())
            with open(path, "rb") as f:
                h.update(f.read())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile and link the library; return its path."""
    stamp = os.path.join(BUILD, "stamp")
    digest = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_unit(unit):
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        cmd = [exe, *ARCH, *FLAGS, "-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    args = ap.parse_args()
    print(build(force=args.force, verbose=args.verbose))
