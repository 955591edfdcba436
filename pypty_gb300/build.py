"""Build the CUDA library of the path: ``pypty_gb300/_lib/libpypty_gb300.so``.

Three translation units (the C ABI and one launch path per window size) are compiled in
parallel with nvcc for sm_103a only and linked into one shared library with a plain C ABI
(``include/pypty_gb300.h``). A stamp of the source hash skips rebuilds when nothing changed.
"""
from __future__ import annotations

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libpypty_gb300.so"
UNITS = ["capi.cu", "path_w64.cu", "path_w128.cu", "path_w256.cu", "noalloc.cu", "optim.cu", "dft_gemm.cu", "layered.cu", "unet.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _nvcc() -> str:
    for cand in [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pypty_gb300")


def _source_hash() -> str:
    h = hashlib.sha256()
    files = sorted(os.listdir(CSRC)) + ["../../include/pypty_gb300.h"]
    for name in files:
        path = os.path.normpath(os.path.join(CSRC, name))
        if os.path.isfile(path):
            with open(path, "rb") as f:
                h.update(name.encode() + b"\0" + f.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library if needed; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(LIBDIR, LIBNAME + ".stamp")
    digest = _source_hash()
    if not force and os.path.exists(lib_path()) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return lib_path()
    nvcc = _nvcc()
    objs = [os.path.join(BUILD, u.replace(".cu", ".o")) for u in UNITS]

    def compile_one(unit, obj):
        cmd = [nvcc, *FLAGS, *ARCH, "-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (unit, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)

    with concurrent.futures.ThreadPoolExecutor(len(UNITS)) as ex:
        list(ex.map(compile_one, UNITS, objs))
    tmp = lib_path() + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib_path())
    with open(stamp, "w") as f:
        f.write(digest)
    return lib_path()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
