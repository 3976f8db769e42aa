"""In-tree build of the CUDA library ``lib/libctm_gb300.so`` (sm_103a).

Compiles every ``csrc/*.cu`` translation unit with nvcc in parallel and links
them into one shared library with the C ABI of ``include/ctm_gb300.h``.
"""

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "lib")
LIB = os.path.join(OUT, "libctm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    path = shutil.which("nvcc")
    if path is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libctm_gb300.so")
    return path


def _sources():
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cu"))


def _fingerprint():
    h = hashlib.sha256()
    inc = os.path.join(os.path.dirname(PKG), "include", "ctm_gb300.h")
    files = _sources() + sorted(os.path.join(SRC, f) for f in os.listdir(SRC)
                                if f.endswith((".cuh", ".h"))) + [inc]
    for f in files:
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Builds the library unless an up-to-date copy exists.  Returns its path.
    An installed copy of the package (no sources beside it) uses the library
    it was installed with."""
    inc = os.path.join(os.path.dirname(PKG), "include", "ctm_gb300.h")
    if not force and os.path.exists(LIB) and not os.path.exists(inc):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "build.stamp")
    fp = _fingerprint()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == fp:
                return LIB
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + ARCH + FLAGS + ["-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(fp)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
