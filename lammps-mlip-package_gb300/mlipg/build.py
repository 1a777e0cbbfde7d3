"""In-tree build of libmlipg.so for sm_103a (GB300).

Compiles the host model and C ABI (g++), the fused CUDA kernels (nvcc, one
translation unit per precision) in parallel, and links one shared library
next to this package: ``lammps-mlip-package_gb300/libmlipg.so``.  The coupling
table (``data/gtinv_table.txt``) is embedded into the library, so the .so is
self-contained.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # lammps-mlip-package_gb300
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmlipg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in [os.environ.get("CUDA_HOME"), "/usr/local/cuda"]:
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(nv))
    raise RuntimeError("nvcc not found")


def _embed_table():
    src = os.path.join(PKG, "data", "gtinv_table.txt")
    dst = os.path.join(OUT_DIR, "gtinv_table.inc")
    text = open(src).read()
    body = 'static const char kGtinvTableText[] = R"GTINV(' + text + ')GTINV";\n'
    if not os.path.exists(dst) or open(dst).read() != body:
        with open(dst, "w") as f:
            f.write(body)
    return dst


def _sources():
    return {
        "model.o": ("g++", os.path.join(CSRC, "model.cpp")),
        "capi.o": ("g++", os.path.join(CSRC, "capi.cpp")),
        "neighbor.o": ("g++", os.path.join(CSRC, "neighbor.cpp")),
        "serve.o": ("g++", os.path.join(CSRC, "serve.cpp")),
        "kernels_common.o": ("nvcc", os.path.join(CSRC, "kernels_common.cu")),
        "peak.o": ("nvcc", os.path.join(CSRC, "peak.cu")),
        "noalloc.o": ("nvcc", os.path.join(CSRC, "noalloc.cu")),
        "md.o": ("nvcc", os.path.join(CSRC, "md.cu")),
        "batch.o": ("nvcc", os.path.join(CSRC, "batch.cu")),
        "dnlist.o": ("nvcc", os.path.join(CSRC, "dnlist.cu")),
        "features.o": ("nvcc", os.path.join(CSRC, "features.cu")),
        "pair.o": ("nvcc", os.path.join(CSRC, "pair.cu")),
        "kernels_f64.o": ("nvcc", os.path.join(CSRC, "kernels_f64.cu")),
        "kernels_f64df.o": ("nvcc", os.path.join(CSRC, "kernels_f64df.cu")),
        "kernels_f32.o": ("nvcc", os.path.join(CSRC, "kernels_f32.cu")),
    }


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(REPO, "include", "mlipg.h"))
    files.append(os.path.join(PKG, "data", "gtinv_table.txt"))
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libmlipg.so if any source is newer than it; returns its path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    _embed_table()
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(cuda, "include"), "-I" + OUT_DIR, "-I" + CSRC,
           "-I" + os.path.join(REPO, "include")]
    procs = []
    for obj, (tool, src) in _sources().items():
        out = os.path.join(OUT_DIR, obj)
        if tool == "g++":
            cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-Wall", "-c", src, "-o",
                   out] + inc
        else:
            cmd = [nvcc] + ARCH + ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler",
                                   "-fPIC,-fopenmp", "-c", src, "-o", out] + inc
            if verbose:
                cmd += ["-Xptxas", "-v"]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("build failed:\n" + "\n".join(failed))
    objs = [os.path.join(OUT_DIR, o) for o in _sources()]
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc] + ARCH + ["-shared", "-o", tmp] + objs +
                          ["-lcudart_static", "-lrt", "-lpthread", "-ldl", "-lgomp"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
