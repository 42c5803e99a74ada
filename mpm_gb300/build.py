"""In-tree build of ``libmpm_gb300.so`` for sm_103a (nvcc, no cmake).

The translation units compile in parallel; the library is written next to this
file so the loader finds it without installation.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmpm_gb300.so")
SOURCES = ["substep.cu", "aux_kernels.cu", "capi.cu", "noalloc.cu", "batch.cu", "adjoint.cu", "seeding.cu", "surface.cu",
           "smooth.cu", "export.cu", "tuning_cache.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include")]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return max(os.path.getmtime(f) for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(BUILD, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [NVCC, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            print(log)
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_with_materials(sources, out: str, force: bool = False) -> str:
    """A build of the library at `out` with material models compiled in: `sources` are .cu
    files that include mpm_gb300_policies.cuh and register their policies with
    MPM_GB300_REGISTER_MATERIAL (the reference's way of choosing a MaterialModel is to edit
    its compile-time alias and rebuild, include/mpm.cuh:25).  The library's own objects
    come from build(); only the given files are compiled here."""
    build()
    sources = [os.path.abspath(s) for s in sources]
    objs = [os.path.join(BUILD, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    newest = max([os.path.getmtime(s) for s in sources] + [os.path.getmtime(o) for o in objs] + [_deps()])
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    outdir = os.path.dirname(os.path.abspath(out))
    os.makedirs(outdir, exist_ok=True)
    plugin_objs = []
    for src in sources:
        obj = os.path.join(outdir, os.path.splitext(os.path.basename(src))[0] + ".plugin.o")
        cmd = [NVCC, *ARCH, *FLAGS, "-I", CSRC, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        plugin_objs.append(obj)
    tmp = out + ".tmp"
    r = subprocess.run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, *plugin_objs, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    import sys

    print(build(force=True, verbose="-v" in sys.argv))
