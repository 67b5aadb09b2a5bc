"""Builds the CUDA library libpansfem2_gb300.so in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into one shared library with a plain C ABI (include/pansfem2_gpu.h).
psf_element.cu is compiled with --fmad=false so that the element matrices
keep the reference's rounding step by step.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpansfem2_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not os.path.exists(NVCC):
    NVCC = "nvcc"

SOURCES = ["psf_element.cu", "psf_mesh.cu", "psf_solve.cu", "psf_opt.cu", "psf_optdw.cu", "psf_mg.cu", "psf_capi.cu", "psf_generic.cu", "psf_fem.cu", "psf_noalloc.cu", "psf_unet.cu", "psf_learned.cu", "psf_vtk.cu", "psf_batch.cu", "psf_mmagen.cu", "psf_krylov.cu"]
PER_FILE = {"psf_element.cu": ["--fmad=false"], "psf_fem.cu": ["--fmad=false"], "psf_krylov.cu": ["--fmad=false"]}


def _compile(src, verbose):
    obj = os.path.join(OUT, src.replace(".cu", ".o"))
    cmd = [NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--extended-lambda", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, *PER_FILE.get(src, []),
           "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, p.returncode, p.stdout + p.stderr


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    hdrs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    hdrs.append(os.path.join(ROOT, "include", "pansfem2_gpu.h"))
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) < t for f in srcs + hdrs + [__file__]):
            return LIB
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    failed = [r for r in results if r[2] != 0]
    for src, obj, rc, log in results:
        if log.strip() and (verbose or rc != 0):
            sys.stderr.write(f"--- {src}\n{log}\n")
    if failed:
        raise RuntimeError("nvcc failed: " + ", ".join(r[0] for r in failed))
    objs = [r[1] for r in results]
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
