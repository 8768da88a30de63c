"""In-tree build of the two libraries for sm_103a (nvcc, one -gencode, translation units
compiled in parallel).  `python -m nebulaviewer_gb300.build` or `build()`.

Both export the same C ABI (include/nebula.h) and differ only in floating-point code
generation:
  libnebula.so       exact: no contraction of a*b+c, IEEE division and square root, no
                     flush-to-zero -- every float operation is the reference's, so results are
                     bit-identical to the reference's kernel source evaluated in
                     IEEE float32 without contraction;
  libnebula_fast.so  fast: a*b+c contracted to FMA, approximate division and square root,
                     denormals flushed to zero in the compute kernels (the snapshot / frame
                     formats and the renderer's voxel pack keep the exact flags, their bytes
                     are part of a format); stays
                     within the path's stated tolerance of the exact build.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBS = {"exact": os.path.join(HERE, "libnebula.so"), "fast": os.path.join(HERE, "libnebula_fast.so")}
LIB = LIBS["exact"]
SOURCES = ["nb_hydro.cu", "nb_step.cu", "nb_rays.cu", "nb_fuv.cu", "nb_snap.cu", "nb_stir.cu", "nb_render.cu",
           "nb_api.cu"]
EXACT_ONLY = {"nb_snap.cu", "nb_render.cu"}   # byte formats: same code generation in both libraries
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-Xptxas", "-v"]
ARITH_FLAGS = {
    "exact": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"],
    "fast": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true", "-DNB_ARITH_FAST=1"],
}
NVCC_FLAGS = COMMON + ARITH_FLAGS["exact"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(job, verbose):
    arith, src = job
    flavour = "exact" if src in EXACT_ONLY else arith
    out = os.path.join(BUILD, arith)
    obj = os.path.join(out, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + COMMON + ARITH_FLAGS[flavour] + ["-c", os.path.join(CSRC, src), "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src} ({arith}):\n{p.stdout}\n{p.stderr}")
    with open(os.path.join(out, os.path.splitext(src)[0] + ".ptxas.txt"), "w") as f:
        f.write(p.stderr)
    if verbose:
        print(f"  built {src} ({arith})", flush=True)
    return obj


def _stale():
    if not all(os.path.exists(p) for p in LIBS.values()):
        return True
    t = min(os.path.getmtime(p) for p in LIBS.values())
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for n in os.listdir(d):
            if os.path.getmtime(os.path.join(d, n)) > t:
                return True
    return os.path.getmtime(__file__) > t


def build(force=False, verbose=True):
    """Compile every translation unit for sm_103a, twice (exact and fast code generation), and
    link libnebula.so and libnebula_fast.so in the package dir."""
    if not force and not _stale():
        return LIB
    for arith in LIBS:
        os.makedirs(os.path.join(BUILD, arith), exist_ok=True)
    jobs = [(a, s) for a in LIBS for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda j: _compile(j, verbose), jobs))
    for arith, path in LIBS.items():
        mine = [o for (a, _), o in zip(jobs, objs) if a == arith]
        tmp = path + ".tmp"
        p = subprocess.run([nvcc()] + ARCH + ["-shared", "-o", tmp] + mine, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
        os.replace(tmp, path)
        if verbose:
            print(f"  linked {path}", flush=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
