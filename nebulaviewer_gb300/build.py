"""In-tree build of libnebula.so for sm_103a (nvcc, one -gencode, translation units compiled
in parallel).  `python -m nebulaviewer_gb300.build` or `build()`."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnebula.so")
SOURCES = ["nb_hydro.cu", "nb_step.cu", "nb_rays.cu", "nb_fuv.cu", "nb_snap.cu", "nb_stir.cu", "nb_api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no contraction of a*b+c, so every float operation is the reference's own
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                     "-Xptxas", "-v"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{p.stdout}\n{p.stderr}")
    with open(os.path.join(BUILD, os.path.splitext(src)[0] + ".ptxas.txt"), "w") as f:
        f.write(p.stderr)
    if verbose:
        print(f"  built {src}", flush=True)
    return obj


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for n in os.listdir(d):
            if os.path.getmtime(os.path.join(d, n)) > t:
                return True
    return os.path.getmtime(__file__) > t


def build(force=False, verbose=True):
    """Compile every translation unit for sm_103a and link libnebula.so in the package dir."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"  linked {LIB}", flush=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
