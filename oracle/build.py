"""Build recipe of the CPU oracle (test infrastructure): oracle/_build/liboracle.so from
oracle/ref_cpu.cpp with g++ (-O2, OpenMP, -ffp-contract=off so no a*b+c is fused)."""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ref_cpu.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False, verbose=True):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           SRC, "-o", tmp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"  built {LIB}", flush=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
