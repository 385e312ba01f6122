"""Build recipe of libafivo_gpu.so (sm_103a only, in-tree).

nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3 --fmad=false:
--fmad=false keeps FP64 kernels free of contractions so that they reproduce
the reference operation order bit for bit; FP32 kernels that want fused
multiply-adds request them explicitly.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libafivo_gpu.so")
OBJ_DIR = os.path.join(HERE, "build")
UNITS = ["afg_runtime.cu", "afg_species_update.cu", "afg_noalloc.cu", "afg_tree_host.cpp", "afg_output_host.cpp"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3",
              "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xcompiler", "-fopenmp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    out = [os.path.join(HERE, "..", "include", "afivo_gpu.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB
    nvcc = _nvcc()
    objs = []

    def compile_unit(u):
        src = os.path.join(CSRC, u)
        obj = os.path.join(OBJ_DIR, os.path.splitext(u)[0] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(UNITS))) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB] + objs + ["-lcudart", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
