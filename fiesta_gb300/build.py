"""In-tree build of libfst.so for sm_103a (nvcc, no cmake).

Translation units and their floating-point contract:
  fst_plain3d.cu, fst_plain2d.cu, fst_bc.cu, fst_noise.cu, fst_gen.cu
                                              --fmad=false: the plain FP64 path
      reproduces the reference's FP64 arithmetic operation for operation
  fst_mixed.cu, fst_mixed3d.cu, fst_hybrid.cu, fst_batch.cu
                                              FMA on, fast FP32 math
  fst_mixedgen.cu                             IEEE FP32 (pair arithmetic)
  fst_api.cu                                  host orchestration
  fst_host.cpp                                host IC generator, g++ with
      -ffp-contract=off so the same seed gives the same bits on x86 and Arm
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfst.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not os.path.exists(NVCC):
    NVCC = "nvcc"

UNITS = [
    ("fst_plain3d.cu", ["--fmad=false"]),
    ("fst_plain2d.cu", ["--fmad=false"]),
    ("fst_bc.cu", ["--fmad=false"]),
    ("fst_mixed.cu", ["--use_fast_math"]),
    ("fst_mixed3d.cu", ["--use_fast_math"]),
    ("fst_hybrid.cu", ["--use_fast_math"]),
    ("fst_batch.cu", ["--use_fast_math"]),
    ("fst_api.cu", ["--fmad=false"]),
    ("fst_noalloc.cu", ["--fmad=false"]),
    ("fst_noise.cu", ["--fmad=false"]),
    ("fst_gen.cu", ["--fmad=false"]),
    ("fst_mixedgen.cu", []),
]
HOST_UNITS = ["fst_host.cpp"]


def _sources():
    out = [os.path.join(CSRC, f) for f, _ in UNITS] + [os.path.join(CSRC, f) for f in HOST_UNITS]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    out.append(os.path.join(HERE, "..", "include", "fst.h"))
    return out


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, ptxas_v=False):
    """Compile every unit (in parallel) and link fiesta_gb300/libfst.so."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", CSRC, "-I", os.path.join(HERE, "..", "include")]
    cmds = []
    objs = []
    for f, extra in UNITS:
        obj = os.path.join(BUILD, f + ".o")
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--extended-lambda",
               "-Xcompiler", "-fPIC,-ffp-contract=off", *extra, *inc, "-c",
               os.path.join(CSRC, f), "-o", obj]
        if ptxas_v:
            cmd.insert(1, "-Xptxas=-v")
        cmds.append(cmd)
        objs.append(obj)
    for f in HOST_UNITS:
        obj = os.path.join(BUILD, f + ".o")
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", *inc, "-c",
                     os.path.join(CSRC, f), "-o", obj])
        objs.append(obj)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=min(8, len(cmds))) as ex:
        results = list(ex.map(run, cmds))
    for cmd, r in results:
        if verbose or r.returncode != 0 or ptxas_v:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd))
    tmp = LIB + ".tmp"
    link = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas" in sys.argv)
    print(LIB)
