"""In-tree build of libfst.so for sm_103a (nvcc, no cmake).

Translation units and their floating-point contract:
  fst_plain3d.cu, fst_plain2d.cu, fst_bc.cu, fst_noise.cu, fst_gen.cu
                                              --fmad=false: the plain FP64 path
      reproduces the reference's FP64 arithmetic operation for operation
  fst_mixed.cu, fst_mixed3d.cu, fst_hybrid.cu, fst_batch*.cu
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
    ("fst_batch_w16.cu", ["--use_fast_math"]),
    ("fst_batch_w32.cu", ["--use_fast_math"]),
    ("fst_batch_w64.cu", ["--use_fast_math"]),
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

    with ThreadPoolExecutor(max_workers=min(max(os.cpu_count() or 1, 4), 16, len(cmds))) as ex:
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


DECK_LIB = os.path.join(HERE, "libfst_deck.so")
LUA_UNITS = ["lapi", "lcode", "lctype", "ldebug", "ldo", "ldump", "lfunc", "lgc", "llex", "lmem",
             "lobject", "lopcodes", "lparser", "lstate", "lstring", "ltable", "ltm", "lundump",
             "lvm", "lzio", "lauxlib", "lbaselib", "lbitlib", "lcorolib", "ldblib", "liolib",
             "lmathlib", "loslib", "lstrlib", "ltablib", "lutf8lib", "loadlib", "linit"]


def lua_sources():
    """The Lua 5.3 sources to build the deck reader against: FST_LUA_SRC,
    tpls/lua/src of the FIESTA tree named by FST_REFERENCE (when set), or the
    copy staged in oracle/_ref/lua.  None when none exists."""
    ref = os.environ.get("FST_REFERENCE")
    cands = [os.environ.get("FST_LUA_SRC"),
             os.path.join(ref, "tpls", "lua", "src") if ref else None,
             # the copy the reference checker's recipe (oracle/ref_build.sh) stages for
             # hosts without the tree, where the tests use it
             os.path.join(HERE, "..", "oracle", "_ref", "lua")]
    for c in cands:
        if c and os.path.exists(os.path.join(c, "lua.h")):
            return c
    return None


def build_deck(force=False, verbose=False):
    """Compile fiesta_gb300/libfst_deck.so: the Lua deck reader
    (csrc/fst_deck.cpp, include/fst_deck.h) and the Lua 5.3 library from the
    sources lua_sources() finds (compiled where they lie, as the reference's
    tpls/lua/CMakeLists.txt builds them: LUA_USE_LINUX), all without FMA
    contraction so that x86 and Arm give the same bits.  Returns the path,
    or None when no Lua sources are present (the library is then absent)."""
    src = lua_sources()
    if src is None:
        return None
    dsrc = os.path.join(CSRC, "fst_deck.cpp")
    deps = [dsrc, os.path.join(HERE, "..", "include", "fst_deck.h"),
            os.path.join(HERE, "..", "include", "fst.h")]
    if (not force and os.path.exists(DECK_LIB)
            and all(os.path.getmtime(x) <= os.path.getmtime(DECK_LIB) for x in deps)):
        return DECK_LIB
    bdir = os.path.join(BUILD, "lua")
    os.makedirs(bdir, exist_ok=True)
    cmds, objs = [], []
    for u in LUA_UNITS:
        obj = os.path.join(bdir, u + ".o")
        cmds.append(["gcc", "-O2", "-std=gnu99", "-fPIC", "-ffp-contract=off", "-DLUA_USE_LINUX",
                     "-w", "-c", os.path.join(src, u + ".c"), "-o", obj])
        objs.append(obj)
    obj = os.path.join(BUILD, "fst_deck.o")
    # no FMA contraction (gcc contracts by default on aarch64): the cell
    # centres and the deck's arithmetic round as in the Python reader
    cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", src, "-c", dsrc,
                 "-o", obj])
    objs.append(obj)

    def run(cmd):
        return cmd, subprocess.run(cmd, capture_output=True, text=True)

    with ThreadPoolExecutor(max_workers=8) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose or r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("compile failed: " + " ".join(cmd))
    tmp = DECK_LIB + ".tmp"
    r = subprocess.run(["g++", "-shared", "-o", tmp, *objs, "-ldl", "-lm"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, DECK_LIB)
    return DECK_LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas" in sys.argv)
    print(LIB)
