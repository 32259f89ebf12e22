"""Builds the native libraries in-tree.

  alsvinn_gb300/lib/libgbfv.so   the CUDA path (sm_103a) behind include/gbfv.h
  oracle/libfvoracle.so          the CPU oracle (test infrastructure)
  oracle/_ref/libalsref.so       the reference's own CPU path, only where the
                                 reference sources are present (REF_ROOT)
  oracle/_ref/cuda/*.cubin       the reference's own CUDA kernels (device code
                                 only), where the reference sources are present
  oracle/librefcuda.so           the host driver of those kernels (test and
                                 baseline infrastructure)

Translation units compile in parallel; a unit is rebuilt only when a source or
header it may include changed (timestamps over csrc/ and include/).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libgbfv.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "libfvoracle.so")
REFCUDA_LIB = os.path.join(ORACLE_DIR, "librefcuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + CSRC, "-I" + INCLUDE]

VARIANTS = (0, 1, 2, 3)   # fp64, fp64 exact, fp32, fp64 state with double-float arithmetic
EQUATIONS = (0, 1, 2, 3)  # burgers, euler1, euler2, euler3
TUNED_VARIANTS = (0, 1, 2, 3)  # variants with autotuning candidates (all; TMA where storage = arithmetic type)
REGION_VARIANTS = (0, 1, 2, 3)  # variants with region kernels (operator calls on part of the grid)


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build alsvinn_gb300")


def _units():
    units = []
    for v in VARIANTS:
        for e in EQUATIONS:
            flags = ["-DFV_VARIANT=%d" % v, "-DFV_EQ=%d" % e]
            if v == 1:
                flags += ["-DFV_EXACT"]
            if v in TUNED_VARIANTS:
                # no automatic multiply-add contraction: the source fixes every
                # rounding, so all tile configurations of a scheme give the same bits
                flags += ["-fmad=false"]
            units.append(("fv_variant.cu", "fv_v%d_e%d.o" % (v, e), flags + ["-DFV_PART=0"]))
            if v in TUNED_VARIANTS:
                units.append(("fv_variant.cu", "fv_v%d_e%d_tune.o" % (v, e), flags + ["-DFV_PART=1"]))
            if v in REGION_VARIANTS:
                units.append(("fv_variant.cu", "fv_v%d_e%d_region.o" % (v, e), flags + ["-DFV_PART=2"]))
    units.append(("gbfv_tune.cu", "gbfv_tune.o", []))
    units.append(("gbfv_api.cu", "gbfv_api.o", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]))
    units.append(("gbfv_stats.cu", "gbfv_stats.o", []))
    units.append(("gbfv_structure.cu", "gbfv_structure.o", []))
    units.append(("gbfv_functional.cu", "gbfv_functional.o", ["-fmad=false"]))
    units.append(("gbfv_noalloc.cu", "gbfv_noalloc.o", []))
    units.append(("gbfv_memory.cu", "gbfv_memory.o", ["-fmad=false"]))
    units.append(("gbfv_batch.cu", "gbfv_batch.o", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]))
    units.append(("gbfv_init.cpp", "gbfv_init.o", ["-Xcompiler", "-ffp-contract=off"]))
    units.append(("gbfv_serve.cpp", "gbfv_serve.o", []))
    return units


def _newest_dep():
    t = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build_cuda(verbose=False, jobs=None):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    dep = _newest_dep()
    todo = []
    objs = []
    for src, obj, flags in _units():
        out = os.path.join(BUILD, obj)
        objs.append(out)
        if not os.path.exists(out) or os.path.getmtime(out) < dep:
            todo.append([nvcc] + ARCH + NVCC_COMMON + flags + ["-c", os.path.join(CSRC, src), "-o", out])
    if todo:
        jobs = jobs or min(len(todo), os.cpu_count() or 4)
        with concurrent.futures.ThreadPoolExecutor(jobs) as ex:
            for out in ex.map(_run, todo):
                if verbose and out.strip():
                    print(out)
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs)
    return LIB


def build_oracle():
    src = os.path.join(ORACLE_DIR, "fvoracle.c")
    if os.path.exists(ORACLE_LIB) and os.path.getmtime(ORACLE_LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(ORACLE_DIR, "fvoracle.h"))):
        return ORACLE_LIB
    cc = os.environ.get("CC", "gcc")
    _run([cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wno-unknown-pragmas",
          "-o", ORACLE_LIB, src, "-lm"])
    return ORACLE_LIB


def build_reference_oracle(ref_root=None):
    """Compiles the reference's CPU path from its sources, where they exist:
    REF_ROOT in the environment, else the location the recipe
    (oracle/refbuild/Makefile) names."""
    refbuild = os.path.join(ORACLE_DIR, "refbuild")
    ref_root = ref_root or os.environ.get("REF_ROOT")
    if not ref_root:
        try:
            ref_root = _run(["make", "-s", "--no-print-directory", "-C", refbuild, "print-ref"]).strip()
        except (OSError, RuntimeError):
            return None
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "alsfvm", "src")):
        return None
    _run(["make", "-s", "-C", refbuild, "-j%d" % (os.cpu_count() or 4), "REF=" + ref_root, "all", "cuda",
          "NVCC=" + _nvcc()])
    return os.path.join(ORACLE_DIR, "_ref", "libalsref.so")


def build_refcuda():
    """The host driver of the reference's CUDA kernels (oracle/refcuda/)."""
    src = os.path.join(ORACLE_DIR, "refcuda", "refcuda.cu")
    hdr = os.path.join(ORACLE_DIR, "refcuda", "refcuda.h")
    if os.path.exists(REFCUDA_LIB) and os.path.getmtime(REFCUDA_LIB) >= max(os.path.getmtime(src),
                                                                            os.path.getmtime(hdr)):
        return REFCUDA_LIB
    _run([_nvcc()] + ARCH + ["-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-I" + os.path.dirname(src),
                             src, "-o", REFCUDA_LIB])
    return REFCUDA_LIB


def build_all(verbose=False):
    lib = build_cuda(verbose=verbose)
    orc = build_oracle()
    ref = build_reference_oracle()
    rcu = build_refcuda()
    return lib, orc, ref, rcu


if __name__ == "__main__":
    for p in build_all(verbose="-v" in sys.argv):
        print(p)
