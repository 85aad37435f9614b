"""Builds libmarbles_gpu.so in-tree with nvcc for sm_103a (no torch needed).

Translation units compile in parallel; the FP64 form is compiled with
-fmad=false so that its multiplies and adds round separately, as in the
reference's CPU build.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmarbles_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction either (aarch64 g++ contracts by default)
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp",
          "--expt-relaxed-constexpr"] + ARCH
UNITS = {
    "mbg_fp64.cu": ["-fmad=false"],
    "mbg_fp64_bc.cu": ["-fmad=false"],
    "mbg_fp64_bcc.cu": ["-fmad=false"],
    "mbg_fp64_gen.cu": ["-fmad=false"],
    "mbg_fp64_shell.cu": ["-fmad=false"],
    "mbg_fp64_amr.cu": ["-fmad=false"],
    "mbg_fp64_out.cu": ["-fmad=false"],
    "mbg_lowp.cu": [],
    "mbg_lowp_f16.cu": [],
    "mbg_lowp_bf16.cu": [],
    "mbg_batch.cu": [],
    "mbg_adjoint.cu": [],
    "mbg_capi.cu": [],
    "lbm_driver.cu": [],
    "lbm_capi.cu": [],
    "lbm_io.cu": [],
    "mbg_geometry.cu": ["-fmad=false"],
    "mbg_noalloc.cu": ["-fmad=false"],
}
EXE = os.path.join(HERE, "marbles_gb300_run")


def nvcc():
    for c in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if os.path.exists(c) or c == "nvcc":
            return c


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "marbles_gb300.h"))
    return max(os.path.getmtime(h) for h in hs if os.path.exists(h))


def _compile(unit, extra):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    # an object newer than its source and every header is kept
    if os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(src), _headers_mtime()):
        return obj
    cmd = [nvcc()] + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr))
    return obj


def _stale(objs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    srcs.append(os.path.join(HERE, "..", "include", "marbles_gb300.h"))
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def build(force=False, verbose=True):
    os.makedirs(BUILD, exist_ok=True)
    units = {u: e for u, e in UNITS.items() if os.path.exists(os.path.join(CSRC, u))}
    if not force and not _stale(units):
        return LIB
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), units.items()))
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-Xcompiler", "-fopenmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    main = os.path.join(CSRC, "marbles_main.cpp")
    cmd = [nvcc(), "-O2", "-std=c++17", main, "-o", EXE, "-L" + HERE, "-lmarbles_gpu",
           "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("executable link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
