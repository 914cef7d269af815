"""Build recipe for the native library (and the CPU oracle used by the tests).

    python -m rank_structured_cholesky_gb300._build          # library + oracle

Outputs stay in-tree:  rank_structured_cholesky_gb300/_build/librschol_gb300.so
and oracle/_build/liboracle.so.  CUDA code is compiled for sm_103a only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "librschol_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_OUT = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_OUT, "liboracle.so")

HOST_SRC = ["host/ordering.cpp", "host/symbolic.cpp", "host/problems.cpp", "host/capi_host.cpp", "host/server.cpp"]
CUDA_SRC = ["cuda/dense.cu", "cuda/gemm_tc.cu", "cuda/factor.cu", "cuda/solve.cu", "cuda/solve_batch.cu", "cuda/pcg.cu", "cuda/pcg_batch.cu", "cuda/capi.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _headers():
    hs = []
    for d, _, files in os.walk(CSRC):
        hs += [os.path.join(d, f) for f in files if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "rschol_gpu.h"))
    return hs


def build_library(verbose=False, jobs=None):
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    nvcc = _nvcc()
    heads = _headers()
    cmds, objs = [], []
    for src in HOST_SRC + CUDA_SRC:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT, "obj", src.replace("/", "_") + ".o")
        objs.append(obj)
        if not _stale(obj, [path] + heads):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c", path, "-o", obj]
        else:
            cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-I" + cuda_inc, "-c", path, "-o", obj]
        cmds.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out:
                print(out)
    if _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_oracle():
    os.makedirs(ORACLE_OUT, exist_ok=True)
    srcs = [os.path.join(ORACLE_DIR, "oracle.cpp")] + [os.path.join(CSRC, s) for s in HOST_SRC[:3]]
    deps = srcs + [os.path.join(ORACLE_DIR, "dense.h")] + _headers()
    if _stale(ORACLE_LIB, deps):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-o", ORACLE_LIB] + srcs)
    return ORACLE_LIB


def reference_dir():
    """Root of the reference's sources (RSCHOL_REFERENCE_DIR, by default the
    read-only checkout this recipe was written against), or None where they
    are absent."""
    root = os.environ.get("RSCHOL_REFERENCE_DIR", "/root/reference")
    return root if os.path.isdir(os.path.join(root, "src", "rschol")) else None


REF_SHIM = os.path.join(ORACLE_DIR, "ref_shim")
REF_OUT = os.path.join(ORACLE_DIR, "_ref")
REF_PCG_LIB = os.path.join(REF_OUT, "libref_pcg.so")
REF_SEPTREE = os.path.join(REF_OUT, "ref_septree_kat")
REF_MT = os.path.join(REF_OUT, "mt_ref_kat")


def build_reference_tools():
    """Compile checking tools from the reference's own sources where they lie
    (only where they are present), into oracle/_ref/:

    * mt_ref_kat        -- draws of src/rschol/util/MERSENNETWISTER.h;
    * ref_septree_kat   -- src/rschol/datastructure/SeparatorTree.h/.cpp, as
                           NestedDissection::ReorderNestedSeparators builds it;
    * libref_pcg.so     -- PCG_SOLVER::solvePCG with VECTOR_FAST.cpp and
                           SPARSE_MATRIX.cpp, preconditioner by callback.

    oracle/ref_shim/ stands in for Boost's names, the CMake-written config.h
    and CBLAS level 1; none of the reference's code is changed or copied.
    Returns the MT tool's path, or None without the reference sources."""
    root = reference_dir()
    if root is None:
        return None
    src = os.path.join(root, "src")
    os.makedirs(os.path.join(REF_OUT, "obj"), exist_ok=True)
    mt_src = os.path.join(ORACLE_DIR, "ref_mt_kat.cpp")
    if _stale(REF_MT, [mt_src]):
        _run(["g++", "-O2", "-std=c++11", "-I", os.path.join(src, "rschol", "util"), mt_src, "-o", REF_MT])
    shim_files = [os.path.join(d, f) for d, _, fs in os.walk(REF_SHIM) for f in fs]
    inc = ["-I", REF_SHIM, "-I", src]
    st_src = os.path.join(ORACLE_DIR, "ref_septree_kat.cpp")
    st_deps = [st_src] + shim_files + [os.path.join(src, "rschol", "datastructure", f)
                                       for f in ("SeparatorTree.h", "SeparatorTree.cpp")]
    if _stale(REF_SEPTREE, st_deps):
        _run(["g++", "-O2", "-std=c++11", "-w"] + inc + [st_src, "-o", REF_SEPTREE])
    la = os.path.join(src, "rschol", "linearalgebra")
    ref_srcs = [os.path.join(la, f) for f in ("PCG_SOLVER.cpp", "VECTOR_FAST.cpp", "SPARSE_MATRIX.cpp")]
    tool = os.path.join(ORACLE_DIR, "ref_pcg_tool.cpp")
    blas = os.path.join(REF_SHIM, "cblas_level1.c")
    if _stale(REF_PCG_LIB, ref_srcs + [tool, blas] + shim_files):
        hidden = ["-fPIC", "-fvisibility=hidden", "-ffunction-sections", "-fdata-sections"]
        objs, cmds = [], []
        for s_ in ref_srcs + [tool]:
            o = os.path.join(REF_OUT, "obj", os.path.basename(s_) + ".o")
            objs.append(o)
            cmds.append(["g++", "-O2", "-std=c++11", "-w"] + hidden + inc + ["-I", la, "-c", s_, "-o", o])
        o = os.path.join(REF_OUT, "obj", "cblas_level1.o")
        objs.append(o)
        cmds.append(["gcc", "-O2"] + hidden + ["-c", blas, "-o", o])
        with cf.ThreadPoolExecutor(max_workers=4) as ex:
            list(ex.map(_run, cmds))
        _run(["g++", "-shared", "-Wl,--gc-sections", "-Wl,--no-undefined", "-o", REF_PCG_LIB] + objs + ["-lz"])
    return REF_MT


def build_all(verbose=False):
    lib = build_library(verbose=verbose)
    orc = build_oracle()
    ref = build_reference_tools()
    return lib, orc, ref


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
