"""Build recipe for the GB300 extension library (libcpanel_gb300.so, in-tree).

CUDA sources are compiled for sm_103a only.  The influence and post-processing
kernels are compiled with --fmad=false so that their FP64 branch decisions round
exactly like the host code; the solver kernels keep fused multiply-adds.  Host
sources use -ffp-contract=off for the same reason.  Translation units compile in
parallel; nothing is rebuilt when the library is newer than every source.
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libcpanel_gb300.so")
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_STRICT = ["assemble.cu", "post.cu", "vpkern.cu"]   # FP64 panel math: no contraction
CU_FAST = ["solve.cu", "lu.cu", "skinny.cu", "particles.cu", "tc_gemm.cu"]  # particles.cu rounds its branch tests explicitly
CPP = ["mesh.cpp", "api.cpp", "octree.cpp", "vpgeom.cpp", "vpcase.cpp", "server.cpp", "batch.cpp", "writers.cpp",
       "streamline.cpp", "shim.cpp", "chtls_host.cpp"]
HEADERS = ["common.cuh", "panel64.cuh", "df.cuh", "assemble.h", "post.h", "mesh.h", "octree.h", "particles.h", "vp.cuh",
           "vpgeom.h", "vpkern.h", "streamline.h", "tc_gemm.h", "skinny.h"]


def _sources():
    return [os.path.join(SRC, f) for f in CU_STRICT + CU_FAST + CPP + HEADERS] + [
        os.path.join(ROOT, "include", "cpanel_gpu.h"), os.path.join(ROOT, "include", "cpanel_vp.h"),
        os.path.join(ROOT, "include", "cpanel_serve.h"), os.path.join(ROOT, "include", "cpanel_batch.h"),
        os.path.join(ROOT, "include", "cpanel_io.h"), os.path.join(ROOT, "include", "cpanel_shim.hpp"),
        os.path.abspath(__file__)]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.exists(s) and os.path.getmtime(s) > t for s in _sources())


def _cmd_cu(name, strict):
    obj = os.path.join(OUT, name + ".o")
    cmd = [NVCC, "-c", os.path.join(SRC, name), "-o", obj, "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC", "-Xptxas", "-v" if os.environ.get("CPG_PTXAS_VERBOSE") else "-O3"] + ARCH
    if strict:
        cmd.append("--fmad=false")
    return cmd, obj


def _cmd_cpp(name):
    obj = os.path.join(OUT, name + ".o")
    cmd = ["g++", "-c", os.path.join(SRC, name), "-o", obj, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
           "-I" + os.path.join(CUDA, "include"), "-DCPG_COMPILED_ARCH=103"]
    return cmd, obj


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    if not os.path.exists(NVCC):
        raise RuntimeError("nvcc not found at %s" % NVCC)
    os.makedirs(OUT, exist_ok=True)
    jobs = [_cmd_cu(f, True) for f in CU_STRICT] + [_cmd_cu(f, False) for f in CU_FAST] + [_cmd_cpp(f) for f in CPP]

    def run(job):
        cmd, obj = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [NVCC, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-Xcompiler", "-pthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
