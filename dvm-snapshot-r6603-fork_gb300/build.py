"""Build the GB300 loop-execution runtime and the workload programs, in tree.

  lib/libdvmh_gb.so          runtime (dvmh_* ABI, csrc/*.cpp, csrc/*.cu) and the
                             hand-written sm_103a loop kernels (csrc/kernels/*.cu)
  lib/libdvmhgb_workloads.so the workload programs (workloads/*.c main code +
                             workloads/*_cuda.cu CUDA handlers) linked against it

Device code: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo
-fmad=false (no FMA contraction: each cell's arithmetic is the source
program's).  Host code of the programs: gcc -O2 -ffp-contract=off -fopenmp.
Translation units compile in parallel; nothing is rebuilt when up to date.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INC = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(PKG, "_build")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                  "-I" + INC, "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + INC, "-I" + os.path.join(CUDA, "include")]
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-Wall", "-Wno-unused-variable",
          "-I" + INC]

RUNTIME = "libdvmh_gb.so"
WORKLOADS = "libdvmhgb_workloads.so"


def _newer(src_list, out):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in src_list)


def _headers():
    return glob.glob(os.path.join(INC, "*.h")) + glob.glob(os.path.join(PKG, "csrc", "*.h")) + \
        glob.glob(os.path.join(PKG, "csrc", "*.inc")) + glob.glob(os.path.join(PKG, "csrc", "kernels", "*.cuh")) + \
        glob.glob(os.path.join(PKG, "workloads", "*.h"))


def _compile(src, extra=()):
    rel = os.path.relpath(src, PKG).replace(os.sep, "_")
    out = os.path.join(OBJ, rel + ".o")
    if not _newer([src] + _headers(), out):
        return out
    if src.endswith(".cu"):
        cmd = [NVCC] + NVFLAGS + list(extra) + ["-c", src, "-o", out]
    elif src.endswith(".cpp"):
        cmd = ["g++"] + CXXFLAGS + list(extra) + ["-c", src, "-o", out]
    else:
        cmd = ["gcc"] + CFLAGS + list(extra) + ["-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if r.stderr.strip() and os.environ.get("DVMHGB_BUILD_VERBOSE"):
        sys.stderr.write(r.stderr)
    return out


def build(verbose=False):
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    rt_src = sorted(glob.glob(os.path.join(PKG, "csrc", "*.cpp")) + glob.glob(os.path.join(PKG, "csrc", "*.cu")) +
                    glob.glob(os.path.join(PKG, "csrc", "kernels", "*.cu")))
    wl_src = sorted(glob.glob(os.path.join(PKG, "workloads", "*.c")) +
                    glob.glob(os.path.join(PKG, "workloads", "*.cpp")) +
                    glob.glob(os.path.join(PKG, "workloads", "*.cu")))
    jobs = max(2, min(16, os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        rt_obj = list(ex.map(_compile, rt_src))
        wl_obj = list(ex.map(lambda s: _compile(s, ["-I" + os.path.join(PKG, "workloads")]), wl_src))
    rt = os.path.join(LIB, RUNTIME)
    if _newer(rt_obj, rt):
        subprocess.check_call([NVCC] + ARCH + ["-shared", "-o", rt + ".tmp"] + rt_obj + ["-lcudart"])
        os.replace(rt + ".tmp", rt)
    wl = os.path.join(LIB, WORKLOADS)
    if _newer(wl_obj + [rt], wl):
        subprocess.check_call([NVCC] + ARCH + ["-shared", "-o", wl + ".tmp"] + wl_obj +
                              ["-L" + LIB, "-ldvmh_gb", "-lcudart", "-lgomp", "-Xlinker", "-rpath=$ORIGIN"])
        os.replace(wl + ".tmp", wl)
    if verbose:
        print(rt)
        print(wl)
    return rt, wl


if __name__ == "__main__":
    build(verbose=True)
