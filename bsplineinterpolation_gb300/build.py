"""Builds the CUDA library in-tree: bsplineinterpolation_gb300/libintp_gb300.so.

nvcc compiles every .cu for sm_103a only; host C++ that must round exactly
like the reference (knot vectors, factors) is compiled with g++ without
floating-point contraction. Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
# objects per host architecture (a tree copied between machines never links
# another machine's objects)
BUILD = os.path.join(HERE, "_build", platform.machine() or "host")
LIB = os.path.join(HERE, "libintp_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "--expt-relaxed-constexpr", "-I" + os.path.join(REPO, "include"), "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             "-I" + os.path.join(REPO, "include"), "-I" + CSRC]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    deps.append(os.path.join(REPO, "include", "intp_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = sources()
    cmds = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, src):
            cmds.append(([nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"], obj))
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, src):
            cmds.append(([os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", src, "-o", obj + ".tmp"], obj))

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    def compile_one(job):
        # written under a temporary name: an interrupted compile never leaves
        # a truncated object that looks up to date
        cmd, obj = job
        err = run(cmd)
        os.replace(obj + ".tmp", obj)
        return err

    # drop objects of sources that no longer exist, and leftovers
    for f in os.listdir(BUILD):
        if (f.endswith(".o") and f[:-2] not in cu + cpp) or f.endswith(".o.tmp"):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for err in ex.map(compile_one, cmds):
            if verbose and err:
                print(err)
    if cmds or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
