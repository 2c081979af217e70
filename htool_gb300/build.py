"""Build libhtgpu.so in-tree (htool_gb300/libhtgpu.so).

CUDA sources are compiled for sm_103a only; host C++ sources with g++ and
-ffp-contract=off (the cluster and block trees must reproduce htool's
floating-point results bit for bit on every host architecture).  Objects go
to htool_gb300/_build; translation units are compiled in parallel.
"""
import concurrent.futures
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "libhtgpu.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# per-file extra nvcc flags
EXTRA = {
    # generator entries and ACA residuals must round exactly like htool's CPU
    # code: no implicit multiply-add contraction in this file
    "build_kernels.cu": ["-fmad=false"],
}


def _sources():
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    return [os.path.join(CSRC, f) for f in srcs]


def _compile(src, verbose):
    name = os.path.basename(src)
    obj = os.path.join(BUILD, name + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh"))] + [os.path.join(os.path.dirname(HERE), "include", "htgpu.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-c", src, "-o", obj] + EXTRA.get(name, [])
        if verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function", "-I" + os.path.join(CUDA, "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    stamp = os.path.join(BUILD, "lib.stamp")
    if os.path.exists(LIB) and os.path.exists(stamp) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = ["g++", "-shared", "-o", LIB] + objs + ["-L" + os.path.join(CUDA, "lib64"), "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stderr))
    open(stamp, "w").write(platform.machine())
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
