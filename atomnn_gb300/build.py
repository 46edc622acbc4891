"""Builds the engine's shared library atomnn_gb300/_build/libnnpgpu.so for sm_103a (GB300).

CUDA sources go through nvcc with one -gencode (compute_103a -> sm_103a); host C++ sources
through g++.  Translation units compile in parallel and are skipped when up to date.  Host code
uses -ffp-contract=off so that the neighbour set-up reproduces the oracle's FP64 rounding on
both x86 and Arm hosts.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnnpgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _cuda_include():
    return os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")


def _deps():
    hdrs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hdrs.append(os.path.join(os.path.dirname(HERE), "include", "nnpgpu.h"))
    return max(os.path.getmtime(h) for h in hdrs)


def _compile(src, verbose=False, ptxas_info=False):
    obj = os.path.join(OUT, "obj", os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps()):
        return obj, ""
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "--expt-relaxed-constexpr", "-c", src, "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + _cuda_include(), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr if ptxas_info else ""


def build(verbose=False, ptxas_info=False, jobs=None):
    """Compile every translation unit and link libnnpgpu.so; returns the library path."""
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    # heaviest translation units first
    srcs.sort(key=lambda s: -os.path.getsize(s))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, ptxas_info), srcs))
    objs = [o for o, _ in results]
    if ptxas_info:
        for _, log in results:
            if log:
                sys.stdout.write(log)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(LIB + ".tmp", LIB)
    build_host()
    return LIB


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_host():
    """The C++ host surface (libatomnn_gpu.so, include/atomnn_gpu.hpp) over libnnpgpu.so, and the
    compute tool nnp_compute_gpu; both find libnnpgpu.so next to themselves."""
    host = os.path.join(HERE, "host")
    inc = os.path.join(os.path.dirname(HERE), "include")
    deps = [LIB, os.path.join(inc, "atomnn_gpu.hpp"), os.path.join(inc, "nnpgpu.h")]
    shim_src = os.path.join(host, "atomnn_gpu.cpp")
    shim = os.path.join(OUT, "libatomnn_gpu.so")
    newest = max(os.path.getmtime(d) for d in deps + [shim_src])
    if not os.path.exists(shim) or os.path.getmtime(shim) < newest:
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-shared", "-I" + inc, shim_src, "-o", shim + ".tmp", "-L" + OUT,
              "-lnnpgpu", "-Wl,-rpath,$ORIGIN"])
        os.replace(shim + ".tmp", shim)
    tool_src = os.path.join(host, "nnp_compute_gpu.cpp")
    tool = os.path.join(OUT, "nnp_compute_gpu")
    if not os.path.exists(tool) or os.path.getmtime(tool) < max(newest, os.path.getmtime(shim), os.path.getmtime(tool_src)):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + inc, tool_src, "-o", tool + ".tmp", "-L" + OUT, "-latomnn_gpu", "-lnnpgpu",
              "-Wl,-rpath,$ORIGIN"])
        os.replace(tool + ".tmp", tool)
    return shim, tool


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
