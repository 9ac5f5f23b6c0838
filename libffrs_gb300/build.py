"""In-tree build of the native parts of libffrs_gb300.

* libffgpu.so   -- CUDA kernels + C ABI (include/ffgpu.h), nvcc for sm_103a
* libffrs.*.so  -- the pybind11 module named ``libffrs`` (host side, C++),
                   linked against libffgpu.so

Both land in libffrs_gb300/ next to this file.  Translation units compile in
parallel and are skipped when up to date.  No cmake.
"""

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "_build", platform.machine())
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_GPU = os.path.join(HERE, "libffgpu.so")


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(_nvcc()))


def _pybind_include():
    try:
        import pybind11  # noqa: F401

        return pybind11.get_include()
    except ImportError:
        pass
    import torch  # torch ships the pybind11 headers

    return os.path.join(os.path.dirname(torch.__file__), "include")


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + [
        os.path.join(ROOT, "include", "ffgpu.h")
    ]


def build_gpu_lib(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    flags = ARCH_FLAGS + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "--expt-relaxed-constexpr",
        "-Xcudafe",
        "--max_cost_constexpr_call=400000000",
        "-Xcompiler",
        "-fPIC",
        "-Xcompiler",
        "-fvisibility=hidden",
        "-I" + os.path.join(ROOT, "include"),
    ]
    if os.environ.get("FFGPU_PTXAS_VERBOSE"):
        flags += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append([nvcc] + flags + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for out in outs:
                if out.strip():
                    print(out)
    if _newer(LIB_GPU, objs):
        tmp = LIB_GPU + f".tmp{os.getpid()}"
        _run([nvcc] + ARCH_FLAGS + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB_GPU)
    return LIB_GPU


def module_path():
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    return os.path.join(HERE, "libffrs" + suffix)


def build_module():
    os.makedirs(OBJ, exist_ok=True)
    out = module_path()
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    hdrs = glob.glob(os.path.join(HOST, "*.h")) + [os.path.join(ROOT, "include", "ffgpu.h")]
    if not _newer(out, srcs + hdrs + [LIB_GPU]):
        return out
    cxx = os.environ.get("CXX", "g++")
    inc = [
        "-I" + _pybind_include(),
        "-I" + sysconfig.get_paths()["include"],
        "-I" + os.path.join(ROOT, "include"),
        "-I" + os.path.join(_cuda_home(), "include"),
    ]
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OBJ, "host_" + os.path.basename(s) + ".o")
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-w"] + inc + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    tmp = out + f".tmp{os.getpid()}"
    _run([cxx, "-shared", "-o", tmp] + objs + ["-L" + HERE, "-lffgpu", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, out)
    return out


def build(verbose=False):
    build_gpu_lib(verbose=verbose)
    return build_module()


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
