"""Builds libhqs.so (CUDA kernels + host engine + C ABI) and the pybind11
module _cppsim_mpi in place, for sm_103a, with nvcc and g++ directly.

Objects go to hiqsimulator_gb300/_build/; the two shared libraries sit in the
package directory. Sources are rebuilt only when newer than their object.
"""
import os
import shutil
import subprocess
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["kernels.cu", "umma_pass.cu", "noalloc.cu"]
CXX_SOURCES = ["fusion.cpp", "workspace.cpp", "engine.cpp", "scheduler.cpp", "server.cpp", "capi.cpp"]
HEADERS = ["hqs_desc.h", "hqs_kernels.h", "hqs_arith.cuh", "hqs_tc05.cuh", "fusion.h", "workspace.h", "engine.h", "server.h"]

LIB = os.path.join(PKG, "libhqs.so")
EXT = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
PYMOD = os.path.join(PKG, "_cppsim_mpi" + EXT)


def _pybind_include():
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        pass
    try:
        import torch
        inc = os.path.join(os.path.dirname(torch.__file__), "include")
        if os.path.isdir(os.path.join(inc, "pybind11")):
            return inc
    except ImportError:
        pass
    raise RuntimeError("pybind11 headers not found (neither the pybind11 package nor torch/include)")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _stale(target, deps):
    return not os.path.exists(target) or os.path.getmtime(target) < _newest(deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False):
    """Compile everything that is out of date. Returns the library paths."""
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "hqs.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([NVCC] + GENCODE + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                                            "-Xptxas", "-v" if verbose else "-O3", "-I", INCLUDE, "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", os.path.join(CUDA_HOME, "include"),
                         "-I", INCLUDE, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            print(o)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([NVCC] + GENCODE + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    pysrc = os.path.join(CSRC, "pymodule.cpp")
    if _stale(PYMOD, [pysrc, LIB, os.path.join(INCLUDE, "hqs.h")]):
        tmp = PYMOD + ".tmp"
        _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
              "-I", _pybind_include(), "-I", sysconfig.get_paths()["include"], "-I", INCLUDE,
              pysrc, "-o", tmp, "-L", PKG, "-lhqs", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, PYMOD)
    return LIB, PYMOD


def build_sanitized():
    """A copy of libhqs.so whose host C++ (engine, fusion, planner, scheduler,
    server, C ABI) is built with AddressSanitizer and UndefinedBehaviorSanitizer,
    linked with the regular kernel objects, in _build/asan/. A process loads it
    with the sanitizer runtimes preloaded (LD_PRELOAD). Returns its path."""
    build()
    out = os.path.join(OBJ, "asan")
    os.makedirs(out, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "hqs.h")]
    flags = ["-O1", "-g", "-std=c++17", "-fPIC", "-fsanitize=address,undefined", "-fno-omit-frame-pointer"]
    jobs, objs = [], []
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++"] + flags + ["-I", os.path.join(CUDA_HOME, "include"), "-I", INCLUDE, "-c", s,
                                           "-o", o])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(_run, jobs))
    lib = os.path.join(out, "libhqs.so")
    cu_objs = [os.path.join(OBJ, src + ".o") for src in CU_SOURCES]
    if _stale(lib, objs + cu_objs):
        _run([NVCC] + GENCODE + ["-shared", "-Xcompiler", "-fPIC", "-o", lib + ".tmp"] + objs + cu_objs +
             ["-Xlinker", "-lasan", "-Xlinker", "-lubsan"])
        os.replace(lib + ".tmp", lib)
    return lib


def clean():
    shutil.rmtree(OBJ, ignore_errors=True)
    for p in (LIB, PYMOD):
        if os.path.exists(p):
            os.remove(p)
