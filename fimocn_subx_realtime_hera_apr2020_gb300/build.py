"""In-tree build of libfimgpu.so (CUDA kernels for sm_103a + C-ABI + grid builder).

Translation units compile in parallel with nvcc (one -gencode, sm_103a) and
g++; the shared library lands in fimocn_subx_realtime_hera_apr2020_gb300/_lib/.
Nothing is installed into site-packages.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIBNAME = "libfimgpu.so"
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

CU_SOURCES = ["fim_dyn.cu", "fim_col.cu", "fim_trc.cu", "fim_trb.cu", "fim_cpl.cu", "fim_synth.cu", "fim_capi.cu"]
CPP_SOURCES = ["fim_grid.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else shutil.which("nvcc") or "nvcc"


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _deps():
    files = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + ["fim_internal.h"]]
    files.append(os.path.join(INCLUDE, "fim_gpu.h"))
    return files


def _up_to_date():
    lib = lib_path()
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(f) <= t for f in _deps())


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res.stdout + res.stderr


def build_library(force=False, verbose=False, extra_nvcc=()):
    """Compile and link libfimgpu.so unless it is newer than every source."""
    if not force and _up_to_date():
        return lib_path()
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(BUILD, f.replace(".cu", ".o"))
        objs.append(o)
        jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                     "-I" + INCLUDE, "-c", os.path.join(CSRC, f), "-o", o] + list(extra_nvcc))
    for f in CPP_SOURCES:
        o = os.path.join(BUILD, f.replace(".cpp", ".o"))
        objs.append(o)
        jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-I" + INCLUDE, "-c", os.path.join(CSRC, f), "-o", o])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    tmp = lib_path() + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
