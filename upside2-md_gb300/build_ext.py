"""Build the in-tree shared libraries of the GB300 Upside engine.

  libupside.so          the engine: sm_103a kernels + drop-in C ABI + batch API
                        + the upside driver (upside_main)
  upside                the upside command line over libupside.so
  libupside_h5lite.so   HDF5-subset reader and writer for Python (config/fixture tools)

Compilation runs in parallel, one process per translation unit, and only
rebuilds what is older than its sources.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")

CU_SOURCES = ["engine.cu", "graph.cu", "pairlist.cu", "warm.cu", "capi.cu", "driver.cu", "mc.cu", "remd.cu"]
HEADERS = ["engine.h", "graph.h", "warm.h", "mc.h", "remd.h", "dev_math.cuh", "launch.cuh", "surface.cuh", "h5lite.h"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(HERE, "..", "include", "engine_c_library.h"),
        os.path.join(HERE, "..", "include", "upside_gb300.h"),
        os.path.join(HERE, "..", "include", "upside_main.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([NVCC] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                         "-c", s, "-o", o])
    h5o = os.path.join(BUILD, "h5lite.o")
    if _stale(h5o, [os.path.join(CSRC, "h5lite.cpp"), os.path.join(CSRC, "h5lite.h")]):
        jobs.append([CXX, "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, "h5lite.cpp"), "-o", h5o])
    h5w = os.path.join(BUILD, "h5lite_write.o")
    if _stale(h5w, [os.path.join(CSRC, "h5lite_write.cpp"), os.path.join(CSRC, "h5lite.h")]):
        jobs.append([CXX, "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, "h5lite_write.cpp"), "-o", h5w])
    capo = os.path.join(BUILD, "h5lite_capi.o")
    if _stale(capo, [os.path.join(CSRC, "h5lite_capi.cpp"), os.path.join(CSRC, "h5lite.h")]):
        jobs.append([CXX, "-O2", "-std=c++17", "-fPIC", "-c", os.path.join(CSRC, "h5lite_capi.cpp"), "-o", capo])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(HERE, "libupside.so")
    if _stale(lib, objs + [h5o, h5w]):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + [h5o, h5w])
    exe = os.path.join(HERE, "upside")
    cli = os.path.join(CSRC, "upside_cli.cpp")
    if _stale(exe, [lib, cli]):
        _run([CXX, "-O2", "-std=c++17", "-o", exe, cli, "-L" + HERE, "-lupside", "-Wl,-rpath,$ORIGIN"])
    h5lib = os.path.join(HERE, "libupside_h5lite.so")
    if _stale(h5lib, [h5o, h5w, capo]):
        _run([CXX, "-shared", "-o", h5lib, h5o, h5w, capo])
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", os.path.join(HERE, "libupside.so"))
