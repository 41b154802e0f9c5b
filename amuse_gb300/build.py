"""Build the in-tree shared libraries (no cmake, no torch extension machinery).

  amuse_gb300/lib/libsapporo.so  -- the drop-in GRAPE-6 ABI library
                                   (C host + sm_103a CUDA kernels, cudart static)
  amuse_gb300/lib/libg6drive.so  -- a small C caller that drives the ABI the
                                   way ph4's gpu.cc does (chunked by npipes);
                                   used by tests and the benchmark's e2e leg.

Every .cu is compiled once for sm_103a only; translation units build in
parallel.  ``python -m amuse_gb300.build`` or ``build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["kern_force.cu", "kern_predict.cu", "kern_step.cu", "kern_ngb.cu", "kern_batch.cu",
              "kern_fixed.cu", "kern_knn.cu"]
C_SOURCES = ["g6_host.c", "g6_struct.c"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _newer(src_list, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def build(verbose=False, force=False):
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    headers = [os.path.join(CSRC, "g6_dev.h"), os.path.join(CSRC, "f32x2.cuh"),
               os.path.join(CSRC, "pdl.cuh"), os.path.join(INCLUDE, "g6.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _newer([s] + headers, o):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I", CSRC, "-I", INCLUDE, "-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or _newer([s] + headers, o):
            jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-Wall", "-Wno-unused-function",
                         "-I", CSRC, "-I", INCLUDE, "-I", os.path.join(cuda, "include"),
                         "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    so = os.path.join(LIB, "libsapporo.so")
    vscript = os.path.join(OBJ, "exports.map")
    with open(vscript, "w") as f:  # export the public ABI only (g6*, g6x*)
        f.write("{ global: g6_*; g6calc*; g6x_*; local: *; };\n")
    if force or _newer(objs, so):
        _run([nvcc, *ARCH, "-shared", "-o", so, *objs, "-lpthread", "-ldl", "-lrt",
              "-Xlinker", "--version-script=" + vscript])
    # pkg-config file under the name AMUSE's configure scripts look for
    # (lib/sapporo_light/Makefile:5-24 installs sapporo_light.pc)
    with open(os.path.join(LIB, "sapporo_light.pc"), "w") as f:
        f.write(f"prefix={ROOT}\nlibdir={LIB}\nincludedir={INCLUDE}\n\n"
                "Name: sapporo_light\nDescription: GRAPE-6 ABI on GB300 (sm_103a)\n"
                "Version: 2.0\nLibs: -L${libdir} -lsapporo -Wl,-rpath,${libdir}\n"
                "Cflags: -I${includedir}\n")
    drv_src = os.path.join(CSRC, "g6_ph4drive.c")
    drv = os.path.join(LIB, "libg6drive.so")
    if force or _newer([drv_src, so] + headers, drv):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-I", INCLUDE, "-o", drv, drv_src,
              "-L", LIB, "-lsapporo", "-Wl,-rpath,$ORIGIN"])
    return so


if __name__ == "__main__":
    print(build(verbose=True))
