"""Build recipe of the native library: every CUDA translation unit for sm_103a (nvcc),
the host setup with g++, linked into valomc_gb300/_build/libvalomc_gb300.so, plus the
drop-in executables MC2D / MC3D.  Units compile in parallel; an up-to-date library is
not rebuilt."""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libvalomc_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_UNITS = ["kern3d32.cu", "kern3d64.cu", "kern2d32.cu", "kern2d64.cu", "runtime.cu", "tools.cu", "server.cu",
            "noalloc.cu"]
CPP_UNITS = ["host_setup.cpp"]
APPS = {"MC3D": "app/mc3d_main.cpp", "MC2D": "app/mc2d_main.cpp", "vmc_textdump": "app/textdump.cpp"}


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources_mtime():
    files = glob.glob(os.path.join(CSRC, "**", "*"), recursive=True) + glob.glob(os.path.join(INCLUDE, "*.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files if os.path.isfile(f))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False, jobs=None):
    """Compile the library (and the executables) if any source is newer than it."""
    os.makedirs(BUILD, exist_ok=True)
    outputs = [LIB] + [os.path.join(BUILD, a) for a in APPS if os.path.exists(os.path.join(CSRC, APPS[a]))]
    if not force and all(os.path.exists(o) for o in outputs) and \
            min(os.path.getmtime(o) for o in outputs) >= _sources_mtime():
        return LIB
    nv = nvcc()
    cuflags = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-I" + INCLUDE, "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
                      "--expt-relaxed-constexpr"]
    cmds = []
    objs = []
    for u in CU_UNITS:
        o = os.path.join(BUILD, u.replace(".cu", ".o"))
        cmds.append([nv] + cuflags + ["-c", os.path.join(CSRC, u), "-o", o])
        objs.append(o)
    for u in CPP_UNITS:
        o = os.path.join(BUILD, u.replace(".cpp", ".o"))
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-I" + INCLUDE,
                     "-I/usr/local/cuda/include", "-c", os.path.join(CSRC, u), "-o", o])
        objs.append(o)
    with ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = LIB + ".tmp"
    _run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    for app, src in APPS.items():
        path = os.path.join(CSRC, src)
        if os.path.exists(path):
            _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I" + INCLUDE, path, "-o", os.path.join(BUILD, app),
                  "-L" + BUILD, "-lvalomc_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
