"""Calls the MC3Dmex / MC2Dmex gateways through the mex stand-in (mexshim.cpp), with numpy
arrays as mxArrays.  Test infrastructure only."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(ROOT, "valomc_gb300", "_build")

CLS = {"logical": 3, "char": 4, "double": 6, "int8": 8, "uint8": 9, "int64": 14, "uint64": 15}
DT = {6: np.float64, 8: np.int8, 9: np.uint8, 14: np.int64, 15: np.uint64, 3: np.uint8}


def build(dim):
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, f"mc{dim}dmex_shim.so")
    src = [os.path.join(HERE, "mexshim.cpp"), os.path.join(ROOT, "valomc_gb300", "csrc", "mex", f"MC{dim}Dmex.cpp")]
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(s) for s in src + [os.path.join(LIBDIR, "libvalomc_gb300.so")]):
        subprocess.run(["g++", "-O1", "-std=c++17", "-fPIC", "-shared", "-I" + HERE, "-I" + os.path.join(ROOT, "include")]
                       + src + ["-L" + LIBDIR, "-lvalomc_gb300", "-Wl,-rpath," + LIBDIR, "-o", out], check=True)
    L = C.CDLL(out)
    L.shim_create.restype = C.c_void_p
    L.shim_create.argtypes = [C.c_int, C.c_size_t, C.c_size_t, C.c_int, C.c_void_p, C.c_void_p]
    L.shim_invoke.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]
    L.shim_error.restype = C.c_char_p
    L.shim_log.restype = C.c_char_p
    for f in ("mxGetData", "mxGetImagData"):
        getattr(L, f).restype = C.c_void_p
        getattr(L, f).argtypes = [C.c_void_p]
    for f in ("shim_m", "shim_n"):
        getattr(L, f).restype = C.c_size_t
        getattr(L, f).argtypes = [C.c_void_p]
    L.shim_class.argtypes = [C.c_void_p]
    L.shim_is_complex.argtypes = [C.c_void_p]
    return L


def mx(L, a, cls):
    a = np.asfortranarray(np.asarray(a, dtype=DT[CLS[cls]]))
    if a.ndim == 0:
        a = a.reshape(1, 1)
    if a.ndim == 1:
        a = a.reshape(-1, 1, order="F")
    m, n = a.shape
    return L.shim_create(CLS[cls], m, n, 0, a.ctypes.data if a.size else None, None)


def read(L, p):
    m, n, cls = L.shim_m(p), L.shim_n(p), L.shim_class(p)
    dt = DT[cls]
    cnt = m * n
    re = np.ctypeslib.as_array(C.cast(L.mxGetData(p), C.POINTER(C.c_char)), shape=(cnt * np.dtype(dt).itemsize,))
    re = np.frombuffer(bytes(re), dtype=dt).reshape(n, m).T
    if L.shim_is_complex(p):
        im = np.ctypeslib.as_array(C.cast(L.mxGetImagData(p), C.POINTER(C.c_char)), shape=(cnt * 8,))
        re = re + 1j * np.frombuffer(bytes(im), dtype=dt).reshape(n, m).T
    return re


def args_for(L, p, hn=None, disable_pbar=1, seed=None, dtype_cls="int8"):
    """The argument list ValoMC.m builds (ValoMC.m:128-157,338), 0-based int64 indices."""
    nb = p.Nb
    a = [mx(L, p.H, "int64"), mx(L, np.zeros((0, 0)) if hn is None else hn, "int64"), mx(L, p.BH, "int64"),
         mx(L, p.r, "double"), mx(L, p.BCType.astype(np.int8), dtype_cls),
         mx(L, p.BCIntensity if p.BCIntensity is not None else np.ones(nb), "double"),
         mx(L, (p.BCLightDirectionType if p.BCLightDirectionType is not None else np.full(nb, ord("n"))).astype(np.int8),
            dtype_cls),
         mx(L, p.BCLNormal if p.BCLNormal is not None else np.zeros((nb, p.dim)), "double"),
         mx(L, p.BCn, "double"), mx(L, p.mua, "double"), mx(L, p.mus, "double"), mx(L, p.g, "double"),
         mx(L, p.n, "double"), mx(L, np.array([p.f]), "double"), mx(L, np.array([p.phase0]), "double"),
         mx(L, np.array([p.Nphoton]), "int64")]
    if p.dim == 2:
        a.append(mx(L, p.GaussianSigma if p.GaussianSigma is not None else np.ones(nb), "double"))
    a.append(mx(L, np.array([disable_pbar]), "int64"))
    a.append(mx(L, np.array([p.seed if seed is None else seed, 1]), "uint64"))
    return a


def call(L, args, nlhs=5):
    prhs = (C.c_void_p * len(args))(*args)
    plhs = (C.c_void_p * max(nlhs, 1))()
    rc = L.shim_invoke(nlhs, plhs, len(args), prhs)
    if rc:
        return None, L.shim_error().decode()
    return [read(L, plhs[i]) for i in range(nlhs)], None
