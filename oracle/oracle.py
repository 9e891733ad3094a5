"""ctypes front end of the CPU oracle (oracle/vmc_oracle.c) and of the reference harness
binaries in oracle/_ref/.  TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check
and bench.py's CPU-baseline leg, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import tempfile
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libvmc_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

RNG_MT, RNG_PHILOX, RNG_TAPE = 0, 1, 2
INT64_MIN = -(2 ** 63)
EV_ROULETTE = INT64_MIN + 1
EV_LOST = INT64_MIN + 2
EV_CAPPED = INT64_MIN + 3
EV_TAPE_END = INT64_MIN + 4
EV_TRUNCATED = INT64_MIN + 5
LEDGER = ["launched", "absorbed", "exited", "roulette_kill", "roulette_gain", "lost"]

_p64 = C.POINTER(C.c_int64)
_pd = C.POINTER(C.c_double)
_pc = C.POINTER(C.c_char)


class VoProblem(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("rng_kind", C.c_int32), ("nthreads", C.c_int32), ("hn_given", C.c_int32),
        ("Ne", C.c_int64), ("Nb", C.c_int64), ("Nr", C.c_int64),
        ("H", _p64), ("HN", _p64), ("BH", _p64), ("r", _pd),
        ("mua", _pd), ("mus", _pd), ("g", _pd), ("n", _pd),
        ("n_mua", C.c_int64), ("n_mus", C.c_int64), ("n_g", C.c_int64), ("n_n", C.c_int64),
        ("BCType", _pc), ("n_BCType", C.c_int64),
        ("BCn", _pd), ("n_BCn", C.c_int64),
        ("BCLNormal", _pd), ("n_BCLNormal", C.c_int64),
        ("BCLightDirectionType", _pc), ("n_BCLDT", C.c_int64),
        ("BCIntensity", _pd), ("n_BCIntensity", C.c_int64),
        ("GaussianSigma", _pd), ("n_GaussianSigma", C.c_int64),
        ("f", C.c_double), ("phase0", C.c_double),
        ("Nphoton", C.c_int64), ("seed", C.c_uint64), ("stream", C.c_uint32),
        ("max_steps", C.c_int64),
        ("tape", C.POINTER(C.c_uint32)), ("tape_off", _p64),
        ("ER", _pd), ("EI", _pd), ("EBR", _pd), ("EBI", _pd), ("DEBR", _pd), ("DEBI", _pd),
        ("normalize", C.c_int32), ("pad0", C.c_int32),
        ("loss", C.c_int64), ("steps", C.c_int64), ("scatters", C.c_int64),
        ("photons_done", C.c_int64), ("capped", C.c_int64),
        ("ledger", C.c_double * 8),
        ("trace", _p64), ("trace_len", _p64), ("trace_stride", C.c_int64), ("trace_photons", C.c_int64),
        ("seconds", C.c_double), ("photon_offset", C.c_int64),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.vo_run.argtypes = [C.POINTER(VoProblem)]
        _lib.vo_run.restype = C.c_int
        _lib.vo_build_neighbours.argtypes = [C.POINTER(VoProblem)]
        _lib.vo_build_neighbours.restype = C.c_int
        _lib.vo_error_checks.argtypes = [C.POINTER(VoProblem)]
        _lib.vo_error_checks.restype = C.c_int
        _lib.vo_mt_words.argtypes = [C.c_uint64, C.POINTER(C.c_uint32), C.c_int64]
        _lib.vo_philox_words.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32), C.c_int64]
        _lib.vo_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        _lib.vo_philox4x64_10.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        _lib.vo_max_threads.restype = C.c_int
    return _lib


def build(quiet=True):
    """make the oracle library (and oracle/_ref/ when the reference tree is present)."""
    cmd = ["make", "-s", "-f", os.path.join(HERE, "Makefile"), "all"]
    subprocess.run(cmd, check=True, capture_output=quiet)


# the reference tree the checker's recipes read (the Makefile's REF): by default the copy
# staged under baseline/_ref/ValoMC, which goes with the working tree to a GPU host
REF_TREE = os.environ.get("REF", os.path.join(os.path.dirname(HERE), "baseline", "_ref", "ValoMC"))


def reference_file(rel):
    """Path of a file of the reference tree, or None where the tree is absent."""
    path = os.path.join(REF_TREE, rel)
    return path if os.path.exists(path) else None


def have_reference_binaries() -> bool:
    return all(os.path.exists(os.path.join(REF_DIR, b)) for b in ("ref3d_run", "ref2d_run", "ref3d_trace", "ref2d_trace"))


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def colmajor(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype)).ravel(order="F").copy()


@dataclass
class OracleResult:
    status: int
    ER: np.ndarray
    EI: np.ndarray
    EBR: np.ndarray
    EBI: np.ndarray
    DEBR: np.ndarray
    DEBI: np.ndarray
    HN: np.ndarray
    loss: int
    steps: int
    scatters: int
    capped: int
    ledger: dict
    seconds: float
    traces: Optional[list] = None


def run(p, rng=RNG_MT, nthreads=1, normalize=True, seed=None, stream=0, max_steps=0,
        tape=None, tape_off=None, trace_photons=0, trace_stride=100000, nphoton=None, photon_offset=0):
    """Run ErrorChecks + Init + MonteCarlo of the oracle on Problem ``p``."""
    L = lib()
    D = p.dim
    keep = []
    P = VoProblem()
    P.dim, P.rng_kind, P.nthreads = D, rng, nthreads
    Ne, Nb, Nr = p.Ne, p.Nb, p.Nr
    P.Ne, P.Nb, P.Nr = Ne, Nb, Nr
    H = colmajor(p.H, np.int64)
    BH = colmajor(p.BH, np.int64)
    r = colmajor(p.r, np.float64)
    if p.HN is not None:
        HN = colmajor(p.HN, np.int64)
        P.hn_given = 1
    else:
        HN = np.zeros(Ne * (D + 1), np.int64)
        P.hn_given = 0
    keep += [H, BH, r, HN]
    P.H, P.BH, P.r, P.HN = _ptr(H, C.c_int64), _ptr(BH, C.c_int64), _ptr(r, C.c_double), _ptr(HN, C.c_int64)
    arrs = {}
    for nm in ("mua", "mus", "g", "n"):
        a = np.ascontiguousarray(getattr(p, nm), dtype=np.float64)
        arrs[nm] = a
        setattr(P, nm, _ptr(a, C.c_double))
        setattr(P, "n_" + nm, len(a))
    bct = np.ascontiguousarray(p.BCType, dtype=np.uint8)
    P.BCType, P.n_BCType = bct.ctypes.data_as(_pc), len(bct)
    keep += [bct, arrs]
    if p.BCn is not None:
        bcn = np.ascontiguousarray(p.BCn, dtype=np.float64)
        P.BCn, P.n_BCn = _ptr(bcn, C.c_double), len(bcn)
        keep.append(bcn)
    if p.BCLNormal is not None:
        bl = colmajor(p.BCLNormal, np.float64)
        P.BCLNormal, P.n_BCLNormal = _ptr(bl, C.c_double), p.BCLNormal.shape[0]
        keep.append(bl)
    dt = np.zeros(max(Nb, 1), np.uint8)
    if p.BCLightDirectionType is not None:
        dt[: len(p.BCLightDirectionType)] = p.BCLightDirectionType
        P.n_BCLDT = len(p.BCLightDirectionType)
    P.BCLightDirectionType = dt.ctypes.data_as(_pc)
    keep.append(dt)
    if p.BCIntensity is not None:
        bi = np.ascontiguousarray(p.BCIntensity, dtype=np.float64)
        P.BCIntensity, P.n_BCIntensity = _ptr(bi, C.c_double), len(bi)
        keep.append(bi)
    if p.GaussianSigma is not None:
        gs = np.ascontiguousarray(p.GaussianSigma, dtype=np.float64)
        P.GaussianSigma, P.n_GaussianSigma = _ptr(gs, C.c_double), len(gs)
        keep.append(gs)
    # callers wrap a negative phase0 into [0, 2 pi) before Init (cpp/3d/MC3D.cpp:141-143,
    # cpp/3d/MC3Dmex.cpp:158-160)
    ph0 = float(p.phase0)
    if ph0 < 0:
        ph0 += 2 * math.pi * math.ceil(-ph0 / (2 * math.pi))
    P.f, P.phase0 = p.f, ph0
    N = int(nphoton if nphoton is not None else p.Nphoton)
    P.Nphoton = N
    P.seed = int(p.seed if seed is None else seed)
    P.stream = stream
    P.max_steps = max_steps
    P.photon_offset = photon_offset
    if tape is not None:
        tape = np.ascontiguousarray(tape, dtype=np.uint32)
        tape_off = np.ascontiguousarray(tape_off, dtype=np.int64)
        P.tape, P.tape_off = _ptr(tape, C.c_uint32), _ptr(tape_off, C.c_int64)
        keep += [tape, tape_off]
    out = {k: np.zeros(Ne if k in ("ER", "EI") else Nb, np.float64) for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI")}
    for k, a in out.items():
        setattr(P, k, _ptr(a, C.c_double))
    P.normalize = 1 if normalize else 0
    tr = trl = None
    if trace_photons:
        tr = np.zeros(trace_photons * trace_stride, np.int64)
        trl = np.zeros(trace_photons, np.int64)
        P.trace, P.trace_len, P.trace_stride, P.trace_photons = _ptr(tr, C.c_int64), _ptr(trl, C.c_int64), trace_stride, trace_photons
    st = L.vo_run(C.byref(P))
    traces = None
    if trace_photons:
        traces = [tr[i * trace_stride: i * trace_stride + trl[i]].copy() for i in range(trace_photons)]
    return OracleResult(st, out["ER"], out["EI"], out["EBR"], out["EBI"], out["DEBR"], out["DEBI"],
                        HN.reshape(D + 1, Ne).T.copy(), P.loss, P.steps, P.scatters, P.capped,
                        {k: P.ledger[i] for i, k in enumerate(LEDGER)}, P.seconds, traces)


def build_neighbours(p):
    """HN of the reference's BuildNeighbourhoods (status, HN (Ne, dim+1))."""
    L = lib()
    D = p.dim
    P = VoProblem()
    P.dim = D
    P.Ne, P.Nb, P.Nr = p.Ne, p.Nb, p.Nr
    H = colmajor(p.H, np.int64)
    BH = colmajor(p.BH, np.int64)
    HN = np.zeros(p.Ne * (D + 1), np.int64)
    P.H, P.BH, P.HN = _ptr(H, C.c_int64), _ptr(BH, C.c_int64), _ptr(HN, C.c_int64)
    st = L.vo_build_neighbours(C.byref(P))
    return st, HN.reshape(D + 1, p.Ne).T.copy()


def mt_words(seed, n):
    out = np.zeros(n, np.uint32)
    lib().vo_mt_words(seed, _ptr(out, C.c_uint32), n)
    return out


def philox_words(seed, stream, photon, n):
    out = np.zeros(n, np.uint32)
    lib().vo_philox_words(seed, stream, photon, _ptr(out, C.c_uint32), n)
    return out


def philox4x32(ctr, key):
    c = np.asarray(ctr, np.uint32).copy()
    k = np.asarray(key, np.uint32).copy()
    o = np.zeros(4, np.uint32)
    lib().vo_philox4x32_10(_ptr(c, C.c_uint32), _ptr(k, C.c_uint32), _ptr(o, C.c_uint32))
    return o


def philox4x64(ctr, key):
    c = np.asarray(ctr, np.uint64).copy()
    k = np.asarray(key, np.uint64).copy()
    o = np.zeros(4, np.uint64)
    lib().vo_philox4x64_10(_ptr(c, C.c_uint64), _ptr(k, C.c_uint64), _ptr(o, C.c_uint64))
    return o


# ---------------------------------------------------------------------------
# reference harness binaries (present only where the reference tree was built)
# ---------------------------------------------------------------------------

def _parse_dump(lines, start):
    i = start
    assert lines[i].startswith("ER_EI")
    ne = int(lines[i].split()[1])
    a = np.array([[float(x) for x in ln.split()] for ln in lines[i + 1:i + 1 + ne]]).reshape(ne, 2)
    i += 1 + ne
    assert lines[i].startswith("EBR_EBI")
    nb = int(lines[i].split()[1])
    b = np.array([[float(x) for x in ln.split()] for ln in lines[i + 1:i + 1 + nb]]).reshape(nb, 4)
    return dict(ER=a[:, 0], EI=a[:, 1], EBR=b[:, 0], EBI=b[:, 1], DEBR=b[:, 2], DEBI=b[:, 3])


def ref_run(p, nthreads=1, workdir=None):
    """The reference engine's MonteCarlo() on ``p`` (MT19937, OpenMP), full precision."""
    from valomc_gb300 import meshgen
    exe = os.path.join(REF_DIR, "ref3d_run" if p.dim == 3 else "ref2d_run")
    with tempfile.TemporaryDirectory(dir=workdir) as td:
        fin, fout = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
        meshgen.write_input(fin, p)
        res = subprocess.run([exe, fin, fout, str(nthreads)], capture_output=True, text=True)
        if res.returncode == 3:
            code = int(res.stdout.split("MCERROR")[1].split()[0])
            return dict(status=1 + code)
        res.check_returncode()
        lines = open(fout).read().splitlines()
    st = lines[0].split()
    out = _parse_dump(lines, 1)
    out.update(status=0, seconds=float(st[2]), loss=int(st[4]), threads=int(st[6]))
    return out


def ref_trace(p, tape, tape_off, workdir=None):
    """Replay: per photon the reference's logged element sequence and terminal code."""
    from valomc_gb300 import meshgen
    exe = os.path.join(REF_DIR, "ref3d_trace" if p.dim == 3 else "ref2d_trace")
    nphot = len(tape_off) - 1
    codes = {"ROULETTE": EV_ROULETTE, "LOST": EV_LOST, "TAPE_END": EV_TAPE_END}
    with tempfile.TemporaryDirectory(dir=workdir) as td:
        fin, ftape, fout = (os.path.join(td, x) for x in ("in.txt", "tape.bin", "out.txt"))
        meshgen.write_input(fin, p)
        with open(ftape, "wb") as fp:
            fp.write(np.int64(nphot).tobytes())
            fp.write(np.asarray(tape_off, np.int64).tobytes())
            fp.write(np.asarray(tape, np.uint32).tobytes())
        subprocess.run([exe, fin, ftape, fout], check=True, capture_output=True)
        lines = open(fout).read().splitlines()
    traces, used = [], []
    for i in range(nphot):
        head, _, body = lines[i].partition(":")
        h = head.split()
        used.append(int(h[3]))
        ev = [int(x) for x in body.split()]
        if len(h) > 6:
            ev.append(codes[h[6]])
        traces.append(np.array(ev, dtype=np.int64))
    acc = _parse_dump(lines, nphot)
    return traces, used, acc
