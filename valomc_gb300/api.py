"""Python binding of the C ABI (include/valomc_gb300.h) through ctypes.

``run(problem, ...)`` is the equivalent of one MC3Dmex / MC2Dmex call
(cpp/3d/MC3Dmex.cpp:98-253): the same arrays in, element fluence, boundary exitance and
the direction-weighted exitance out.  The compute path is the CUDA library only; when it
is missing or no sm_103 device is present the calls raise instead of computing anything
on the CPU.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import build as _build

VMC_FP64, VMC_FP32 = 0, 1
VMC_RNG_PHILOX, VMC_RNG_TAPE = 0, 1
INT64_MIN = -(2 ** 63)
EV_ROULETTE, EV_LOST, EV_CAPPED, EV_TAPE_END, EV_TRUNCATED = (INT64_MIN + k for k in range(1, 6))
LEDGER = ["launched", "absorbed", "exited", "roulette_kill", "roulette_gain", "lost"]

STATUS = {
    0: "VMC_OK", 1: "VMC_NO_LIGHTSOURCE", 2: "VMC_SIZE_MISMATCH_G", 3: "VMC_SIZE_MISMATCH_MUA",
    4: "VMC_SIZE_MISMATCH_MUS", 5: "VMC_SIZE_MISMATCH_N", 6: "VMC_SIZE_MISMATCH_BCN", 7: "VMC_MISSING_BCN",
    8: "VMC_SIZE_MISMATCH_BCTYPE", 9: "VMC_SIZE_MISMATCH_LIGHT_DIRECTION",
    10: "VMC_SIZE_MISMATCH_LIGHT_DIRECTION_TYPE", 11: "VMC_INCONSISTENT_H", 12: "VMC_INCONSISTENT_BH",
    13: "VMC_INCONSISTENT_MESH", 14: "VMC_INCONSISTENT_MESH_DUPLICATE_NEIGHBORS", 15: "VMC_NO_GAUSSIAN_SIGMA",
    16: "VMC_MISSING_BOUNDARY", 32: "VMC_ERR_INVALID_ARGUMENT", 33: "VMC_ERR_CUDA", 34: "VMC_ERR_NO_DEVICE",
    35: "VMC_ERR_OUT_OF_MEMORY", 36: "VMC_ERR_CANCELLED", 37: "VMC_ERR_TIMEOUT", 38: "VMC_ERR_TAPE",
    39: "VMC_ERR_ADMISSION", 40: "VMC_ERR_NOT_FOUND", 41: "VMC_ERR_SIZE_LIMIT",
}

# every entry point the header declares (checked by the CPU tests)
EXPORTS = [
    "vmc_abi_version", "vmc_status_string", "vmc_last_error", "vmc_default_options", "vmc_run",
    "vmc_build_neighbourhood", "vmc_mesh_create", "vmc_mesh_destroy", "vmc_mesh_device_bytes", "vmc_run_batch",
    "vmc_autotune", "vmc_server_create", "vmc_server_add_mesh", "vmc_server_submit", "vmc_server_poll",
    "vmc_server_wait", "vmc_server_destroy", "vmc_bench_gather", "vmc_bench_fp64", "vmc_run_noalloc",
]

_p64 = C.POINTER(C.c_int64)
_pd = C.POINTER(C.c_double)
_pc = C.c_char_p
PROGRESS_FN = C.CFUNCTYPE(C.c_int, C.c_double, C.c_void_p)


class VmcInput(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("seed_given", C.c_int32),
        ("Ne", C.c_int64), ("Nb", C.c_int64), ("Nr", C.c_int64),
        ("H", _p64), ("HN", _p64), ("n_HN", C.c_int64), ("BH", _p64), ("r", _pd),
        ("BCType", C.c_void_p), ("n_BCType", C.c_int64),
        ("BCIntensity", _pd), ("n_BCIntensity", C.c_int64),
        ("BCLightDirectionType", C.c_void_p), ("n_BCLightDirectionType", C.c_int64),
        ("BCLNormal", _pd), ("n_BCLNormal", C.c_int64),
        ("BCn", _pd), ("n_BCn", C.c_int64),
        ("mua", _pd), ("n_mua", C.c_int64), ("mus", _pd), ("n_mus", C.c_int64),
        ("g", _pd), ("n_g", C.c_int64), ("n", _pd), ("n_n", C.c_int64),
        ("f", C.c_double), ("phase0", C.c_double), ("Nphoton", C.c_int64),
        ("GaussianSigma", _pd), ("n_GaussianSigma", C.c_int64),
        ("seed", C.c_uint64),
    ]


class VmcOutput(C.Structure):
    _fields_ = [("ER", _pd), ("EI", _pd), ("EBR", _pd), ("EBI", _pd), ("DEBR", _pd), ("DEBI", _pd), ("HN", _p64)]


class VmcOptions(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("rng", C.c_int32), ("device", C.c_int32), ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32), ("fetch_chunk", C.c_int32), ("max_steps", C.c_int64),
        ("timeout_s", C.c_double), ("stream_id", C.c_uint32), ("normalize", C.c_int32),
        ("progress", PROGRESS_FN), ("progress_user", C.c_void_p), ("cancel", C.POINTER(C.c_int32)),
        ("tape", C.POINTER(C.c_uint32)), ("tape_off", _p64), ("tape_photons", C.c_int64),
        ("trace", _p64), ("trace_len", _p64), ("trace_stride", C.c_int64), ("trace_photons", C.c_int64),
        ("photon_offset", C.c_int64), ("use_graph", C.c_int32), ("stage_slots", C.c_int32),
        ("refill_lanes", C.c_int32),
    ]


class VmcStats(C.Structure):
    _fields_ = [
        ("photons_requested", C.c_int64), ("photons_done", C.c_int64), ("loss", C.c_int64), ("capped", C.c_int64),
        ("steps", C.c_int64), ("scatters", C.c_int64), ("roulette_kills", C.c_int64), ("seed_used", C.c_uint64),
        ("seconds_setup", C.c_double), ("seconds_kernel", C.c_double), ("seconds_total", C.c_double),
        ("ledger", C.c_double * 8), ("grid_blocks", C.c_int32), ("block_size", C.c_int32),
        ("status_detail", C.c_int32), ("reserved", C.c_int32), ("bytes_h2d", C.c_int64), ("bytes_d2h", C.c_int64),
    ]


class VmcServerConfig(C.Structure):
    _fields_ = [
        ("device", C.c_int32), ("precision", C.c_int32), ("max_slots", C.c_int32), ("use_graph", C.c_int32),
        ("memory_budget", C.c_int64), ("epoch_photons", C.c_int64), ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32), ("slicing", C.c_int32), ("epoch_max_ms", C.c_int32),
    ]


class VmcNoallocBuffers(C.Structure):
    """Caller-owned device buffers of vmc_run_noalloc (device addresses as integers)."""
    _fields_ = [("optics", C.c_void_p), ("bctype", C.c_void_p), ("bcn", C.c_void_p), ("acc", C.c_void_p)]


class VmcError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = f"{where}: status {status} {STATUS.get(status, '?')}"
        try:
            msg += f" ({lib().vmc_status_string(status).decode()})"
            le = lib().vmc_last_error().decode()
            if le:
                msg += f" [{le}]"
        except Exception:
            pass
        super().__init__(msg)


_lib = None


def lib(build_if_missing=True):
    """The loaded native library (built on first use when missing)."""
    global _lib
    if _lib is None:
        path = os.environ.get("VALOMC_GB300_LIB", _build.LIB)  # an alternative build of the library
        if path == _build.LIB and not os.path.exists(path) and build_if_missing:
            _build.build()
        L = C.CDLL(path)
        L.vmc_status_string.restype = C.c_char_p
        L.vmc_status_string.argtypes = [C.c_int]
        L.vmc_last_error.restype = C.c_char_p
        L.vmc_default_options.argtypes = [C.POINTER(VmcOptions)]
        L.vmc_run.argtypes = [C.POINTER(VmcInput), C.POINTER(VmcOptions), C.POINTER(VmcOutput), C.POINTER(VmcStats)]
        L.vmc_build_neighbourhood.argtypes = [C.POINTER(VmcInput), _p64]
        L.vmc_mesh_create.argtypes = [C.POINTER(VmcInput), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]
        L.vmc_mesh_destroy.argtypes = [C.c_void_p]
        L.vmc_mesh_device_bytes.argtypes = [C.c_void_p]
        L.vmc_mesh_device_bytes.restype = C.c_int64
        L.vmc_run_batch.argtypes = [C.POINTER(C.c_void_p), C.POINTER(VmcInput), C.c_int32, C.POINTER(VmcOptions),
                                    C.POINTER(VmcOutput), C.POINTER(VmcStats), C.POINTER(VmcStats)]
        L.vmc_autotune.argtypes = [C.POINTER(C.c_void_p), C.POINTER(VmcInput), C.c_int32, C.POINTER(VmcOptions),
                                   C.c_double]
        L.vmc_server_create.argtypes = [C.POINTER(VmcServerConfig), C.POINTER(C.c_void_p)]
        L.vmc_server_add_mesh.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]
        L.vmc_server_submit.argtypes = [C.c_void_p, C.c_int32, C.POINTER(VmcInput), C.POINTER(C.c_int64)]
        L.vmc_server_poll.argtypes = [C.c_void_p, C.c_int64, C.POINTER(VmcOutput), C.POINTER(VmcStats)]
        L.vmc_server_wait.argtypes = [C.c_void_p, C.c_int64, C.POINTER(VmcOutput), C.POINTER(VmcStats), C.c_double]
        L.vmc_server_destroy.argtypes = [C.c_void_p]
        L.vmc_bench_gather.argtypes = [C.c_int32, C.c_int64, C.c_double, _pd]
        L.vmc_bench_fp64.argtypes = [C.c_int32, C.c_double, _pd]
        L.vmc_run_noalloc.argtypes = [C.c_void_p, C.POINTER(VmcInput), C.POINTER(VmcOptions),
                                      C.POINTER(VmcNoallocBuffers), C.POINTER(VmcOutput), C.POINTER(VmcStats)]
        _lib = L
    return _lib


def _ptr(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def colmajor(a, dtype):
    return np.asfortranarray(np.asarray(a, dtype=dtype)).ravel(order="F").copy()


class _Marshal:
    """Keeps the numpy buffers behind a VmcInput alive."""

    def __init__(self, p, geometry=True, nphoton=None, seed=None):
        self.keep = []
        s = VmcInput()
        D = p.dim
        s.dim = D
        s.Ne, s.Nb, s.Nr = p.Ne, p.Nb, p.Nr
        if geometry:
            self.H = colmajor(p.H, np.int64)
            self.BH = colmajor(p.BH, np.int64)
            self.r = colmajor(p.r, np.float64)
            s.H, s.BH, s.r = _ptr(self.H, C.c_int64), _ptr(self.BH, C.c_int64), _ptr(self.r)
            if p.HN is not None:
                self.HN = colmajor(p.HN, np.int64)
                s.HN, s.n_HN = _ptr(self.HN, C.c_int64), p.HN.shape[0]
        self.bct = np.ascontiguousarray(p.BCType, dtype=np.uint8)
        s.BCType, s.n_BCType = self.bct.ctypes.data, len(self.bct)
        for nm in ("mua", "mus", "g", "n"):
            a = np.ascontiguousarray(getattr(p, nm), dtype=np.float64)
            self.keep.append(a)
            setattr(s, nm, _ptr(a))
            setattr(s, "n_" + nm, len(a))
        if p.BCn is not None:
            a = np.ascontiguousarray(p.BCn, dtype=np.float64)
            self.keep.append(a)
            s.BCn, s.n_BCn = _ptr(a), len(a)
        if p.BCIntensity is not None:
            a = np.ascontiguousarray(p.BCIntensity, dtype=np.float64)
            self.keep.append(a)
            s.BCIntensity, s.n_BCIntensity = _ptr(a), len(a)
        if p.BCLightDirectionType is not None:
            a = np.ascontiguousarray(p.BCLightDirectionType, dtype=np.uint8)
            self.keep.append(a)
            s.BCLightDirectionType, s.n_BCLightDirectionType = a.ctypes.data, len(a)
        if p.BCLNormal is not None:
            a = colmajor(p.BCLNormal, np.float64)
            self.keep.append(a)
            s.BCLNormal, s.n_BCLNormal = _ptr(a), p.BCLNormal.shape[0]
        if p.GaussianSigma is not None:
            a = np.ascontiguousarray(p.GaussianSigma, dtype=np.float64)
            self.keep.append(a)
            s.GaussianSigma, s.n_GaussianSigma = _ptr(a), len(a)
        s.f, s.phase0 = float(p.f), float(p.phase0)
        s.Nphoton = int(p.Nphoton if nphoton is None else nphoton)
        sd = p.seed if seed is None else seed
        s.seed, s.seed_given = int(sd) & (2 ** 64 - 1), 1 if (p.seedflag or seed is not None) else 0
        self.s = s


@dataclass
class Result:
    ER: np.ndarray
    EI: np.ndarray
    EBR: np.ndarray
    EBI: np.ndarray
    DEBR: np.ndarray
    DEBI: np.ndarray
    HN: Optional[np.ndarray]
    stats: dict
    traces: Optional[list] = None


def stats_dict(st: VmcStats):
    d = {k: getattr(st, k) for k, _ in VmcStats._fields_ if k not in ("ledger", "reserved")}
    d["ledger"] = {k: st.ledger[i] for i, k in enumerate(LEDGER)}
    return d


def _outputs(Ne, Nb, dim, want_hn):
    arr = {k: np.zeros(Ne if k in ("ER", "EI") else Nb) for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI")}
    o = VmcOutput()
    for k, a in arr.items():
        setattr(o, k, _ptr(a))
    hn = None
    if want_hn:
        hn = np.zeros(Ne * (dim + 1), np.int64)
        o.HN = _ptr(hn, C.c_int64)
    return o, arr, hn


def options(precision=VMC_FP32, device=0, block_size=0, blocks_per_sm=0, fetch_chunk=0, max_steps=0,
            timeout_s=0.0, stream_id=0, normalize=True, progress=None, cancel=None, photon_offset=0, use_graph=False,
            stage_slots=None, refill_lanes=0):
    o = VmcOptions()
    lib().vmc_default_options(C.byref(o))
    o.use_graph = int(bool(use_graph))
    o.refill_lanes = int(refill_lanes)
    if stage_slots is not None:
        o.stage_slots = int(stage_slots)
    o.precision, o.device = precision, device
    o.block_size, o.blocks_per_sm, o.fetch_chunk, o.max_steps = block_size, blocks_per_sm, fetch_chunk, max_steps
    o.timeout_s, o.stream_id, o.normalize, o.photon_offset = timeout_s, stream_id, int(bool(normalize)), photon_offset
    keep = []
    if progress is not None:
        cb = PROGRESS_FN(lambda pct, user: int(bool(progress(pct))))
        o.progress = cb
        keep.append(cb)
    if cancel is not None:
        o.cancel = cancel.ctypes.data_as(C.POINTER(C.c_int32))
        keep.append(cancel)
    o._keep = keep
    return o


def run(p, precision=VMC_FP32, nphoton=None, seed=None, want_hn=False, tape=None, tape_off=None,
        trace_photons=0, trace_stride=100000, opts: Optional[VmcOptions] = None, check=True, **kw) -> Result:
    """One simulation of Problem ``p`` on the GPU (vmc_run)."""
    L = lib()
    m = _Marshal(p, nphoton=nphoton, seed=seed)
    o = opts if opts is not None else options(precision=precision, **kw)
    keep = []
    if tape is not None:
        tape = np.ascontiguousarray(tape, np.uint32)
        tape_off = np.ascontiguousarray(tape_off, np.int64)
        o.rng = VMC_RNG_TAPE
        o.tape, o.tape_off, o.tape_photons = _ptr(tape, C.c_uint32), _ptr(tape_off, C.c_int64), len(tape_off) - 1
        keep += [tape, tape_off]
    tr = trl = None
    if trace_photons:
        tr = np.zeros(trace_photons * trace_stride, np.int64)
        trl = np.zeros(trace_photons, np.int64)
        o.trace, o.trace_len = _ptr(tr, C.c_int64), _ptr(trl, C.c_int64)
        o.trace_stride, o.trace_photons = trace_stride, trace_photons
    out, arr, hn = _outputs(p.Ne, p.Nb, p.dim, want_hn)
    st = VmcStats()
    s = L.vmc_run(C.byref(m.s), C.byref(o), C.byref(out), C.byref(st))
    if s != 0 and check:
        raise VmcError(s, "vmc_run")
    traces = None
    if trace_photons:
        traces = [tr[i * trace_stride: i * trace_stride + trl[i]].copy() for i in range(trace_photons)]
    if hn is not None:
        hn = hn.reshape(p.dim + 1, p.Ne).T.copy()
    res = Result(arr["ER"], arr["EI"], arr["EBR"], arr["EBI"], arr["DEBR"], arr["DEBI"], hn, stats_dict(st), traces)
    res.stats["status"] = s
    return res


def build_neighbourhood(p):
    m = _Marshal(p)
    hn = np.zeros(p.Ne * (p.dim + 1), np.int64)
    s = lib().vmc_build_neighbourhood(C.byref(m.s), _ptr(hn, C.c_int64))
    return s, hn.reshape(p.dim + 1, p.Ne).T.copy()


class Mesh:
    """A resident mesh (vmc_mesh_create)."""

    def __init__(self, p, precision=VMC_FP32, device=0):
        self.dim, self.Ne, self.Nb, self.Nr = p.dim, p.Ne, p.Nb, p.Nr
        m = _Marshal(p)
        h = C.c_void_p()
        s = lib().vmc_mesh_create(C.byref(m.s), precision, device, C.byref(h))
        if s:
            raise VmcError(s, "vmc_mesh_create")
        self.h = h

    @property
    def device_bytes(self):
        return lib().vmc_mesh_device_bytes(self.h)

    def close(self):
        if self.h:
            lib().vmc_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_batch(meshes: Sequence[Mesh], problems, precision=VMC_FP32, opts=None, **kw):
    """Many problems in one persistent launch (vmc_run_batch); returns (results, totals)."""
    L = lib()
    n = len(problems)
    ms = [_Marshal(p, geometry=False) for p in problems]
    jobs = (VmcInput * n)(*[m.s for m in ms])
    hs = (C.c_void_p * n)(*[m.h for m in meshes])
    outs = (VmcOutput * n)()
    arrs = []
    for i, p in enumerate(problems):
        o, a, _ = _outputs(p.Ne, p.Nb, p.dim, False)
        outs[i] = o
        arrs.append(a)
    o = opts if opts is not None else options(precision=precision, **kw)
    st = VmcStats()
    jst = (VmcStats * n)()
    s = L.vmc_run_batch(hs, jobs, n, C.byref(o), outs, C.byref(st), jst)
    if s:
        raise VmcError(s, "vmc_run_batch")
    res = [Result(a["ER"], a["EI"], a["EBR"], a["EBI"], a["DEBR"], a["DEBI"], None, stats_dict(jst[i]))
           for i, a in enumerate(arrs)]
    return res, stats_dict(st)


def autotune(meshes, problems, precision=VMC_FP32, budget_s=2.0):
    n = len(problems)
    ms = [_Marshal(p, geometry=False) for p in problems]
    jobs = (VmcInput * n)(*[m.s for m in ms])
    hs = (C.c_void_p * n)(*[m.h for m in meshes])
    o = options(precision=precision)
    s = lib().vmc_autotune(hs, jobs, n, C.byref(o), budget_s)
    if s:
        raise VmcError(s, "vmc_autotune")
    return o


class Server:
    """Serving loop (vmc_server_*): resident meshes, admission by device-memory footprint,
    continuous batching of admitted requests."""

    def __init__(self, precision=VMC_FP32, max_slots=32, memory_budget=8 << 30, epoch_photons=0, device=0,
                 block_size=0, blocks_per_sm=0, use_graph=True, slicing=0, epoch_max_ms=0):
        cfg = VmcServerConfig(device, precision, max_slots, int(bool(use_graph)), memory_budget, epoch_photons,
                              block_size, blocks_per_sm, slicing, epoch_max_ms)
        h = C.c_void_p()
        s = lib().vmc_server_create(C.byref(cfg), C.byref(h))
        if s:
            raise VmcError(s, "vmc_server_create")
        self.h = h
        self.meshes = []
        self.pending = {}

    def add_mesh(self, mesh: Mesh):
        mid = C.c_int32()
        s = lib().vmc_server_add_mesh(self.h, mesh.h, C.byref(mid))
        if s:
            raise VmcError(s, "vmc_server_add_mesh")
        self.meshes.append(mesh)
        return mid.value

    def submit(self, mesh_id, p, nphoton=None, seed=None):
        m = _Marshal(p, geometry=False, nphoton=nphoton, seed=seed)
        rid = C.c_int64()
        s = lib().vmc_server_submit(self.h, mesh_id, C.byref(m.s), C.byref(rid))
        if s:
            raise VmcError(s, "vmc_server_submit")
        self.pending[rid.value] = (p.Ne, p.Nb, p.dim)
        return rid.value

    def _collect(self, rid, fn, *extra):
        Ne, Nb, dim = self.pending[rid]
        out, arr, _ = _outputs(Ne, Nb, dim, False)
        st = VmcStats()
        r = fn(self.h, rid, C.byref(out), C.byref(st), *extra)
        if r < 0:
            raise VmcError(-r, "vmc_server request")
        if r == 0:
            return None
        del self.pending[rid]
        return Result(arr["ER"], arr["EI"], arr["EBR"], arr["EBI"], arr["DEBR"], arr["DEBI"], None, stats_dict(st))

    def poll(self, rid):
        return self._collect(rid, lib().vmc_server_poll)

    def wait(self, rid, timeout_s=0.0):
        return self._collect(rid, lib().vmc_server_wait, timeout_s)

    def close(self):
        if self.h:
            lib().vmc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bench_gather(nbytes, seconds=0.3, device=0):
    v = C.c_double()
    s = lib().vmc_bench_gather(device, int(nbytes), seconds, C.byref(v))
    if s:
        raise VmcError(s, "vmc_bench_gather")
    return v.value


def bench_fp64(seconds=0.3, device=0):
    v = C.c_double()
    s = lib().vmc_bench_fp64(device, seconds, C.byref(v))
    if s:
        raise VmcError(s, "vmc_bench_fp64")
    return v.value
