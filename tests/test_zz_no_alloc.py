"""vmc_run_noalloc: the photon run for callers that cannot let a library allocate device
memory (their device memory is owned by their own allocator -- here PyTorch's caching
allocator stands in for it -- so a library-side cudaMalloc would synchronise the device
and take memory outside their accounting).  The caller hands in device buffers it owns;
the kernel's scratch lives in the library's fixed-size static device array.

Checked through the C ABI against the existing entry point (vmc_run_batch on the same
resident mesh, job and seed) on two calls in a row, so the second call also shows that the
shared scratch is cleared between calls.  Kept in a file of its own, collected last."""
import ctypes as C

import numpy as np
import pytest

import valomc_gb300 as V
from golden.make_golden import cases
from valomc_gb300 import api

pytestmark = pytest.mark.gpu
RTOL = 1e-9  # same photons and draws; only the order of the FP64 atomic additions differs


def noalloc_run(mesh, p, bufs):
    m = api._Marshal(p, geometry=False)
    o = V.options(precision=V.VMC_FP32)
    out, arr, _ = api._outputs(p.Ne, p.Nb, p.dim, False)
    st = api.VmcStats()
    s = V.lib().vmc_run_noalloc(mesh.h, C.byref(m.s), C.byref(o), C.byref(bufs), C.byref(out), C.byref(st))
    return s, arr, api.stats_dict(st)


def test_noalloc_matches_the_allocating_entry_point_twice(built):
    torch = pytest.importorskip("torch")
    p = cases()["phantom3d"][0].copy(Nphoton=40000, seed=2718)
    mesh = V.Mesh(p, precision=V.VMC_FP32)
    want, _ = V.run_batch([mesh], [p], precision=V.VMC_FP32)
    want = want[0]
    # the caller's own device memory
    dev = torch.device("cuda", 0)
    optics = torch.empty(p.Ne * 4, dtype=torch.float32, device=dev)
    bctype = torch.empty(p.Nb, dtype=torch.uint8, device=dev)
    bcn = torch.empty(p.Nb, dtype=torch.float64, device=dev)
    acc = torch.full((2 * p.Ne + 4 * p.Nb,), 7.0, dtype=torch.float64, device=dev)  # stale contents
    torch.cuda.synchronize()
    bufs = api.VmcNoallocBuffers(optics.data_ptr(), bctype.data_ptr(), bcn.data_ptr(), acc.data_ptr())
    for call in range(2):
        s, got, st = noalloc_run(mesh, p, bufs)
        assert s == 0, (call, s, V.lib().vmc_last_error())
        assert st["photons_done"] == p.Nphoton
        for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI"):
            np.testing.assert_allclose(got[k], getattr(want, k), rtol=RTOL, atol=1e-300, err_msg=f"call {call} {k}")


def test_noalloc_refuses_more_faces_than_its_scratch_holds(built):
    p = cases()["phantom3d"][0].copy()
    p.BCType[:] = ord("l")  # every boundary triangle emits: more faces than the scratch holds
    assert p.Nb > 512
    mesh = V.Mesh(p, precision=V.VMC_FP32)
    bufs = api.VmcNoallocBuffers(1, 1, 1, 1)  # never touched: the size check comes first
    s, _, _ = noalloc_run(mesh, p.copy(Nphoton=10), bufs)
    assert s == 41  # VMC_ERR_SIZE_LIMIT
    assert b"at most 512" in V.lib().vmc_last_error()
