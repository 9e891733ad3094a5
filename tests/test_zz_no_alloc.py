"""vmc_run_noalloc: the photon run for callers that cannot let a library allocate device
memory (their device memory is owned by their own allocator -- here PyTorch's caching
allocator stands in for it -- so a library-side cudaMalloc would synchronise the device
and take memory outside their accounting).  The caller hands in device buffers it owns;
the kernel's scratch lives in the library's fixed-size static device array.

Checked through the C ABI against the existing entry point on two calls in a row, so the
second call also shows that the shared scratch is cleared between calls.  The existing call
is vmc_run_batch on the same resident mesh, job and seed, batched with a second job of no
photons: a batch of more than one job runs the per-job form of the pool kernel, the form
this entry point launches, so both walk the same photons with the same instructions and
differ only in the order of the FP64 atomic additions (the one-job form that a lone FP32
job runs is compiled separately, and its FP32 rounding may differ in the last bit).
Kept in a file of its own, collected last."""
import ctypes as C

import numpy as np
import pytest

import valomc_gb300 as V
from golden.make_golden import cases
from valomc_gb300 import api

pytestmark = pytest.mark.gpu
RTOL = 1e-9  # same photons and draws; only the order of the FP64 atomic additions differs


def noalloc_run(mesh, p, bufs, precision=V.VMC_FP32, **kw):
    m = api._Marshal(p, geometry=False)
    o = V.options(precision=precision, **kw)
    out, arr, _ = api._outputs(p.Ne, p.Nb, p.dim, False)
    st = api.VmcStats()
    s = V.lib().vmc_run_noalloc(mesh.h, C.byref(m.s), C.byref(o), C.byref(bufs), C.byref(out), C.byref(st))
    return s, arr, api.stats_dict(st)


def caller_buffers(torch, p, precision):
    """Device buffers the caller owns (PyTorch's allocator), the accumulators holding stale
    contents from an earlier use."""
    dev = torch.device("cuda", 0)
    keep = [torch.empty(p.Ne * 4, dtype=torch.float32 if precision == V.VMC_FP32 else torch.float64, device=dev),
            torch.empty(p.Nb, dtype=torch.uint8, device=dev),
            torch.empty(p.Nb, dtype=torch.float64, device=dev),
            torch.full((2 * p.Ne + 4 * p.Nb,), 7.0, dtype=torch.float64, device=dev)]
    torch.cuda.synchronize()
    return keep, api.VmcNoallocBuffers(*(t.data_ptr() for t in keep))


# tetrahedra in continuous wave and in the frequency domain, triangles; both arithmetic forms
@pytest.mark.parametrize("precision", [V.VMC_FP32, V.VMC_FP64])
@pytest.mark.parametrize("name", ["phantom3d", "phantom3d_fd", "mixed2d"])
def test_noalloc_matches_the_allocating_entry_point_twice(built, name, precision):
    torch = pytest.importorskip("torch")
    p = cases()[name][0].copy(Nphoton=40000 if precision == V.VMC_FP32 else 10000, seed=2718)
    mesh = V.Mesh(p, precision=precision)
    want, _ = V.run_batch([mesh, mesh], [p, p.copy(Nphoton=0)], precision=precision)
    want = want[0]
    keep, bufs = caller_buffers(torch, p, precision)
    for call in range(2):
        s, got, st = noalloc_run(mesh, p, bufs, precision)
        assert s == 0, (call, s, V.lib().vmc_last_error())
        assert st["photons_done"] == p.Nphoton
        for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI"):
            np.testing.assert_allclose(got[k], getattr(want, k), rtol=RTOL, atol=1e-300, err_msg=f"call {call} {k}")


def test_noalloc_refuses_host_buffers_and_polling_options(built):
    """A host pointer among the buffers, or a cancel flag / timeout it would not poll, is
    refused before anything is launched."""
    torch = pytest.importorskip("torch")
    p = cases()["phantom3d"][0].copy(Nphoton=1000, seed=1)
    mesh = V.Mesh(p, precision=V.VMC_FP32)
    keep, bufs = caller_buffers(torch, p, V.VMC_FP32)
    host_acc = np.zeros(2 * p.Ne + 4 * p.Nb)
    bad = api.VmcNoallocBuffers(bufs.optics, bufs.bctype, bufs.bcn, host_acc.ctypes.data)
    s, _, _ = noalloc_run(mesh, p, bad)
    assert s == 32 and b"acc must be device memory" in V.lib().vmc_last_error()
    s, _, _ = noalloc_run(mesh, p, bufs, timeout_s=5.0)
    assert s == 32 and b"does not poll" in V.lib().vmc_last_error()
    s, _, st = noalloc_run(mesh, p, bufs)
    assert s == 0 and st["photons_done"] == p.Nphoton


def test_noalloc_refuses_more_faces_than_its_scratch_holds(built):
    p = cases()["phantom3d"][0].copy()
    p.BCType[:] = ord("l")  # every boundary triangle emits: more faces than the scratch holds
    assert p.Nb > 512
    mesh = V.Mesh(p, precision=V.VMC_FP32)
    bufs = api.VmcNoallocBuffers(1, 1, 1, 1)  # never touched: the size check comes first
    s, _, _ = noalloc_run(mesh, p.copy(Nphoton=10), bufs)
    assert s == 41  # VMC_ERR_SIZE_LIMIT
    assert b"at most 512" in V.lib().vmc_last_error()
