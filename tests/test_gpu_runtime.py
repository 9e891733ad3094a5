"""Batched launches, the serving loop, cancellation / timeout, progress, and the drop-in
executables, on the GPU through the C ABI."""
import os
import subprocess
import tempfile
import threading
import time

import numpy as np
import pytest

import valomc_gb300 as V
from golden.make_golden import cases
from valomc_gb300 import build as vbuild
from valomc_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu
RTOL = 1e-9  # same photons, same draws: only the order of the FP64 atomic additions differs


def small_jobs():
    c = cases()
    jobs = [c["phantom3d"][0].copy(Nphoton=30000, seed=21), c["pencil3d"][0].copy(Nphoton=20000, seed=22),
            mg.pencil_box(10, 0.03, 8.0, 0.9, 1.37, (4.3, 5.2), 25000, seed=23),
            mg.pencil_box(14, 0.08, 15.0, 0.85, 1.41, (6.6, 2.3), 15000, seed=24)]
    return jobs


@pytest.mark.parametrize("precision", [V.VMC_FP64, V.VMC_FP32])
def test_batch_equals_individual_runs(built, precision):
    jobs = small_jobs()
    meshes = [V.Mesh(p, precision=precision) for p in jobs]
    res, tot = V.run_batch(meshes, jobs, precision=precision)
    assert tot["photons_done"] == sum(p.Nphoton for p in jobs)
    for p, r in zip(jobs, res):
        one = V.run(p, precision=precision)
        np.testing.assert_allclose(r.ER, one.ER, rtol=RTOL, atol=1e-300)
        np.testing.assert_allclose(r.EBR, one.EBR, rtol=RTOL, atol=1e-300)
        assert r.stats["steps"] == one.stats["steps"] > 0  # per-job step counts
    assert sum(r.stats["steps"] for r in res) == tot["steps"]


@pytest.mark.parametrize("use_graph", [False, True])
def test_calls_from_two_threads_overlap_and_equal_sequential_runs(built, use_graph):
    # each call runs on a stream of its own; ctypes drops the GIL for the call
    jobs = small_jobs()[:2]
    opts = V.options(use_graph=use_graph)
    seq = [V.run(p, precision=V.VMC_FP32, opts=opts) for p in jobs]
    out = [None, None]
    errs = []

    def work(i):
        try:
            out[i] = [V.run(jobs[i], precision=V.VMC_FP32, opts=opts) for _ in range(3)]
        except Exception as e:  # noqa: BLE001 -- reported below
            errs.append(e)

    th = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join(timeout=300)
    assert not errs and all(o is not None for o in out)
    for i in range(2):
        for r in out[i]:
            np.testing.assert_allclose(r.ER, seq[i].ER, rtol=RTOL, atol=1e-300)
            np.testing.assert_allclose(r.DEBR, seq[i].DEBR, rtol=RTOL, atol=1e-300)
            assert r.stats["steps"] == seq[i].stats["steps"]


@pytest.mark.parametrize("precision", [V.VMC_FP64, V.VMC_FP32])
def test_zero_photon_jobs(built, precision):
    """An empty run launches nothing and normalises to NaN as the reference does; an empty
    job inside a batch leaves the others as they are alone."""
    p = cases()["square2d"][0]
    r = V.run(p, precision=precision, nphoton=0)
    assert r.stats["photons_done"] == 0 and r.stats["steps"] == 0
    assert np.isnan(r.ER).all() and np.isnan(r.EBR).all()
    raw = V.run(p, precision=precision, nphoton=0, normalize=False)
    assert not raw.ER.any() and not raw.EBR.any()
    # a negative count runs no photon and divides by itself, as MonteCarlo does: -0.0
    neg = V.run(p, precision=precision, nphoton=-5)
    assert neg.stats["photons_done"] == 0 and not neg.ER.any() and np.signbit(neg.ER).all()
    jobs = small_jobs()[:2]
    jobs = [jobs[0].copy(Nphoton=0), jobs[1]]
    meshes = [V.Mesh(q, precision=precision) for q in jobs]
    res, tot = V.run_batch(meshes, jobs, precision=precision)
    assert tot["photons_done"] == jobs[1].Nphoton
    assert np.isnan(res[0].ER).all()
    one = V.run(jobs[1], precision=precision)
    np.testing.assert_allclose(res[1].ER, one.ER, rtol=RTOL, atol=1e-300)


def test_batch_through_a_cuda_graph_equals_the_plain_launch(built):
    jobs = small_jobs()
    meshes = [V.Mesh(p) for p in jobs]
    plain, _ = V.run_batch(meshes, jobs)
    for _ in range(2):  # the second launch updates the instantiated graph in place
        g, tot = V.run_batch(meshes, jobs, opts=V.options(use_graph=True))
        assert tot["photons_done"] == sum(p.Nphoton for p in jobs)
        for a, b in zip(plain, g):
            np.testing.assert_allclose(b.ER, a.ER, rtol=RTOL, atol=1e-300)


def staging_case(name):
    if name == "box5":  # 750 tets, 300 boundary triangles: the whole set fits a CTA's stage
        return mg.pencil_box(5, 0.05, 6.0, 0.9, 1.4, (2.2, 2.9), 50000, seed=31)
    return cases()[name][0].copy(Nphoton=50000, seed=31)


@pytest.mark.parametrize("precision", [V.VMC_FP64, V.VMC_FP32])
@pytest.mark.parametrize("slots", [64, 2048, 0])
@pytest.mark.parametrize("name", ["phantom3d", "box5", "square2d", "mixed2d_fd"])
def test_shared_memory_staging_equals_global_atomics(built, slots, name, precision):
    # slots > 0: hashed element table (3D FP32 continuous wave); 0: the whole accumulator set
    # of a small mesh; -1: global reductions only
    if precision == V.VMC_FP64 and slots != 0:
        pytest.skip("the hashed table is a tracking-form option")
    p = staging_case(name)
    mesh = V.Mesh(p, precision=precision)
    o = dict(precision=precision)
    plain, _ = V.run_batch([mesh], [p], opts=V.options(stage_slots=-1, **o))
    staged, _ = V.run_batch([mesh], [p], opts=V.options(stage_slots=slots, **o))
    for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI"):
        np.testing.assert_allclose(getattr(staged[0], k), getattr(plain[0], k), rtol=RTOL, atol=1e-300, err_msg=k)
    assert staged[0].stats["steps"] == plain[0].stats["steps"]


@pytest.mark.parametrize("name", ["square2d", "phantom3d"])
def test_refill_threshold_leaves_results_unchanged(built, name):
    # a photon's draws depend on its index only, so launching idle lanes one at a time or in
    # groups changes nothing but the order of the FP64 additions
    p = cases()[name][0].copy(Nphoton=40000, seed=41)
    ref = V.run(p, opts=V.options(refill_lanes=1))
    for k in (4, 32):
        r = V.run(p, opts=V.options(refill_lanes=k))
        np.testing.assert_allclose(r.ER, ref.ER, rtol=RTOL, atol=1e-300)
        np.testing.assert_allclose(r.EBR, ref.EBR, rtol=RTOL, atol=1e-300)
        assert r.stats["steps"] == ref.stats["steps"] and r.stats["photons_done"] == p.Nphoton


def test_autotuner_returns_a_valid_shape(built):
    jobs = small_jobs()
    meshes = [V.Mesh(p) for p in jobs]
    o = V.autotune(meshes, jobs, budget_s=1.0)
    assert o.block_size in (64, 128, 256) and o.fetch_chunk in (32, 64, 128)
    res, _ = V.run_batch(meshes, jobs, opts=o)
    assert all(r.ER.sum() > 0 for r in res)


@pytest.mark.parametrize("precision", [V.VMC_FP64, V.VMC_FP32])
def test_server_result_alone_equals_result_in_the_mix(built, precision):
    jobs = small_jobs()
    meshes = [V.Mesh(p, precision=precision) for p in jobs]
    # alone: one request at a time, small epochs so requests are sliced across launches
    srv = V.Server(precision=precision, max_slots=8, memory_budget=1 << 30, epoch_photons=7000)
    ids = [srv.add_mesh(m) for m in meshes]
    alone = []
    for k, p in enumerate(jobs):
        rid = srv.submit(ids[k], p)
        alone.append(srv.wait(rid))
    # mixed: everything in flight together, submitted while others run
    rids = [srv.submit(ids[k], p) for k, p in enumerate(jobs)]
    mixed = [srv.wait(r) for r in rids]
    srv.close()
    for p, a, m in zip(jobs, alone, mixed):
        one = V.run(p, precision=precision)
        np.testing.assert_allclose(a.ER, m.ER, rtol=RTOL, atol=1e-300)
        np.testing.assert_allclose(a.ER, one.ER, rtol=RTOL, atol=1e-300)
        np.testing.assert_allclose(m.EBR, one.EBR, rtol=RTOL, atol=1e-300)
        assert m.stats["photons_done"] == p.Nphoton
        assert a.stats["steps"] == m.stats["steps"] == one.stats["steps"]


def test_server_default_epochs_keep_each_result(built):
    """Epochs sized by the backlog and water-filled slices (the server's defaults): requests
    of very different sizes submitted together each equal their run alone."""
    jobs = small_jobs()
    sizes = [400, 60000, 3000, 25000]
    meshes = [V.Mesh(p) for p in jobs]
    srv = V.Server(max_slots=8, memory_budget=1 << 30)
    ids = [srv.add_mesh(m) for m in meshes]
    rids = [srv.submit(ids[k], p, nphoton=n) for k, (p, n) in enumerate(zip(jobs, sizes))]
    res = [srv.wait(r, timeout_s=120) for r in rids]
    srv.close()
    for p, n, r in zip(jobs, sizes, res):
        one = V.run(p, nphoton=n)
        assert r.stats["photons_done"] == n and r.stats["steps"] == one.stats["steps"]
        np.testing.assert_allclose(r.ER, one.ER, rtol=RTOL, atol=1e-300)
        np.testing.assert_allclose(r.EBR, one.EBR, rtol=RTOL, atol=1e-300)


def test_server_admission_by_memory_footprint(built):
    p = cases()["phantom3d"][0]
    mesh = V.Mesh(p)
    srv = V.Server(max_slots=4, memory_budget=200_000)  # smaller than one request's state
    mid = srv.add_mesh(mesh)
    rid = srv.submit(mid, p, nphoton=1000)
    with pytest.raises(V.VmcError) as e:
        srv.wait(rid, timeout_s=30)
    assert e.value.status == 39  # VMC_ERR_ADMISSION
    srv.close()


def test_server_releases_memory_of_finished_requests(built):
    """A budget that holds one request at a time: every request is admitted in turn, so the
    memory of finished requests (returned to the server's pool) is accounted back."""
    p = cases()["phantom3d"][0]
    mesh = V.Mesh(p)
    one = V.run(p, nphoton=3000, seed=5)
    srv = V.Server(max_slots=4, memory_budget=900_000)  # one request's state (~0.6 MB) fits, two do not
    mid = srv.add_mesh(mesh)
    rids = [srv.submit(mid, p, nphoton=3000, seed=5) for _ in range(6)]
    res = [srv.wait(r, timeout_s=120) for r in rids]
    srv.close()
    for r in res:
        assert r is not None and r.stats["photons_done"] == 3000
        np.testing.assert_allclose(r.ER, one.ER, rtol=RTOL, atol=1e-300)


def test_server_poll_before_finish(built):
    p = mg.config_3d_phantom(nphoton=1, seed=2)
    mesh = V.Mesh(p)
    srv = V.Server(max_slots=4, memory_budget=1 << 30)
    mid = srv.add_mesh(mesh)
    rid = srv.submit(mid, p, nphoton=5_000_000)
    assert srv.poll(rid) is None
    r = srv.wait(rid, timeout_s=120)
    assert r is not None and r.stats["photons_done"] == 5_000_000
    assert r.stats["seconds_total"] >= r.stats["seconds_kernel"] > 0
    srv.close()


def test_timeout_stops_the_kernel_and_the_context_stays_usable(built):
    p = mg.config_3d_phantom(nphoton=2_000_000_000, seed=3)
    t0 = time.time()
    r = V.run(p, check=False, timeout_s=0.5)
    assert r.stats["status"] == 37  # VMC_ERR_TIMEOUT
    assert time.time() - t0 < 30
    assert 0 < r.stats["photons_done"] < p.Nphoton
    ok = V.run(cases()["phantom3d"][0], nphoton=1000)
    assert ok.stats["photons_done"] == 1000


def test_cancel_flag_and_progress_callback(built):
    p = mg.config_3d_phantom(nphoton=2_000_000_000, seed=4)
    flag = np.zeros(1, np.int32)
    threading.Timer(0.4, lambda: flag.__setitem__(0, 1)).start()
    r = V.run(p, check=False, cancel=flag)
    assert r.stats["status"] == 36  # VMC_ERR_CANCELLED
    seen = []

    def prog(pct):
        seen.append(pct)
        return len(seen) < 3  # abort at the third report, like the MEX waitbar's cancel

    r = V.run(p, check=False, progress=prog)
    assert r.stats["status"] == 36 and len(seen) == 3
    assert all(0 <= s <= 100 for s in seen)


@pytest.mark.parametrize("dim", [3, 2])
def test_executable_writes_the_reference_format(built, dim):
    p = cases()["phantom3d" if dim == 3 else "square2d"][0].copy(Nphoton=20000, seed=77)
    exe = os.path.join(vbuild.BUILD, f"MC{dim}D")
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
        mg.write_input(fin, p)
        res = subprocess.run([exe, fin, fout] + (["-s"] if dim == 2 else []), capture_output=True, text=True,
                             timeout=300)
        assert res.returncode == 0, res.stdout + res.stderr
        assert "Computation took" in res.stdout
        lines = open(fout).read().splitlines()
    assert len(lines) == 1 + p.Ne + p.Nb
    assert lines[0].endswith(" 0")
    if dim == 3:
        assert len(lines[1]) == 37  # "%18.10e %18.10e"
    vals = np.array([[float(x) for x in ln.split()] for ln in lines[1:]])
    one = V.run(p)
    rt = 1e-9 if dim == 3 else 1e-5
    np.testing.assert_allclose(vals[:p.Ne, 0], one.ER, rtol=rt, atol=1e-300)
    np.testing.assert_allclose(vals[p.Ne:, 0], one.EBR, rtol=rt, atol=1e-300)
