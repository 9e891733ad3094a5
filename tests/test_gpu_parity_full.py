"""GPU parity at full size and on the batched and served paths, through the C ABI.

* The 648k-tet inclusion phantom, continuous wave and frequency domain, both arithmetic
  forms: per-element batch means against batch means of the oracle (the reference's
  algorithm with MT19937 on all host cores), and integrated quantities (absorbed fraction,
  total exitance, exitance through rings around the source and through the opposite
  face, absorption in the inclusion) against batches of the reference engine itself
  (tests/golden/phantom_scalars.npz, phantom_fd_scalars.npz).
* A multi-job launch of uneven pencil-beam cubes with their own optics (the batched
  workload scaled down), and requests that went through the serving loop (cosinic-disk
  and Gaussian-footprint sources at random top-face points), each against the oracle.
* The reference's own NetGen example mesh (21 597 triangles, the optics of
  examples/netgentest.m) on the GPU: same Philox streams as the oracle, and batch means.

Statistics (tests/parity_stats.py): per element, Welch t of the GPU's batch means
against the reference side's, gated against the same comparison with a second, independent
set of GPU batches of the reference side's size (the null); integrated quantities, z of the
batch means against the reference engine's batches, |z| < 4.
"""
import os

import numpy as np
import pytest

import oracle
import valomc_gb300 as V
from golden.make_phantom_scalars import functionals
from parity_stats import Batches, check_elements, element_report, fmt, scalar_z
from valomc_gb300 import meshgen as mg
from valomc_gb300 import meshio

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu
NCPU = os.cpu_count() or 1


# ---------------------------------------------------------------------------------------
# the full phantom: oracle batches shared by the tests of a session
# ---------------------------------------------------------------------------------------

B = 20
N_REF = 100_000


@pytest.fixture(scope="session")
def phantom_oracle(built):
    p = mg.config_3d_phantom(nphoton=1, seed=1)
    rows = []
    for b in range(B):
        r = oracle.run(p, rng=oracle.RNG_MT, nthreads=NCPU, nphoton=N_REF, seed=70000 + 1000 * b)
        rows.append(np.concatenate([r.ER, r.EBR]))
    return p, Batches(rows)


@pytest.fixture(scope="session")
def phantom_fd_oracle(built):
    p = mg.config_3d_fd(nphoton=1, seed=1)
    rows = []
    for b in range(B):
        r = oracle.run(p, rng=oracle.RNG_MT, nthreads=NCPU, nphoton=N_REF, seed=80000 + 1000 * b)
        rows.append(np.concatenate([r.ER, r.EI, r.EBR, r.EBI]))
    return p, Batches(rows)


def gpu_rows(p, precision, n, seeds, fd=False):
    mesh = V.Mesh(p, precision=precision)
    rows = []
    for s in seeds:
        res, _ = V.run_batch([mesh], [p.copy(Nphoton=n, seed=s)], precision=precision)
        r = res[0]
        rows.append(np.concatenate([r.ER, r.EI, r.EBR, r.EBI] if fd else [r.ER, r.EBR]))
    mesh.close()
    return rows


FORMS = [pytest.param(V.VMC_FP32, 1_000_000, id="fp32"), pytest.param(V.VMC_FP64, 200_000, id="fp64")]


@pytest.mark.parametrize("precision,n_gpu", FORMS)
def test_full_phantom_elements_within_batch_means_error(phantom_oracle, precision, n_gpu):
    p, ref = phantom_oracle
    gpu = Batches(gpu_rows(p, precision, n_gpu, [3000 + b for b in range(B)]))
    null = Batches(gpu_rows(p, precision, N_REF, [8000 + b for b in range(B)]))
    check_elements(f"full phantom {'fp32' if precision else 'fp64'} per element", element_report(gpu, ref, null),
                   min_well=50_000)


def test_full_phantom_fp32_at_the_plain_forms_batch_size(phantom_oracle):
    """The FP32 form with the FP64 form's batch size: the same Welch degrees of freedom, so
    the two forms' chi2/dof are directly comparable (with 5x larger batches than the
    oracle's, the oracle's skewed batch means dominate t and chi2/dof rises above the
    t-expectation, for either form)."""
    p, ref = phantom_oracle
    gpu = Batches(gpu_rows(p, V.VMC_FP32, 200_000, [5000 + b for b in range(B)]))
    null = Batches(gpu_rows(p, V.VMC_FP32, N_REF, [9000 + b for b in range(B)]))
    check_elements("full phantom fp32 (FP64 batch size) per element", element_report(gpu, ref, null), min_well=50_000)


@pytest.mark.parametrize("precision,n_gpu", FORMS)
def test_full_fd_phantom_elements_within_batch_means_error(phantom_fd_oracle, precision, n_gpu):
    p, ref = phantom_fd_oracle
    gpu = Batches(gpu_rows(p, precision, n_gpu, [4000 + b for b in range(B)], fd=True))
    null = Batches(gpu_rows(p, precision, N_REF, [10000 + b for b in range(B)], fd=True))
    check_elements(f"full FD phantom {'fp32' if precision else 'fp64'} per element", element_report(gpu, ref, null),
                   min_well=50_000)


def reference_scalars(name):
    path = os.path.join(GOLD, name)
    if not os.path.exists(path):
        pytest.skip(f"{name} not generated (tests/golden/make_phantom_scalars.py)")
    return np.load(path)


# FP32: 20 batches of 5e6 photons (1e8); FP64: 20 of 5e5 (its error is already below the
# reference's 2e7 photons)
SCALAR_FORMS = [pytest.param(V.VMC_FP32, 5_000_000, id="fp32"), pytest.param(V.VMC_FP64, 500_000, id="fp64")]


@pytest.mark.parametrize("precision,n_gpu", SCALAR_FORMS)
def test_full_phantom_integrated_quantities_match_the_reference(built, precision, n_gpu):
    ref = reference_scalars("phantom_scalars.npz")
    p = mg.config_3d_phantom(nphoton=1, seed=1)
    names, We, Wb = functionals(p)
    assert list(ref["names"]) == names
    mesh = V.Mesh(p, precision=precision)
    rows = []
    for b in range(B):
        res, _ = V.run_batch([mesh], [p.copy(Nphoton=n_gpu, seed=6000 + b)], precision=precision)
        rows.append(We @ res[0].ER + Wb @ res[0].EBR)
    z = scalar_z(f"full phantom {'fp32' if precision else 'fp64'}", names, rows, ref["real"])
    assert np.all(np.abs(z) < 4.0), dict(zip(names, z))


@pytest.mark.parametrize("precision,n_gpu", SCALAR_FORMS)
def test_full_fd_phantom_integrated_quantities_match_the_reference(built, precision, n_gpu):
    ref = reference_scalars("phantom_fd_scalars.npz")
    p = mg.config_3d_fd(nphoton=1, seed=1)
    names, We, Wb = functionals(p)
    assert list(ref["names"]) == names
    mesh = V.Mesh(p, precision=precision)
    re, im = [], []
    for b in range(B):
        res, _ = V.run_batch([mesh], [p.copy(Nphoton=n_gpu, seed=7000 + b)], precision=precision)
        r = res[0]
        re.append(We @ r.ER + Wb @ r.EBR)
        im.append(We @ r.EI + Wb @ r.EBI)
    label = f"full FD phantom {'fp32' if precision else 'fp64'}"
    z = np.concatenate([scalar_z(label + " real", names, re, ref["real"]), scalar_z(label + " imag", names, im, ref["imag"])])
    assert np.all(np.abs(z) < 4.0), z


# ---------------------------------------------------------------------------------------
# batched and served paths against the oracle
# ---------------------------------------------------------------------------------------

def oracle_batches(p, n, seed0, fd=False):
    rows = []
    for b in range(B):
        r = oracle.run(p, rng=oracle.RNG_MT, nthreads=NCPU, nphoton=n, seed=seed0 + 1000 * b)
        rows.append(np.concatenate([r.ER, r.EI, r.EBR, r.EBI] if fd else [r.ER, r.EBR]))
    return Batches(rows)


@pytest.mark.parametrize("precision", [V.VMC_FP32, V.VMC_FP64])
def test_multi_job_launch_of_uneven_cubes_matches_the_oracle(built, precision):
    """Eight cubes (8-16 mm edges, 3k-25k tets) with their own optics and pencil beams at
    random top-face points: B batches of each, and B null batches of the oracle's size, of
    all of them in ONE persistent launch (320 jobs), each instance against B oracle
    batches."""
    probs = mg.config_batch(count=8, gen_seed=41, lmin=8, lmax=16, pmin=1, pmax=1)
    meshes = [V.Mesh(p, precision=precision) for p in probs]
    n_gpu = 100_000 if precision == V.VMC_FP32 else 20_000
    n_ref = 20_000
    jobs, ms = [], []
    for k, p in enumerate(probs):
        for b in range(B):
            jobs.append(p.copy(Nphoton=n_gpu, seed=100 * k + b + 1))
            ms.append(meshes[k])
        for b in range(B):
            jobs.append(p.copy(Nphoton=n_ref, seed=100 * k + b + 51))
            ms.append(meshes[k])
    res, tot = V.run_batch(ms, jobs, precision=precision)
    assert tot["photons_done"] == sum(j.Nphoton for j in jobs)
    for k, p in enumerate(probs):
        rows = [np.concatenate([r.ER, r.EBR]) for r in res[2 * B * k: 2 * B * (k + 1)]]
        gpu, null = Batches(rows[:B]), Batches(rows[B:])
        ref = oracle_batches(p, n_ref, 9000 + 7 * k)
        check_elements(f"multi-job instance {k} (L {int(round(p.r[:, 0].max()))} mm, mua {p.mua[0]:.3f}, "
                       f"mus {p.mus[0]:.1f}, g {p.g[0]:.2f}) {'fp32' if precision else 'fp64'}",
                       element_report(gpu, ref, null), min_well=200)


def test_served_requests_match_the_oracle(built):
    """Requests of the serving workload (cosinic-disk and Gaussian-footprint sources at
    random top-face points, random optics) on small resident cubes: B copies of each with
    distinct seeds, and B null copies of the oracle's size, all submitted at once so they
    share the device, each request's batch means against the oracle's."""
    mix = mg.ServingMix(seed=55, meshes=3, tmin=3_000, tmax=12_000, pmin=50_000, pmax=50_000)
    meshes = [V.Mesh(b) for b in mix.base]
    srv = V.Server(max_slots=64, memory_budget=2 << 30)
    ids = [srv.add_mesh(m) for m in meshes]
    specs = [mix.request() for _ in range(4)]
    n_ref = 10_000
    rids = [[srv.submit(ids[k], p, seed=200 * i + b + 1) for b in range(B)] +
            [srv.submit(ids[k], p, nphoton=n_ref, seed=200 * i + b + 101) for b in range(B)]
            for i, (k, p) in enumerate(specs)]
    for i, (k, p) in enumerate(specs):
        res = [srv.wait(r, timeout_s=300) for r in rids[i]]
        rows = [np.concatenate([r.ER, r.EBR]) for r in res]
        gpu, null = Batches(rows[:B]), Batches(rows[B:])
        ref = oracle_batches(p, n_ref, 11000 + 13 * i)
        src = "cosinic disk" if (p.BCType == ord("c")).any() else "gaussian footprint"
        check_elements(f"served request {i} ({src}, mesh {k}, {p.Ne} tets)", element_report(gpu, ref, null),
                       min_well=200)
    srv.close()


# ---------------------------------------------------------------------------------------
# the reference's NetGen example mesh
# ---------------------------------------------------------------------------------------

REF_VOL = oracle.reference_file("examples/square_with_two_circles.vol")


def netgen_example_problem(nphoton, seed=2024):
    """examples/netgentest.m on importNetGenMesh.m's mesh: background mua 0.01, mus 1.3,
    g 0.9, n 1.3; circles mua 0.09, mus 1.3, g 0.5, n 1.5; cosinic light source on the
    'lightsource' boundary; the exterior index of each boundary row is its element's."""
    m = meshio.read_vol(REF_VOL, preserve_boundary=False)
    ne, nb = len(m.H), len(m.BH)
    bg, ci = m.regions[1], m.regions[2]
    mua, mus, g, n = np.zeros(ne), np.zeros(ne), np.zeros(ne), np.zeros(ne)
    mua[bg], mus[bg], g[bg], n[bg] = 0.01, 1.3, 0.9, 1.3
    mua[ci], mus[ci], g[ci], n[ci] = 0.09, 1.3, 0.5, 1.5
    types = np.full(nb, ord("a"), np.uint8)
    types[m.boundaries[2]] = ord("c")
    bcn = n[meshio.boundary_mothers(m.H, m.BH)]
    return mg.Problem(dim=2, H=m.H, BH=m.BH, r=m.r, mua=mua, mus=mus, g=g, n=n, BCType=types, BCn=bcn,
                      Nphoton=nphoton, seed=seed)


needs_vol = pytest.mark.skipif(REF_VOL is None, reason="the reference's example mesh is not staged")


@needs_vol
def test_netgen_example_fp64_matches_the_oracle_on_the_same_philox_streams(built):
    p = netgen_example_problem(20000)
    gpu = V.run(p, precision=V.VMC_FP64, seed=4242)
    ref = oracle.run(p, rng=oracle.RNG_PHILOX, nthreads=NCPU, seed=4242)
    assert ref.status == 0 and gpu.stats["photons_done"] == p.Nphoton
    worst = 0.0
    for k in ("ER", "EBR", "DEBR"):
        a, b = getattr(gpu, k), getattr(ref, k)
        d = np.abs(a - b).sum() / np.abs(b).sum()
        worst = max(worst, d)
        assert d < 1e-6, (k, d)
    print(f"NetGen example, same Philox streams: worst L1 relative difference {worst:.2e}, "
          f"steps {gpu.stats['steps']} / {ref.steps}")
    assert gpu.stats["steps"] == ref.steps and gpu.stats["scatters"] == ref.scatters


@needs_vol
@pytest.mark.parametrize("precision", [V.VMC_FP32, V.VMC_FP64])
def test_netgen_example_within_batch_means_error_of_the_oracle(built, precision):
    p = netgen_example_problem(1)
    def gpu(n, seed0):
        return Batches([np.concatenate([r.ER, r.EBR, r.DEBR]) for r in
                        (V.run(p, precision=precision, nphoton=n, seed=seed0 + b) for b in range(B))])
    ref_rows = []
    for b in range(B):
        r = oracle.run(p, rng=oracle.RNG_MT, nthreads=NCPU, nphoton=20_000, seed=12000 + 1000 * b)
        ref_rows.append(np.concatenate([r.ER, r.EBR, r.DEBR]))
    check_elements(f"NetGen example {'fp32' if precision else 'fp64'}",
                   element_report(gpu(200_000, 300), Batches(ref_rows), gpu(20_000, 600)), min_well=1000)
