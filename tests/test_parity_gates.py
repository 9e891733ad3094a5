"""The statistical gates of the GPU parity tests (tests/parity_stats.py), checked on the CPU
against known answers.  The oracle stands in for both sides: 20 Philox batches play the GPU
form, 20 MT19937 batches the reference, and 20 further Philox batches of the reference's
size the null comparison.  An exact match must pass every gate; a physics error planted in
the oracle's input (on the CPU) must fail one:

* a phase function changed from g = 0.90 to 0.89 reshapes the fluence: the per-element
  gates (within 3 sigma, chi2/dof against its null) fail;
* an absorption coefficient 5% too high lowers every element by about the same fraction.
  On the 200 strongly correlated elements of the 2D square, 20 batches do not resolve that
  per element (the mean signed t moves by about two of its jackknife errors), which is why
  the GPU tests also gate integrated quantities: the absorbed fraction moves by many of its
  standard errors.
"""
import numpy as np
import pytest

import oracle
from parity_stats import Batches, chi2_excess_ok, element_report, fmt, mean_t_ok, scalar_z, within3_ok
from valomc_gb300 import meshgen as mg

B = 20
N_GPU, N_REF = 100_000, 20_000


def _runs(p, rng, n, seeds):
    out = []
    for s in seeds:
        r = oracle.run(p.copy(Nphoton=n, seed=s), rng=rng, nthreads=4)
        assert r.status == 0
        out.append(r)
    return out


def _element_gates(rep):
    h, w = rep["hit"], rep["well"]
    return (within3_ok(h, 0.985) and chi2_excess_ok(h) and w["n"] >= 100 and within3_ok(w, 0.99)
            and chi2_excess_ok(w) and mean_t_ok(w))


@pytest.fixture(scope="module")
def square():
    return mg.config_2d_square(nphoton=1, seed=1)


@pytest.fixture(scope="module")
def reference_side(built, square):
    return _runs(square, oracle.RNG_MT, N_REF, [1000 * b + 7 for b in range(B)])


def _gpu_side(p):
    return (_runs(p, oracle.RNG_PHILOX, N_GPU, [50_000 + 1000 * b for b in range(B)]),
            _runs(p, oracle.RNG_PHILOX, N_REF, [90_000 + 1000 * b for b in range(B)]))


def _verdicts(label, gpu, null, ref):
    rep = element_report(Batches([r.ER for r in gpu]), Batches([r.ER for r in ref]), Batches([r.ER for r in null]))
    print(fmt(label, rep))
    names = ("absorbed", "exited")
    z = scalar_z(label, names, [[r.ledger[k] / N_GPU for k in names] for r in gpu],
                 [[r.ledger[k] / N_REF for k in names] for r in ref])
    return _element_gates(rep), bool(np.all(np.abs(z) < 4.0))


def test_gates_pass_an_exact_match(square, reference_side):
    gpu, null = _gpu_side(square)
    elements_ok, scalars_ok = _verdicts("exact", gpu, null, reference_side)
    assert elements_ok and scalars_ok


def test_element_gates_catch_a_changed_phase_function(square, reference_side):
    gpu, null = _gpu_side(square.copy(g=np.full_like(square.g, 0.89)))
    elements_ok, _ = _verdicts("g 0.89", gpu, null, reference_side)
    assert not elements_ok


def test_integrated_gate_catches_a_uniform_absorption_offset(square, reference_side):
    gpu, null = _gpu_side(square.copy(mua=square.mua * 1.05))
    _, scalars_ok = _verdicts("mua x 1.05", gpu, null, reference_side)
    assert not scalars_ok


def test_bench_error_to_noise_reads_one_for_a_match_and_more_for_an_error(square, reference_side):
    """bench.py's matched-error figure (error-to-noise: sqrt of chi2/dof against the oracle
    over chi2/dof against independent batches of the oracle's size) on the same known
    answers: near 1 for the exact match, well above the 1.1 target for the planted phase
    function error."""
    import bench
    ref = [r.ER for r in reference_side]
    gpu, null = _gpu_side(square)
    exact = bench.welch_error_to_noise([r.ER for r in gpu], ref, [r.ER for r in null])
    gpu_bad, null_bad = _gpu_side(square.copy(g=np.full_like(square.g, 0.89)))
    bad = bench.welch_error_to_noise([r.ER for r in gpu_bad], ref, [r.ER for r in null_bad])
    print("error-to-noise: exact", exact, "g 0.89", bad)
    assert exact["elements"] >= 100 and bad["elements"] >= 100
    assert 0.7 < exact["error_to_noise"] < 1.1
    assert bad["error_to_noise"] > 1.5
