"""Pins the CPU oracle (oracle/vmc_oracle.c) to the reference engine: its MT19937 runs must
equal the reference's MonteCarlo() output bit for bit, and its tape replays must visit the
same elements, on every golden fixture (made by tests/golden/make_golden.py from the
reference itself)."""
import os

import numpy as np
import pytest

import oracle
from golden.make_golden import TRACE_CASES, cases, tape_for

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_reference_run(built, name):
    p, nthr = CASES[name]
    g = np.load(os.path.join(GOLD, f"run_{name}.npz"))
    assert int(g["threads"]) == nthr
    o = oracle.run(p, rng=oracle.RNG_MT, nthreads=nthr)
    assert o.status == 0
    assert o.loss == int(g["loss"])
    for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI"):
        np.testing.assert_array_equal(getattr(o, k), g[k], err_msg=f"{name}:{k}")


@pytest.mark.parametrize("name", TRACE_CASES)
def test_oracle_replays_reference_trajectories(built, name):
    p = CASES[name][0]
    g = np.load(os.path.join(GOLD, f"trace_{name}.npz"))
    tape, off = tape_for(name)
    n = len(g["lens"])
    o = oracle.run(p, rng=oracle.RNG_TAPE, nphoton=n, tape=tape, tape_off=off, trace_photons=n, normalize=False)
    ev = np.split(g["events"], np.cumsum(g["lens"])[:-1])
    for i in range(n):
        np.testing.assert_array_equal(o.traces[i], ev[i], err_msg=f"{name} photon {i}")
    for k in ("ER", "EI", "EBR", "EBI", "DEBR"):
        np.testing.assert_array_equal(getattr(o, k), g[k], err_msg=f"{name}:{k}")


def test_oracle_energy_closure(built):
    """absorbed + exited (+ roulette and loss ledgers) == launched, CW, to rounding."""
    p = CASES["phantom3d"][0]
    o = oracle.run(p, rng=oracle.RNG_MT, nthreads=2, normalize=False)
    L = o.ledger
    lhs = L["launched"] + L["roulette_gain"] - L["roulette_kill"] - L["lost"]
    assert abs(L["absorbed"] + L["exited"] - lhs) / L["launched"] < 1e-12
    assert abs(o.ER.sum() - L["absorbed"]) / L["absorbed"] < 1e-12


def test_reference_binaries_match_fixtures_when_present(built):
    """Where the reference tree is available, re-run it and compare with the fixture."""
    if not oracle.have_reference_binaries():
        pytest.skip("reference harness not built on this host")
    p, nthr = CASES["square2d"]
    out = oracle.ref_run(p, nthreads=nthr)
    g = np.load(os.path.join(GOLD, "run_square2d.npz"))
    np.testing.assert_array_equal(out["ER"], g["ER"])


@pytest.mark.parametrize("name", ["square2d", "phantom3d"])
def test_zero_photons_normalise_to_nan_as_the_reference(built, name):
    """An empty run: MonteCarlo divides the zero sums by N = 0 (MC3D.hpp:1792-1818), so every
    normalised output is NaN; unnormalised they are zero.  Checked against the reference
    binaries where they are built."""
    p = CASES[name][0].copy(Nphoton=0)
    o = oracle.run(p, rng=oracle.RNG_MT, nthreads=1)
    assert o.status == 0 and np.isnan(o.ER).all() and np.isnan(o.EBR).all()
    raw = oracle.run(p, rng=oracle.RNG_MT, nthreads=1, normalize=False)
    assert not raw.ER.any() and not raw.EBR.any()
    if oracle.have_reference_binaries():
        ref = oracle.ref_run(p, nthreads=1)
        for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI"):
            np.testing.assert_array_equal(np.isnan(getattr(o, k)), np.isnan(ref[k]), err_msg=k)


def test_negative_photon_count_runs_none_as_the_reference(built):
    """MonteCarlo's loop runs no photon for N < 0 and the normalisation divides by N:
    -0.0 everywhere; bit for bit (signs included) against the reference where built."""
    p = CASES["square2d"][0].copy(Nphoton=-5)
    o = oracle.run(p, rng=oracle.RNG_MT, nthreads=1)
    assert o.status == 0 and not o.ER.any() and np.signbit(o.ER).all()
    if oracle.have_reference_binaries():
        ref = oracle.ref_run(p, nthreads=1)
        for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI"):
            np.testing.assert_array_equal(getattr(o, k), ref[k], err_msg=k)
            np.testing.assert_array_equal(np.signbit(getattr(o, k)), np.signbit(ref[k]), err_msg=k)
