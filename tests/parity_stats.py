"""Batch-means statistics of the GPU parity tests (test infrastructure).

With B batches on each side, the difference of two batch means over its standard error is
close to t-distributed with the Welch-Satterthwaite degrees of freedom nu, so "within 3
sigma" is |t| below the t quantile of the 3-sigma coverage (0.99730) at nu, and chi2/dof
is near the mean of nu / (nu - 2) rather than 1.  Two things make the analytic values
unreliable as a gate:

* Batch means of Monte Carlo tallies are skewed (an element's score in a batch is a sum of
  a few dozen to a few hundred photon contributions), and a side whose variance rises with
  its mean makes t heavier-tailed than Student's: chi2/dof comes out 5-20 % above the
  t-expectation, in the plain FP64 form too, whose walk replays the reference's bit for bit.
  So each statistic is compared with its null value: the same comparison between the GPU
  batches and a second, independent set of GPU batches of the reference side's batch size
  (under the null hypothesis -- the GPU form is distributed as the reference -- both have
  one distribution), on the same elements.
* Elements share photons and whole batches fluctuate together (a batch whose photons went
  deeper raises a whole region), so these statistics fluctuate far more than their
  independent-element error suggests.  Their standard errors come from a delete-one-batch
  jackknife over the batches of both sides, which carries every correlation between
  elements.

Offsets shared by many elements are also tested on integrated quantities with
batch-to-batch errors (scalar_z).
"""
import math

import numpy as np

COVER3 = 0.99730020393674  # P(|z| < 3) of a normal variable


class Batches:
    """B batches (rows) of per-element tallies: mean, squared standard error of the mean,
    scored-in-every-batch mask; the rows are kept for the jackknife."""

    def __init__(self, rows):
        self.x = np.asarray(rows, dtype=np.float64)
        self.B = self.x.shape[0]
        self.mean = self.x.mean(0)
        self.se2 = self.x.var(0, ddof=1) / self.B
        self.hit = np.all(self.x != 0, axis=0)

    def leave_out(self, sel):
        """(mean, se2) of the selected elements with each batch left out in turn."""
        x = self.x[:, sel]
        B = self.B
        S, Q = x.sum(0), (x * x).sum(0)
        for i in range(B):
            m = (S - x[i]) / (B - 1)
            v = (Q - x[i] * x[i] - (B - 1) * m * m) / (B - 2)
            yield m, np.maximum(v, 0.0) / (B - 1)


def welch_nu(s2a, s2b, Ba, Bb):
    return (s2a + s2b) ** 2 / (s2a ** 2 / (Ba - 1) + s2b ** 2 / (Bb - 1))


def t_quantile(p, nu):
    from scipy.stats import t as student_t
    return student_t.ppf(p, nu)


def _summary(ma, s2a, mb, s2b, q):
    s2 = s2a + s2b
    ok = s2 > 0
    t = (ma[ok] - mb[ok]) / np.sqrt(s2[ok])
    return float(np.mean(t * t)), float(np.mean(np.abs(t) < q[ok])), float(np.mean(t))


def _stats(a: Batches, b: Batches, sel):
    ma, s2a, mb, s2b = a.mean[sel], a.se2[sel], b.mean[sel], b.se2[sel]
    nu = welch_nu(s2a, s2b, a.B, b.B)
    q = t_quantile(0.5 + COVER3 / 2, nu)
    chi2, within3, mean_t = _summary(ma, s2a, mb, s2b, q)
    # delete-one-batch jackknife over both sides (independent), the quantiles held fixed
    var = np.zeros(3)
    for side in (a, b):
        reps = []
        for m, s2 in side.leave_out(sel):
            reps.append(_summary(m, s2, mb, s2b, q) if side is a else _summary(ma, s2a, m, s2, q))
        reps = np.array(reps)
        var += (side.B - 1) / side.B * ((reps - reps.mean(0)) ** 2).sum(0)
    se = np.sqrt(var)
    return dict(n=int(sel.sum()), within3=within3, chi2=chi2, expect=float(np.mean(nu / (nu - 2.0))),
                se=float(se[0]), se_within3=float(se[1]), mean_t=mean_t, se_mean_t=float(se[2]))


def element_report(a: Batches, b: Batches, null: Batches = None, rel=0.05):
    """GPU batches `a` against reference batches `b` over the elements scored in every
    batch ("hit"), and over the well-sampled ones (relative standard error below `rel`);
    with `null` (independent GPU batches of b's size), the same statistics of a against
    null on the same elements."""
    sides = [a, b] + ([null] if null is not None else [])
    hit = np.logical_and.reduce([x.hit for x in sides])
    well = hit.copy()
    for x in sides:
        well[hit] &= np.sqrt(x.se2[hit]) < rel * np.abs(x.mean[hit])
    out = {}
    for name, sel in (("hit", hit), ("well", well)):
        if not sel.any():
            out[name] = dict(n=0)
            continue
        out[name] = _stats(a, b, sel)
        if null is not None:
            out[name]["null"] = _stats(a, null, sel)
    return out


def fmt(label, rep):
    s = []
    for k in ("hit", "well"):
        r = rep[k]
        if r["n"]:
            x = (f"{k} {r['n']}: within 3 sigma {r['within3']:.4f} +- {r['se_within3']:.4f}, chi2/dof {r['chi2']:.3f} "
                 f"+- {r['se']:.3f} (t-expectation {r['expect']:.3f}), mean t {r['mean_t']:+.3f} +- {r['se_mean_t']:.3f}")
            if "null" in r:
                nl = r["null"]
                x += (f" [null: within 3 sigma {nl['within3']:.4f}, chi2/dof {nl['chi2']:.3f} +- {nl['se']:.3f}, "
                      f"mean t {nl['mean_t']:+.3f} +- {nl['se_mean_t']:.3f}]")
            s.append(x)
    return f"{label}: " + "; ".join(s)


def chi2_excess_ok(r):
    """chi2/dof at its null value, within three standard errors of the difference (the
    two share the GPU side, so the sum of their variances bounds it from above)."""
    nl = r["null"]
    return abs(r["chi2"] - nl["chi2"]) <= 3.0 * math.hypot(r["se"], nl["se"]) + 0.01


def mean_t_ok(r):
    """The mean signed t over the elements at its null value (an offset shared by many
    elements moves it long before it moves chi2/dof)."""
    nl = r["null"]
    return abs(r["mean_t"] - nl["mean_t"]) <= 3.0 * math.hypot(r["se_mean_t"], nl["se_mean_t"]) + 0.01


def within3_ok(r, floor):
    nl = r["null"]
    return r["within3"] >= floor and \
        r["within3"] >= nl["within3"] - 3.0 * math.hypot(r["se_within3"], nl["se_within3"]) - 0.001


def check_elements(label, rep, min_well=100):
    """The gate: on every element scored in every batch, at least 98.5 % within 3 sigma
    and chi2/dof at its null value; on the well-sampled ones (at least min_well of them),
    at least 99 % within 3 sigma and no fewer than the null comparison's fraction, and
    chi2/dof and the mean signed t at their null values; each within three jackknife
    standard errors."""
    print(fmt(label, rep))
    h, w = rep["hit"], rep["well"]
    assert h["n"] > 50, (label, rep)
    assert within3_ok(h, 0.985) and chi2_excess_ok(h), (label, rep)
    assert w["n"] >= min_well, (label, rep)
    assert within3_ok(w, 0.99) and chi2_excess_ok(w) and mean_t_ok(w), (label, rep)


def scalar_z(label, names, g_rows, r_rows):
    """z of each integrated quantity: GPU batches against reference batches."""
    g, r = np.asarray(g_rows), np.asarray(r_rows)
    gm, gs = g.mean(0), g.std(0, ddof=1) / math.sqrt(len(g))
    rm, rs = r.mean(0), r.std(0, ddof=1) / math.sqrt(len(r))
    z = (gm - rm) / np.sqrt(gs ** 2 + rs ** 2)
    for k, nm in enumerate(names):
        print(f"{label} {nm}: GPU {gm[k]:.6e} +- {gs[k]:.1e}, reference {rm[k]:.6e} +- {rs[k]:.1e}, "
              f"relative difference {(gm[k] - rm[k]) / rm[k]:+.2e}, z {z[k]:+.2f}")
    return z
