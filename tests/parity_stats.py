"""Batch-means statistics of the GPU parity tests (test infrastructure).

With B batches on each side, the difference of two batch means over its standard error is
close to t-distributed with the Welch-Satterthwaite degrees of freedom nu, so "within 3
sigma" is |t| below the t quantile of the 3-sigma coverage (0.99730) at nu, and chi2/dof
is near the mean of nu / (nu - 2) rather than 1.  Batch means of Monte Carlo tallies are
skewed, though (an element's score in a batch is a sum of a few dozen to a few hundred
photon contributions), and a skewed side with a variance that rises with its mean makes t
heavier-tailed than Student's: chi2/dof comes out above the t-expectation by 5-20 % on
elements with a relative standard error of a few percent, in the plain FP64 form too,
whose walk replays the reference's bit for bit.  So the gate compares each statistic with
its null value, measured on the same elements by the same comparison between the GPU
batches and a second, independent set of GPU batches of the oracle's batch size: under the
null hypothesis (the GPU form is distributed as the oracle) both have one distribution.
Neighbouring elements share photons and whole batches fluctuate together, so a mean of t
over elements has no small standard error; global offsets are tested on integrated
quantities with batch-to-batch errors instead (scalar_z).
"""
import math

import numpy as np

COVER3 = 0.99730020393674  # P(|z| < 3) of a normal variable


# ---------------------------------------------------------------------------------------

class Batches:
    """Per-element mean, squared standard error and scored-in-every-batch mask of B
    batches (rows)."""

    def __init__(self, rows):
        x = np.asarray(rows)
        self.B = x.shape[0]
        self.mean = x.mean(0)
        self.se2 = x.var(0, ddof=1) / self.B
        self.hit = np.all(x != 0, axis=0)


def welch(a: Batches, b: Batches, sel):
    """t statistic and Welch-Satterthwaite degrees of freedom of each selected element."""
    s2 = a.se2[sel] + b.se2[sel]
    t = (a.mean[sel] - b.mean[sel]) / np.sqrt(s2)
    nu = s2 ** 2 / (a.se2[sel] ** 2 / (a.B - 1) + b.se2[sel] ** 2 / (b.B - 1))
    return t, nu


def t_quantile(p, nu):
    from scipy.stats import t as student_t
    return student_t.ppf(p, nu)


def block_se(d, blocks=200):
    """Standard error of mean(d) from contiguous blocks of elements (element indices of the
    grid meshes run through space slab by slab, so a block is a compact region)."""
    parts = np.array_split(d, min(blocks, len(d)))
    n = np.array([len(q) for q in parts], float)
    m = np.array([q.mean() for q in parts])
    D = (n * m).sum() / n.sum()
    K = len(parts)
    return math.sqrt(K / (K - 1) * ((n * (m - D)) ** 2).sum()) / n.sum()


def _stats(a: Batches, b: Batches, sel):
    t, nu = welch(a, b, sel)
    q = t_quantile(0.5 + COVER3 / 2, nu)
    e = nu / (nu - 2.0)
    return dict(n=int(sel.sum()), within3=float(np.mean(np.abs(t) < q)), chi2=float(np.mean(t * t)),
                expect=float(np.mean(e)), se=block_se(t * t), mean_t=float(np.mean(t)))


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
            x = (f"{k} {r['n']}: within 3 sigma {r['within3']:.4f}, chi2/dof {r['chi2']:.3f} +- {r['se']:.3f} "
                 f"(t-expectation {r['expect']:.3f}), mean t {r['mean_t']:+.3f}")
            if "null" in r:
                nl = r["null"]
                x += f" [null: within 3 sigma {nl['within3']:.4f}, chi2/dof {nl['chi2']:.3f} +- {nl['se']:.3f}]"
            s.append(x)
    return f"{label}: " + "; ".join(s)


def chi2_excess_ok(r, rel_tol=0.05):
    """chi2/dof against its null value: within 5 % or three combined standard errors."""
    nl = r["null"]
    tol = max(rel_tol * nl["chi2"], 3.0 * math.hypot(r["se"], nl["se"]))
    return abs(r["chi2"] - nl["chi2"]) <= tol


def check_elements(label, rep, min_well=100):
    """The gate: on every element scored in every batch, at least 98.5 % within 3 sigma
    and chi2/dof at its null value; on the well-sampled ones (at least min_well of them),
    at least 99 % within 3 sigma, no fewer than the null comparison's fraction less 0.3 %,
    and chi2/dof at its null value."""
    print(fmt(label, rep))
    h, w = rep["hit"], rep["well"]
    assert h["n"] > 50, (label, rep)
    assert h["within3"] >= 0.985, (label, rep)
    assert chi2_excess_ok(h), (label, rep)
    assert w["n"] >= min_well, (label, rep)
    assert w["within3"] >= 0.99 and w["within3"] >= w["null"]["within3"] - 0.003, (label, rep)
    assert chi2_excess_ok(w), (label, rep)


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
