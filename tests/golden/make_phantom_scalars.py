"""Integrated quantities of the 648k-tet inclusion phantom from the reference engine itself,
in independent batches, for the full-size GPU parity tests.

The per-element batch-means test compares each element's fluence within its own noise; a
small systematic error spread over many elements (a 0.5 % bias near the source passed it)
shows far more clearly in integrated quantities, whose batch-to-batch noise is small: the
absorbed fraction, the total exitance, the exitance through rings around the source and
through the opposite face, and the energy absorbed in the inclusion.  This script runs the
reference's MonteCarlo() (oracle/_ref/ref3d_run, MT19937, all host cores) on the phantom in
B batches of distinct seeds and stores, per batch, those linear functionals of its
normalised outputs (fixture phantom_scalars.npz; the frequency-domain phantom's in
phantom_fd_scalars.npz).

    python tests/golden/make_phantom_scalars.py [cw|fd] [batches] [photons per batch]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from valomc_gb300 import meshgen as mg  # noqa: E402

# ring edges (mm) of the top-face exitance around the source centre (30, 30)
RINGS = [(0.0, 1.0), (1.0, 2.0), (2.0, 5.0), (5.0, 10.0), (10.0, 20.0)]


def geometry(p):
    """Element volumes, boundary-triangle areas and centroids of a tetrahedral problem."""
    v = p.r[p.H]
    vol = np.abs(np.einsum("ij,ij->i", v[:, 1] - v[:, 0], np.cross(v[:, 2] - v[:, 0], v[:, 3] - v[:, 0]))) / 6.0
    b = p.r[p.BH]
    area = 0.5 * np.linalg.norm(np.cross(b[:, 1] - b[:, 0], b[:, 2] - b[:, 0]), axis=1)
    return vol, area, b.mean(axis=1), v.mean(axis=1)


def functionals(p):
    """Names and weights of the integrated quantities: (names, We [k x Ne], Wb [k x Nb]).
    Applied to the normalised outputs, sum(We ER) + sum(Wb EBR) is, in continuous wave,
    the absorbed or exited weight per launched photon (MonteCarlo's normalisation,
    cpp/3d/MC3D.hpp:1792-1818, divides ER by mua V N and EBR by A N)."""
    vol, area, bc, ec = geometry(p)
    cx, cy = 30.0, 30.0
    zmax = p.r[:, 2].max()
    top = np.abs(bc[:, 2]) < 1e-9
    bottom = np.abs(bc[:, 2] - zmax) < 1e-9
    rho = np.hypot(bc[:, 0] - cx, bc[:, 1] - cy)
    inc = ((ec - [cx, cy, 10.0]) ** 2).sum(1) < 25.0
    ne, nb = p.Ne, p.Nb
    names, We, Wb = [], [], []

    def add(name, we=None, wb=None):
        names.append(name)
        We.append(np.zeros(ne) if we is None else we)
        Wb.append(np.zeros(nb) if wb is None else wb)

    cw = p.f == 0
    ew = p.mua * vol if cw else vol
    add("absorbed" if cw else "element_sum", we=ew)
    add("exited", wb=area)
    for a, b in RINGS:
        add(f"top_ring_{a:g}_{b:g}mm", wb=np.where(top & (rho >= a) & (rho < b), area, 0.0))
    add("bottom_face", wb=np.where(bottom, area, 0.0))
    add("inclusion" if cw else "inclusion_sum", we=np.where(inc, ew, 0.0))
    return names, np.array(We), np.array(Wb)


def apply(W, ER, EBR):
    names, We, Wb = W
    return We @ ER + Wb @ EBR


def main():
    import oracle
    kind = sys.argv[1] if len(sys.argv) > 1 else "cw"
    B = int(sys.argv[2]) if len(sys.argv) > 2 else 20
    n = int(float(sys.argv[3])) if len(sys.argv) > 3 else 1_000_000
    p = mg.config_3d_phantom(nphoton=n, seed=1) if kind == "cw" else mg.config_3d_fd(nphoton=n, seed=1)
    W = functionals(p)
    threads = os.cpu_count() or 1
    rows_r, rows_i, secs = [], [], []
    for b in range(B):
        t0 = time.time()
        # thread t of a reference run draws from MT seed (seed + t) (MonteCarlo seeds thread t
        # with seed * totalthreads + t, cpp/3d/MC3D.hpp:1658, and totalthreads is 1 without
        # MPI): seeds 1000 apart keep every batch's streams apart
        out = oracle.ref_run(p.copy(seed=90000 + 1000 * b), nthreads=threads)
        assert out["status"] == 0
        rows_r.append(apply(W, out["ER"], out["EBR"]))
        rows_i.append(apply(W, out["EI"], out["EBI"]))
        secs.append(out["seconds"])
        print(f"batch {b}: {time.time() - t0:.1f} s, MonteCarlo {out['seconds']:.1f} s", flush=True)
    name = "phantom_scalars.npz" if kind == "cw" else "phantom_fd_scalars.npz"
    np.savez_compressed(os.path.join(HERE, name), names=np.array(W[0]), real=np.array(rows_r), imag=np.array(rows_i),
                        photons=n, threads=threads, seconds=np.array(secs),
                        engine="reference MonteCarlo() (oracle/_ref/ref3d_run), MT19937, seeds 90000 + 1000 batch")


if __name__ == "__main__":
    main()
