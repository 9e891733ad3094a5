"""Generates the golden fixtures of tests/golden/ by running the reference engine itself.

The reference (cpp/3d/MC3D.hpp, cpp/2d/MC2D.hpp) is compiled from the reference tree by
oracle/Makefile into oracle/_ref/ (timed runner and tape-replay tracer, see
oracle/ref_harness.cpp).  This script needs that tree and those binaries; the fixtures it
writes are what the tests use everywhere else, so nothing at test time needs the
reference.

    python tests/golden/make_golden.py [case ...]

Fixtures (numpy .npz, float64 at full precision):
  run_<case>.npz    MonteCarlo() output of the reference with MT19937, given thread count
  trace_<case>.npz  per-photon element sequences of the reference fed a tape of uniforms
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from valomc_gb300 import meshgen as mg  # noqa: E402


def mixed_3d(seed=1, nphoton=3000, f=0.0):
    """A small box with every 3D boundary type, direction type, per-element optics and
    index jumps, so every branch of CreatePhoton / PropagatePhoton is taken."""
    r, H, BH = mg.box_mesh_3d(6, 5, 4)
    ne, nb = len(H), len(BH)
    rng = np.random.default_rng(seed)
    types = rng.choice([ord(c) for c in "aamlicCILp"], size=nb).astype(np.uint8)
    dtype = rng.choice([ord(c) for c in "nnar"], size=nb).astype(np.uint8)
    dtype[types == ord("p")] = ord("p")
    for bad in (ord("L"), ord("I")):  # the reference leaves these undefined with type 'n'
        dtype[(types == bad) & (dtype == ord("n"))] = ord("a")
    bcl = rng.normal(size=(nb, 3))
    # pencil points inside their triangles but off the centroid: an axis-aligned ray from a
    # face centroid of this grid runs inside an interior face plane of the six-tet split
    w = np.array([0.2, 0.3, 0.5])
    pts = np.einsum("k,ikc->ic", w, r[BH])
    bcl[types == ord("p")] = pts[types == ord("p")]
    return mg.Problem(dim=3, H=H, BH=BH, r=r, mua=rng.uniform(0.01, 0.5, ne), mus=rng.uniform(0, 5, ne),
                      g=rng.uniform(0, .95, ne), n=rng.uniform(1.0, 1.5, ne), BCType=types,
                      BCn=rng.uniform(0, 1.5, nb), BCLNormal=bcl, BCLightDirectionType=dtype,
                      BCIntensity=rng.uniform(0.5, 2, nb), Nphoton=nphoton, seed=7, f=f, phase0=-1.0 if f else 0.0)


def mixed_2d(seed=2, nphoton=3000, f=0.0):
    r, H, BH = mg.rectangular_mesh(6, 4, 0.5)
    ne, nb = len(H), len(BH)
    rng = np.random.default_rng(seed)
    types = rng.choice([ord(c) for c in "aamlicgLIC"], size=nb).astype(np.uint8)
    dtype = rng.choice([ord(c) for c in "nnar"], size=nb).astype(np.uint8)
    return mg.Problem(dim=2, H=H, BH=BH, r=r, mua=rng.uniform(0.0, 0.5, ne), mus=rng.uniform(0, 5, ne),
                      g=rng.uniform(0, .95, ne), n=rng.uniform(1.0, 1.5, ne), BCType=types,
                      BCn=rng.uniform(0, 1.5, nb), BCLNormal=rng.normal(size=(nb, 2)), BCLightDirectionType=dtype,
                      BCIntensity=rng.uniform(0.5, 2, nb), GaussianSigma=rng.uniform(0.2, 1.0, nb),
                      Nphoton=nphoton, seed=9, f=f)


def cases():
    """name -> (Problem, reference thread count)"""
    return {
        "square2d": (mg.config_2d_square(nphoton=20000, seed=12345), 1),
        "square2d_t3": (mg.config_2d_square(nphoton=20000, seed=12345), 3),
        "phantom3d": (mg.config_3d_phantom(nphoton=2000, seed=12345, scale=0.25), 2),
        "phantom3d_fd": (mg.config_3d_fd(nphoton=1000, seed=77, scale=0.25), 1),
        "mixed3d": (mixed_3d(), 2),
        "mixed3d_fd": (mixed_3d(f=2e8), 1),
        "mixed2d": (mixed_2d(), 2),
        "mixed2d_fd": (mixed_2d(f=1e8), 1),
        "pencil3d": (mg.pencil_box(8, 0.05, 12.0, 0.85, 1.4, (3.3, 4.45), 2000, seed=11), 1),
        # uneven meshes: jittered nodes, random cell diagonals, boundaries from createBH
        "circles2d": (mg.circles_2d(nphoton=20000, seed=321), 2),
        "jitter3d": (mg.jittered_box_3d(nphoton=3000, seed=654), 2),
        # isotropic scattering of a beam along the z axis: every first scatter takes
        # ScatterPhoton's on-axis branch, half of them backwards
        "iso3d": (mg.pencil_box(8, 0.05, 6.0, 0.0, 1.4, (3.35, 4.15), 3000, seed=13), 2),
    }


def tape_for(case, nphot=24, words=6000, seed=424242):
    rng = np.random.default_rng(seed + sum(map(ord, case)))
    tape = rng.integers(0, 2 ** 32, size=nphot * words, dtype=np.uint64).astype(np.uint32)
    return tape, np.arange(nphot + 1, dtype=np.int64) * words


TRACE_CASES = ["phantom3d", "mixed3d", "mixed3d_fd", "pencil3d", "square2d", "mixed2d", "mixed2d_fd", "circles2d",
               "jitter3d", "iso3d"]


def main(only=None):
    import oracle
    oracle.build()
    if not oracle.have_reference_binaries():
        raise SystemExit("oracle/_ref/ binaries are missing: the reference tree is needed to make fixtures")
    for name, (p, nthr) in cases().items():
        if only and name not in only:
            continue
        out = oracle.ref_run(p, nthreads=nthr)
        assert out["status"] == 0, (name, out)
        np.savez_compressed(os.path.join(HERE, f"run_{name}.npz"), threads=nthr, loss=out["loss"],
                            **{k: out[k] for k in ("ER", "EI", "EBR", "EBI", "DEBR", "DEBI")})
        print(name, "threads", nthr, "loss", out["loss"])
    for name in TRACE_CASES:
        if only and name not in only:
            continue
        p = cases()[name][0]
        tape, off = tape_for(name)
        tr, used, acc = oracle.ref_trace(p, tape, off)
        assert max(used) < off[1], f"tape too short for {name}"
        lens = np.array([len(t) for t in tr], np.int64)
        np.savez_compressed(os.path.join(HERE, f"trace_{name}.npz"), lens=lens, events=np.concatenate(tr),
                            used=np.array(used, np.int64), **{k: acc[k] for k in ("ER", "EI", "EBR", "EBI", "DEBR")})
        print("trace", name, "photons", len(tr), "max len", lens.max(), "max words", max(used))


if __name__ == "__main__":
    # optional case names: regenerate only those fixtures
    main(set(sys.argv[1:]) or None)
