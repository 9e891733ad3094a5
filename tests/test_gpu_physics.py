"""Known-answer checks of the photon physics on the GPU (both arithmetic forms):
Beer-Lambert attenuation, the normal-incidence Fresnel split, total internal reflection,
mirror boundaries keeping all weight inside, and the frequency-domain result reducing to
the continuous-wave one as f -> 0."""
import math

import numpy as np
import pytest

import valomc_gb300 as V
from valomc_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu
FORMS = [V.VMC_FP64, V.VMC_FP32]


def face_mask(p, axis, value):
    return np.all(np.isclose(p.r[p.BH][:, :, axis], value), axis=1)


@pytest.mark.parametrize("precision", FORMS)
def test_beer_lambert_through_a_non_scattering_slab(built, precision):
    L = 10
    r, H, BH = mg.box_mesh_3d(4, 4, L)
    ne = len(H)
    # pencil on the z = 0 face of a 4 x 4 x 10 mm box, matched index outside (no Fresnel)
    q = mg.Problem(dim=3, H=H, BH=BH, r=r, mua=np.full(ne, 0.1), mus=np.zeros(ne), g=np.zeros(ne),
                   n=np.ones(ne), BCType=np.zeros(len(BH), np.uint8), Nphoton=20000, seed=3)
    bct = np.full(len(BH), ord("a"), np.uint8)
    top = np.nonzero(face_mask(q, 2, 0.0))[0]
    # the z = 0 triangle containing (1.3, 2.45): x in [1, 2], y in [2, 3], lower-left half
    ib = [i for i in top if np.allclose(sorted(q.r[BH[i]][:, 0]), [1, 1, 2]) and
          np.allclose(sorted(q.r[BH[i]][:, 1]), [2, 2, 3])][0]
    bct[ib] = ord("p")
    bcl = np.zeros((len(BH), 3))
    bcl[ib] = [1.3, 2.45, 0.0]
    dt = np.full(len(BH), ord("n"), np.uint8)
    dt[ib] = ord("p")
    q = q.copy(BCType=bct, BCLNormal=bcl, BCLightDirectionType=dt, BCn=np.ones(len(BH)), BCIntensity=None)
    res = V.run(q, precision=precision, normalize=False)
    bottom = face_mask(q, 2, float(L))
    got = res.EBR[bottom].sum() / q.Nphoton
    assert res.stats["loss"] == 0
    assert abs(got - math.exp(-0.1 * L)) < 2e-6, got
    assert res.EBR[~bottom].sum() == 0


@pytest.mark.parametrize("precision", FORMS)
def test_normal_incidence_fresnel_split(built, precision):
    """n = 1.4 inside, 1.0 outside, no absorption or scattering: a normally incident photon
    leaves through the far face with probability 1 / (1 + R), R = ((n1 - n2)/(n1 + n2))^2."""
    r, H, BH = mg.box_mesh_3d(4, 4, 6)
    ne, nb = len(H), len(BH)
    bct = np.full(nb, ord("a"), np.uint8)
    top = face_mask(mg.Problem(3, H, BH, r, None, None, None, None, None), 2, 0.0)
    bct[top] = ord("l")
    p = mg.Problem(dim=3, H=H, BH=BH, r=r, mua=np.zeros(ne), mus=np.zeros(ne), g=np.zeros(ne), n=np.full(ne, 1.4),
                   BCType=bct, BCn=np.ones(nb), Nphoton=400000, seed=5)
    res = V.run(p, precision=precision, normalize=False)
    bottom = face_mask(p, 2, 6.0)
    R = ((1.4 - 1.0) / 2.4) ** 2
    frac = res.EBR[bottom].sum() / p.Nphoton
    want = 1 / (1 + R)
    sigma = math.sqrt(want * (1 - want) / p.Nphoton)
    assert abs(frac - want) < 5 * sigma, (frac, want)
    assert abs(res.EBR.sum() / p.Nphoton - 1.0) < 1e-9  # nothing absorbed, nothing lost


@pytest.mark.parametrize("precision", FORMS)
def test_total_internal_reflection(built, precision):
    """Direct light tilted 60 deg from the normal in n = 1.5 (critical angle 41.8 deg) can
    never leave through the top or bottom faces; it escapes through the sides only."""
    r, H, BH = mg.box_mesh_3d(12, 12, 2)
    ne, nb = len(H), len(BH)
    shell = mg.Problem(3, H, BH, r, None, None, None, None, None)
    top, bottom = face_mask(shell, 2, 0.0), face_mask(shell, 2, 2.0)
    bct = np.where(top, ord("l"), ord("a")).astype(np.uint8)
    bcl = np.zeros((nb, 3))
    bcl[:] = [math.sin(math.radians(60)), 0.0, math.cos(math.radians(60))]
    dt = np.where(top, ord("a"), ord("n")).astype(np.uint8)
    p = mg.Problem(dim=3, H=H, BH=BH, r=r, mua=np.full(ne, 1e-3), mus=np.zeros(ne), g=np.zeros(ne),
                   n=np.full(ne, 1.5), BCType=bct, BCn=np.ones(nb), BCLNormal=bcl, BCLightDirectionType=dt,
                   Nphoton=100000, seed=6)
    res = V.run(p, precision=precision, normalize=False)
    assert res.EBR[top | bottom].sum() == 0.0
    assert res.EBR.sum() > 0.5 * p.Nphoton
    assert res.stats["loss"] == 0


@pytest.mark.parametrize("precision", FORMS)
def test_mirror_box_keeps_all_weight(built, precision):
    """Every face a mirror except one direct source face ('L' = mirror that also emits):
    nothing exits; absorbed weight plus the roulette ledger closes the launched weight."""
    r, H, BH = mg.box_mesh_3d(5, 5, 5)
    ne, nb = len(H), len(BH)
    shell = mg.Problem(3, H, BH, r, None, None, None, None, None)
    bct = np.full(nb, ord("m"), np.uint8)
    bct[np.nonzero(face_mask(shell, 2, 0.0))[0][:4]] = ord("L")
    bcl = np.tile([0.0, 0.0, 1.0], (nb, 1))
    dt = np.full(nb, ord("a"), np.uint8)
    p = mg.Problem(dim=3, H=H, BH=BH, r=r, mua=np.full(ne, 0.2), mus=np.full(ne, 5.0), g=np.full(ne, 0.8),
                   n=np.full(ne, 1.33), BCType=bct, BCn=np.ones(nb), BCLNormal=bcl, BCLightDirectionType=dt,
                   Nphoton=200000, seed=7)
    res = V.run(p, precision=precision, normalize=False)
    L = res.stats["ledger"]
    assert res.EBR.sum() == 0.0
    closed = L["launched"] + L["roulette_gain"] - L["roulette_kill"] - L["lost"]
    assert abs(L["absorbed"] - closed) / L["launched"] < 1e-6, L


def test_frequency_domain_tends_to_continuous_wave(built):
    from golden.make_golden import cases
    p = cases()["phantom3d"][0]
    cw = V.run(p, precision=V.VMC_FP64, nphoton=20000, seed=12)
    fd = V.run(p.copy(f=1.0), precision=V.VMC_FP64, nphoton=20000, seed=12)
    hit = cw.ER > 0
    np.testing.assert_allclose(fd.ER[hit], cw.ER[hit], rtol=1e-6)
    assert np.abs(fd.EI).max() < 1e-6 * np.abs(fd.ER).max()
    np.testing.assert_allclose(fd.EBR, cw.EBR, rtol=1e-9, atol=1e-300)


@pytest.mark.parametrize("g", [0.0, 0.5])
def test_backscatter_from_the_beam_axis_matches_the_plain_form(built, g):
    """A pencil beam along +z into a scattering box (isotropic and forward scattering):
    the first scatter turns a direction that is exactly on the z axis, the case
    ScatterPhoton handles apart (MC3D.hpp:1316-1320, dz' = cos(theta) sign(dz)). The FP32
    form must backscatter there like the plain form: the same absorbed and exited
    fractions within 5 sigma, and the same mean walk length within 1%."""
    # the entry point lies on no cell diagonal (x - y and x + y not integers), so the beam
    # runs inside no face plane
    p = mg.pencil_box(12, 0.02, 5.0, 0.9, 1.4, (6.35, 5.15), 400000, seed=91)
    p = p.copy(g=np.full(p.Ne, g))
    out = {}
    for prec in FORMS:
        r = V.run(p, precision=prec, normalize=False)
        L = r.stats["ledger"]
        assert r.stats["loss"] == 0 and r.stats["photons_done"] == p.Nphoton
        out[prec] = (L["absorbed"] / p.Nphoton, L["exited"] / p.Nphoton, r.stats["steps"] / p.Nphoton)
    a64, e64, s64 = out[V.VMC_FP64]
    a32, e32, s32 = out[V.VMC_FP32]
    sig = math.sqrt(2 * a64 * (1 - a64) / p.Nphoton)
    assert abs(a32 - a64) < 5 * sig, (g, a32, a64, sig)
    assert abs(e32 - e64) < 5 * sig, (g, e32, e64, sig)
    assert abs(s32 / s64 - 1) < 0.01, (g, s32, s64)
