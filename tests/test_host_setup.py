"""Host half of the drop-in, without a GPU: the library loads and exports every entry
point of include/valomc_gb300.h; ErrorChecks codes and order; BuildNeighbourhoods equal to
the reference's (restated in the oracle), including its error cases."""
import os
import re

import numpy as np
import pytest

import oracle
import valomc_gb300 as V
from golden.make_golden import cases
from valomc_gb300 import api
from valomc_gb300 import meshgen as mg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "valomc_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(vmc_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_entry_point(built):
    L = V.lib()
    names = header_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(api.EXPORTS) == set(names)
    assert L.vmc_abi_version() == 1


def test_status_strings_are_the_reference_texts(built):
    L = V.lib()
    assert L.vmc_status_string(1) == b"No lightsource"
    assert L.vmc_status_string(4) == b"Undefined error"  # SIZE_MISMATCH_MUS has no text in the reference
    assert L.vmc_status_string(16).startswith(b"Ill defined mesh - a complete boundary")


def run_status(p):
    """Status of vmc_run; the checks run before any device is touched."""
    r = V.run(p, check=False, nphoton=1)
    return r.stats["status"]


@pytest.mark.parametrize("mutate,code", [
    (lambda p: p.copy(g=p.g[:-1]), 2),
    (lambda p: p.copy(mua=p.mua[:-1]), 3),
    (lambda p: p.copy(mus=p.mus[:-1]), 4),
    (lambda p: p.copy(n=p.n[:-1]), 5),
    (lambda p: p.copy(BCn=p.BCn[:-1]), 6),
    (lambda p: p.copy(BCn=None), 7),
    (lambda p: p.copy(BCType=p.BCType[:-1]), 8),
    (lambda p: p.copy(BCLNormal=np.zeros((3, p.dim))), 9),
    (lambda p: p.copy(BCLightDirectionType=np.full(3, ord("n"), np.uint8)), 10),
    (lambda p: p.copy(H=np.where(p.H == 0, p.Nr + 5, p.H)), 11),
    (lambda p: p.copy(BH=np.where(p.BH == 0, -1, p.BH)), 12),
    (lambda p: p.copy(BCType=np.full(p.Nb, ord("a"), np.uint8)), 1),
])
def test_errorchecks_codes_match_oracle(built, mutate, code):
    p = mutate(cases()["phantom3d"][0])
    assert run_status(p) == code
    assert oracle.run(p, nphoton=1).status == code


def test_errorchecks_order_mua_before_mus(built):
    p = cases()["phantom3d"][0]
    q = p.copy(mua=p.mua[:-1], mus=p.mus[:-1])
    assert run_status(q) == 3


def test_no_emitting_face_is_reported(built):
    # only mirror faces: the reference's has_lightsource passes but no source exists
    p = cases()["phantom3d"][0].copy()
    p.BCType[:] = ord("m")
    assert run_status(p) == 1
    assert oracle.run(p, nphoton=1).status == 1


def test_2d_gaussian_needs_sigma(built):
    p = mg.config_2d_square(nphoton=1)
    p.BCType[3] = ord("g")
    assert run_status(p) == 15


MESHES = {
    "phantom": lambda: cases()["phantom3d"][0],
    "mixed3d": lambda: cases()["mixed3d"][0],
    "square2d": lambda: cases()["square2d"][0],
    "mixed2d": lambda: cases()["mixed2d"][0],
    "pencil": lambda: cases()["pencil3d"][0],
}


@pytest.mark.parametrize("name", sorted(MESHES))
def test_neighbourhood_equals_reference(built, name):
    p = MESHES[name]()
    s, hn = V.build_neighbourhood(p)
    s2, hn2 = oracle.build_neighbours(p)
    assert s == s2 == 0
    np.testing.assert_array_equal(hn, hn2)
    # every interior face is shared both ways, every boundary element appears once
    D = p.dim + 1
    inner = hn >= 0
    for el, f in zip(*np.nonzero(inner)):
        assert el in hn[hn[el, f]]
    b = -1 - hn[hn < 0]
    assert np.array_equal(np.sort(b), np.arange(p.Nb))


def test_neighbourhood_errors_match_reference(built):
    # a boundary triangle listed twice: two candidates for one face
    p = cases()["phantom3d"][0]
    q = p.copy(BH=np.concatenate([p.BH, p.BH[:1]]), BCType=np.concatenate([p.BCType, p.BCType[:1]]),
               BCn=np.concatenate([p.BCn, p.BCn[:1]]), BCIntensity=np.concatenate([p.BCIntensity, p.BCIntensity[:1]]))
    assert V.build_neighbourhood(q)[0] == oracle.build_neighbours(q)[0] == 14
    # 3D open face: left at INT64_MAX, like the reference
    q = p.copy(BH=p.BH[1:], BCType=p.BCType[1:], BCn=p.BCn[1:], BCIntensity=p.BCIntensity[1:])
    s, hn = V.build_neighbourhood(q)
    s2, hn2 = oracle.build_neighbours(q)
    assert s == s2 == 0
    np.testing.assert_array_equal(hn, hn2)
    assert (hn == np.iinfo(np.int64).max).sum() == 1
    # 2D missing boundary edge
    p2 = cases()["square2d"][0]
    q2 = p2.copy(BH=p2.BH[1:], BCType=p2.BCType[1:], BCn=p2.BCn[1:])
    assert V.build_neighbourhood(q2)[0] == oracle.build_neighbours(q2)[0] == 16
    # 2D duplicate edge
    q2 = p2.copy(BH=np.concatenate([p2.BH, p2.BH[5:6]]), BCType=np.concatenate([p2.BCType, p2.BCType[:1]]),
                 BCn=np.concatenate([p2.BCn, p2.BCn[:1]]))
    assert V.build_neighbourhood(q2)[0] == oracle.build_neighbours(q2)[0] == 13


def test_meshgen_matches_createGridMesh_counts():
    r, H, BH = mg.box_mesh_3d(60, 60, 30)
    assert (len(H), len(BH), len(r)) == (648000, 28800, 115351)
    r2, H2, BH2 = mg.rectangular_mesh(10, 10, 1)
    assert (len(H2), len(BH2), len(r2)) == (200, 40, 121)
    # boundary edges 4..7 of simpletest.m are the x = -5 side's first four, y from -5 to -1
    assert np.allclose(r2[BH2[3:7]][:, :, 0], -5.0)
