"""Mesh import (valomc_gb300/meshio.py): createBH / createHN / createBH3 restated, NetGen
.vol reading as importNetGenMesh.m reads it, and -- where the reference tree is present --
the reference's own NetGen example (examples/square_with_two_circles.vol, the optics of
examples/netgentest.m) run by the oracle and by the reference engine, bit for bit."""
import os
import tempfile

import numpy as np
import pytest

import oracle
from valomc_gb300 import meshgen as mg
from valomc_gb300 import meshio

REF_VOL = oracle.reference_file("examples/square_with_two_circles.vol")


def rowset(a):
    return {tuple(x) for x in np.sort(np.asarray(a), axis=1).tolist()}


def test_create_bh_2d_is_the_grid_boundary():
    r, H, BH = mg.rectangular_mesh(6, 4, 0.5)
    B = meshio.create_bh(H)
    assert len(B) == len(BH) and rowset(B) == rowset(BH)


def test_create_bh_2d_lists_edges_column_major():
    # two triangles sharing edge (1, 2): boundary edges of element 0 are its edges 1 (0,1)
    # and 3 (2,0); of element 1, edges 2 (2,3) and 3 (3,1) -- listed edge by edge
    H = np.array([[0, 1, 2], [1, 3, 2]])
    np.testing.assert_array_equal(meshio.create_hn_2d(H), [[-1, 1, -1], [-1, -1, 0]])
    np.testing.assert_array_equal(meshio.create_bh(H), [[0, 1], [1, 3], [3, 2], [2, 0]])


def test_create_bh_3d_is_the_box_boundary_in_element_order():
    r, H, BH = mg.box_mesh_3d(4, 3, 2)
    B = meshio.create_bh(H)
    assert len(B) == len(BH) and rowset(B) == rowset(BH)
    # element by element, faces (0,1,2), (0,1,3), (0,2,3), (1,2,3) in order
    faces = H[:, meshio.FACES_3D]
    pos = []
    for row in B.tolist():
        hit = np.nonzero(np.all(faces == np.array(row)[None, None, :], axis=2))
        pos.append(hit[0][0] * 4 + hit[1][0])
    assert pos == sorted(pos)


def test_boundary_mothers_hold_the_boundary_nodes():
    for p in (mg.circles_2d(), mg.jittered_box_3d()):
        m = meshio.boundary_mothers(p.H, p.BH)
        assert np.all(m >= 0)
        for i in range(p.Nb):
            assert set(p.BH[i].tolist()) <= set(p.H[m[i]].tolist())


@pytest.mark.parametrize("maker", [mg.circles_2d, mg.jittered_box_3d])
def test_vol_round_trip(maker):
    p = maker()
    regions = {1: np.nonzero(p.n != 1.5)[0], 2: np.nonzero(p.n == 1.5)[0]}
    src = ord("c") if p.dim == 2 else ord("l")
    boundaries = {1: np.nonzero(p.BCType != src)[0], 2: np.nonzero(p.BCType == src)[0]}
    m = meshio.VolMesh(p.dim, p.H, p.r, p.BH, regions, {1: "tissue", 2: "inclusion"}, boundaries,
                       {1: "outside", 2: "lightsource"}, {1: False, 2: False})
    with tempfile.TemporaryDirectory() as td:
        f = os.path.join(td, "m.vol")
        meshio.write_vol(f, m)
        a = meshio.read_vol(f)
        b = meshio.read_vol(f, preserve_boundary=False)
    np.testing.assert_array_equal(a.H, p.H)
    np.testing.assert_array_equal(a.BH, p.BH)
    np.testing.assert_array_equal(a.r, p.r)
    assert a.region_names == {1: "tissue", 2: "inclusion"} and a.boundary_names[2] == "lightsource"
    for k in regions:
        np.testing.assert_array_equal(a.regions[k], regions[k])
    assert rowset(b.BH) == rowset(p.BH)
    # a rebuilt boundary keeps each named boundary, as indices into the new rows
    assert rowset(b.BH[b.boundaries[2]]) == rowset(p.BH[boundaries[2]])


def test_grid_fluence_averages_each_pixel_and_voxel():
    # a field constant per cell, given in MATLAB image order [y, x(, z)], comes back as is
    r, H, _ = mg.rectangular_mesh(6, 4, 1.0)
    c = r[H].mean(axis=1)
    ix, iy = np.floor(c[:, 0] + 3).astype(int), np.floor(c[:, 1] + 2).astype(int)
    f2 = np.random.default_rng(1).normal(size=(4, 6))
    np.testing.assert_allclose(mg.grid_fluence(f2[iy, ix], 4, 6), f2)
    r, H, _ = mg.box_mesh_3d(5, 4, 3)
    v = np.floor(r[H].mean(axis=1)).astype(int)
    f3 = np.random.default_rng(0).normal(size=(4, 5, 3))
    np.testing.assert_allclose(mg.grid_fluence(f3[v[:, 1], v[:, 0], v[:, 2]], 4, 5, 3), f3)
    with pytest.raises(ValueError):
        mg.grid_fluence(np.zeros(10), 4, 5, 3)


needs_vol = pytest.mark.skipif(REF_VOL is None, reason="reference example mesh not present")


@needs_vol
def test_reference_netgen_example_is_read():
    m = meshio.read_vol(REF_VOL, preserve_boundary=False)
    assert m.dim == 2 and m.H.shape == (21597, 3) and m.r.shape == (11002, 2)
    assert m.region_names == {1: "background", 2: "circles"}
    assert sum(len(v) for v in m.regions.values()) == 21597
    # the rebuilt boundary is the outer square; the circles' segments are interior
    assert len(m.BH) == 405 and rowset(m.BH) == rowset(meshio.create_bh(m.H))
    assert m.boundary_names[2] == "lightsource" and len(m.boundaries[2]) == 40 and not m.boundary_is_nodes[2]
    assert all(m.boundary_is_nodes[k] for k in range(7, 15))
    keep = meshio.read_vol(REF_VOL)
    assert len(keep.BH) == 597


def netgen_example_problem(nphoton):
    """examples/netgentest.m: background mua 0.01, mus 1.3, g 0.9, n 1.3; circles mua 0.09,
    mus 1.3, g 0.5, n 1.5; cosinic light source on the 'lightsource' boundary; the exterior
    index of each boundary row is its element's (createBoundary.m:72-82)."""
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
                      Nphoton=nphoton, seed=2024)


@needs_vol
@pytest.mark.skipif(not oracle.have_reference_binaries(), reason="reference engine not built")
def test_reference_netgen_example_oracle_equals_reference_engine(built):
    p = netgen_example_problem(20000)
    ref = oracle.ref_run(p, nthreads=2)
    ours = oracle.run(p, rng=oracle.RNG_MT, nthreads=2)
    assert ref["status"] == 0 and ours.status == 0
    for k in ("ER", "EBR", "DEBR"):
        np.testing.assert_array_equal(getattr(ours, k), ref[k], err_msg=k)
