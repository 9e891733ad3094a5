"""Synthetic meshes and problem definitions for the photon-propagation path.

The grid builders restate ValoMC's MATLAB mesh generators so that element and boundary
numbering match what a ValoMC user gets:

* ``grid_mesh_2d``  -- createGridMesh.m (two-argument branch), two triangles per pixel;
  ``rectangular_mesh`` is createRectangularMesh.m:28 on top of it.
* ``grid_mesh_3d``  -- createGridMesh.m (three-argument branch), six tetrahedra per voxel
  with the connectivity table of createGridMesh.m:208-209 and the boundary triangles of
  createGridMesh.m:236-285.

All index arrays are 0-based, stored row-major as ``(rows, cols)`` numpy arrays; the C-ABI
wrappers convert them to the column-major layout of the reference's ``Array<T>``.
The named workloads (``config_*``) are the synthetic stand-ins for the benchmark
configurations: a 10x10 mm square (2D), the 60x60x30 mm inclusion phantom (3D CW and
frequency-domain), the 64-instance batch and the serving request mix.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

C0_MM_PER_S = 2.99792458e11  # speed of light used by the engines, cpp/3d/MC3D.hpp:178


@dataclasses.dataclass
class Problem:
    """One ValoMC problem: the arrays the MEX entry points receive (cpp/3d/MC3Dmex.cpp:98-139)."""

    dim: int
    H: np.ndarray                    # (Ne, dim+1) int64, 0-based
    BH: np.ndarray                   # (Nb, dim) int64
    r: np.ndarray                    # (Nr, dim) float64
    mua: np.ndarray
    mus: np.ndarray
    g: np.ndarray
    n: np.ndarray
    BCType: np.ndarray               # (Nb,) uint8 characters
    BCn: Optional[np.ndarray] = None
    BCLNormal: Optional[np.ndarray] = None        # (Nb, dim)
    BCLightDirectionType: Optional[np.ndarray] = None  # (Nb,) uint8
    BCIntensity: Optional[np.ndarray] = None
    GaussianSigma: Optional[np.ndarray] = None    # 2D only
    HN: Optional[np.ndarray] = None
    f: float = 0.0
    phase0: float = 0.0
    Nphoton: int = 1
    seed: int = 5489
    seedflag: int = 1

    @property
    def Ne(self) -> int:
        return int(self.H.shape[0])

    @property
    def Nb(self) -> int:
        return int(self.BH.shape[0])

    @property
    def Nr(self) -> int:
        return int(self.r.shape[0])

    def copy(self, **changes) -> "Problem":
        d = {}
        for fld in dataclasses.fields(self):
            v = getattr(self, fld.name)
            d[fld.name] = v.copy() if isinstance(v, np.ndarray) else v
        d.update(changes)
        return Problem(**d)


def chars(s, n=None) -> np.ndarray:
    """A BCType-style uint8 array from a string or list of one-character strings."""
    if isinstance(s, str) and n is not None and len(s) == 1:
        return np.full(n, ord(s), dtype=np.uint8)
    return np.frombuffer("".join(s).encode("ascii"), dtype=np.uint8).copy()


# ---------------------------------------------------------------------------
# 2D
# ---------------------------------------------------------------------------

def grid_mesh_2d(xvec, yvec):
    """createGridMesh(xvec, yvec): nodes at pixel corners, two triangles per pixel."""
    xvec = np.asarray(xvec, dtype=np.float64)
    yvec = np.asarray(yvec, dtype=np.float64)
    dx = abs(xvec[1] - xvec[0])
    dy = abs(yvec[1] - yvec[0])
    gx = np.append(xvec - dx / 2, xvec[-1] - dx / 2 + dx)
    gy = np.append(yvec - dy / 2, yvec[-1] - dy / 2 + dy)
    nx, ny = len(xvec), len(yvec)
    ysize, xsize = ny + 1, nx + 1
    # meshgrid(gx, gy) flattened column-major: y index fastest
    X, Y = np.meshgrid(gx, gy)
    r = np.stack([X.ravel(order="F"), Y.ravel(order="F")], axis=1)
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    k = (1 + j + i * ysize).ravel()  # 1-based running index of createGridMesh.m
    H1 = np.stack([k, k + 1, k + ysize], axis=1)
    H2 = np.stack([k + 1, k + ysize + 1, k + ysize], axis=1)
    H = np.concatenate([H1, H2]) - 1
    BH = []
    for jj in range(1, ny + 1):
        BH.append([jj, jj + 1])
    for jj in range(1, nx + 1):
        BH.append([ysize * jj, ysize * (jj + 1)])
    for jj in range(1, ny + 1):
        BH.append([ysize * xsize - (jj - 1), ysize * xsize - jj])
    for jj in range(1, nx + 1):
        BH.append([ysize * (xsize - 1) + 1 - ysize * (jj - 1), ysize * (xsize - 1) + 1 - ysize * jj])
    return r, H.astype(np.int64), np.asarray(BH, dtype=np.int64) - 1


def rectangular_mesh(xsize, ysize, dh):
    """createRectangularMesh.m:28."""
    xv = np.arange(-xsize / 2 + dh / 2, xsize / 2 - dh / 2 + dh / 2, dh)
    yv = np.arange(-ysize / 2 + dh / 2, ysize / 2 - dh / 2 + dh / 2, dh)
    return grid_mesh_2d(xv, yv)


# ---------------------------------------------------------------------------
# 3D
# ---------------------------------------------------------------------------

_POINTS = np.array([[0, 0, 0], [0, 1, 0], [1, 0, 0], [1, 1, 0], [0, 0, 1], [0, 1, 1], [1, 0, 1], [1, 1, 1]])
_CONN = np.array([[5, 1, 2, 3], [6, 5, 2, 3], [6, 7, 5, 3], [6, 4, 7, 3], [6, 2, 4, 3], [6, 8, 7, 4]]) - 1


def grid_mesh_3d(xvec, yvec, zvec):
    """createGridMesh(xvec, yvec, zvec): six tetrahedra per voxel, boundary triangles on the box."""
    xvec = np.asarray(xvec, dtype=np.float64)
    yvec = np.asarray(yvec, dtype=np.float64)
    zvec = np.asarray(zvec, dtype=np.float64)
    d = [abs(v[1] - v[0]) for v in (xvec, yvec, zvec)]
    gx = np.append(xvec - d[0] / 2, xvec[-1] - d[0] / 2 + d[0])
    gy = np.append(yvec - d[1] / 2, yvec[-1] - d[1] / 2 + d[1])
    gz = np.append(zvec - d[2] / 2, zvec[-1] - d[2] / 2 + d[2])
    NX, NY, NZ = len(gx), len(gy), len(gz)
    nx, ny, nz = NX - 1, NY - 1, NZ - 1

    def idx(i, j, k):  # 1-based (i: x, j: y, k: z) -> 1-based node index, createGridMesh.m:204
        return (k - 1) * NX * NY + (i - 1) * NY + j

    # node order: y fastest, then x, then z (meshgrid(x, y, z)(:))
    K, I, J = np.meshgrid(np.arange(NZ), np.arange(NX), np.arange(NY), indexing="ij")
    r = np.stack([gx[I.ravel()], gy[J.ravel()], gz[K.ravel()]], axis=1)
    # voxel loop order: t, k, i, j (j fastest)
    K, I, J = np.meshgrid(np.arange(1, nz + 1), np.arange(1, nx + 1), np.arange(1, ny + 1), indexing="ij")
    K, I, J = K.ravel(), I.ravel(), J.ravel()
    H = []
    for t in range(6):
        o = _POINTS[_CONN[t]]
        H.append(np.stack([idx(I + o[c, 0], J + o[c, 1], K + o[c, 2]) for c in range(4)], axis=1))
    H = np.concatenate(H) - 1
    BH = []
    # z faces: for i, for j: bottom pair then top pair
    I2, J2 = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), indexing="ij")
    I2, J2 = I2.ravel(), J2.ravel()
    rows = []
    for k in (1, nz + 1):
        a = np.stack([idx(I2, J2, k), idx(I2 + 1, J2, k), idx(I2, J2 + 1, k)], axis=1)
        b = np.stack([idx(I2 + 1, J2 + 1, k), idx(I2, J2 + 1, k), idx(I2 + 1, J2, k)], axis=1)
        rows += [a, b]
    BH.append(np.stack(rows, axis=1).reshape(-1, 3))
    # x faces: for j, for k
    J2, K2 = np.meshgrid(np.arange(1, ny + 1), np.arange(1, nz + 1), indexing="ij")
    J2, K2 = J2.ravel(), K2.ravel()
    rows = []
    for i in (1, nx + 1):
        a = np.stack([idx(i, J2, K2), idx(i, J2 + 1, K2), idx(i, J2, K2 + 1)], axis=1)
        b = np.stack([idx(i, J2 + 1, K2 + 1), idx(i, J2, K2 + 1), idx(i, J2 + 1, K2)], axis=1)
        rows += [a, b]
    BH.append(np.stack(rows, axis=1).reshape(-1, 3))
    # y faces: for k, for i
    K2, I2 = np.meshgrid(np.arange(1, nz + 1), np.arange(1, nx + 1), indexing="ij")
    K2, I2 = K2.ravel(), I2.ravel()
    rows = []
    for j in (1, ny + 1):
        a = np.stack([idx(I2, j, K2), idx(I2, j, K2 + 1), idx(I2 + 1, j, K2)], axis=1)
        b = np.stack([idx(I2 + 1, j, K2 + 1), idx(I2 + 1, j, K2), idx(I2, j, K2 + 1)], axis=1)
        rows += [a, b]
    BH.append(np.stack(rows, axis=1).reshape(-1, 3))
    BH = np.concatenate(BH) - 1
    return r, H.astype(np.int64), BH.astype(np.int64)


def box_mesh_3d(nx, ny, nz, dh=1.0, origin=(0.0, 0.0, 0.0)):
    """An nx*ny*nz voxel box of spacing dh with its corner at ``origin``."""
    xv = origin[0] + dh / 2 + dh * np.arange(nx)
    yv = origin[1] + dh / 2 + dh * np.arange(ny)
    zv = origin[2] + dh / 2 + dh * np.arange(nz)
    return grid_mesh_3d(xv, yv, zv)


def grid_fluence(element_fluence, nx, ny, nz=None):
    """ValoMC.m:266-271 / :340-351: the element fluence of a grid mesh (grid_mesh_2d: two
    triangles per pixel; grid_mesh_3d: six tetrahedra per voxel) averaged per pixel / voxel.
    nx, ny, nz are the sizes of the medium arrays' dimensions (createMedium.m:69-72, MATLAB
    image order): for a mesh from grid_mesh_2d / grid_mesh_3d(xvec, yvec[, zvec]) they are
    len(yvec), len(xvec)[, len(zvec)], and the result is indexed [y, x(, z)].  The mesh lists
    its elements in blocks, one per sub-element of every cell, each block in column-major
    cell order; each block is reshaped in that order and the blocks are averaged."""
    x = np.asarray(element_fluence)
    shape = (nx, ny) if nz is None else (nx, ny, nz)
    ncell = int(np.prod(shape))
    parts = 2 if nz is None else 6
    if x.shape[0] != parts * ncell:
        raise ValueError(f"{x.shape[0]} elements is not {parts} x {ncell} cells")
    blocks = [x[k * ncell:(k + 1) * ncell].reshape(shape, order="F") for k in range(parts)]
    return sum(blocks) / parts


# ---------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------

def config_2d_square(nphoton=1_000_000, seed=12345):
    """10x10 mm square, dh = 1 mm (200 triangles, 121 nodes); mua 0.01, mus 1.0, g 0.9,
    n 1.3 inside and 1.0 outside; cosinic source on boundary edges 4..7 (MATLAB numbering,
    examples/simpletest.m:37)."""
    r, H, BH = rectangular_mesh(10, 10, 1)
    ne, nb = len(H), len(BH)
    bct = np.full(nb, ord("a"), np.uint8)
    bct[3:7] = ord("c")
    return Problem(dim=2, H=H, BH=BH, r=r,
                   mua=np.full(ne, 0.01), mus=np.full(ne, 1.0), g=np.full(ne, 0.9), n=np.full(ne, 1.3),
                   BCType=bct, BCn=np.ones(nb), Nphoton=int(nphoton), seed=seed, seedflag=1)


def top_face_mask(r, BH, z0=0.0):
    return np.all(np.isclose(r[BH][:, :, 2], z0), axis=1)


def gaussian_footprint(r, BH, cx, cy, sigma=1.0, z0=0.0, floor=1e-6):
    """Spatial Gaussian source: 'l' (direct) on top-face triangles weighted by
    exp(-rho^2 / 2 sigma^2) at the triangle centroid; weights below ``floor`` become 'a'."""
    c = r[BH].mean(axis=1)
    top = top_face_mask(r, BH, z0)
    w = np.exp(-((c[:, 0] - cx) ** 2 + (c[:, 1] - cy) ** 2) / (2 * sigma * sigma))
    sel = top & (w > floor)
    bct = np.where(sel, ord("l"), ord("a")).astype(np.uint8)
    inten = np.where(sel, w, 1.0)
    return bct, inten


def config_3d_phantom(nphoton=100_000_000, seed=12345, scale=1.0):
    """60x60x30 mm inclusion phantom on a 1 mm grid (648 000 tetrahedra): background
    mua 0.01, mus 10, g 0.9, n 1.4; a sphere r = 5 mm at depth 10 mm with mua 0.05;
    Fresnel boundary to n = 1.0; Gaussian (sigma 1 mm) direct source at the top centre.
    ``scale`` < 1 shrinks the box (same optics) for quick parity cases."""
    nx, ny, nz = int(round(60 * scale)), int(round(60 * scale)), int(round(30 * scale))
    r, H, BH = box_mesh_3d(nx, ny, nz)
    ne, nb = len(H), len(BH)
    cx, cy = nx / 2.0, ny / 2.0
    cz = 10.0 * scale
    rad = 5.0 * scale
    cen = r[H].mean(axis=1)
    mua = np.where(((cen - [cx, cy, cz]) ** 2).sum(1) < rad * rad, 0.05, 0.01)
    bct, inten = gaussian_footprint(r, BH, cx, cy, sigma=1.0)
    return Problem(dim=3, H=H, BH=BH, r=r, mua=mua, mus=np.full(ne, 10.0), g=np.full(ne, 0.9),
                   n=np.full(ne, 1.4), BCType=bct, BCn=np.ones(nb), BCIntensity=inten,
                   Nphoton=int(nphoton), seed=seed, seedflag=1)


def config_3d_fd(nphoton=100_000_000, seed=12345, gen_seed=3, scale=1.0):
    """The phantom with per-tet mua ~ lognormal (arithmetic mean 0.01, log-sd 0.3) and
    mus ~ U(8, 12), source modulated at 100 MHz."""
    p = config_3d_phantom(nphoton, seed, scale)
    rng = np.random.default_rng(gen_seed)
    s = 0.3
    p.mua = rng.lognormal(mean=math.log(0.01) - s * s / 2, sigma=s, size=p.Ne)
    p.mus = rng.uniform(8.0, 12.0, size=p.Ne)
    p.f = 100e6
    return p


def pencil_box(L, mua, mus, g, n, point, nphoton, seed, dh=1.0):
    """An L^3 mm cube with homogeneous optics and a pencil beam entering at ``point`` on the
    z = 0 face: 'p' on the top triangle containing the point, direction type 'p', BCLNormal =
    the point (ValoMC.m:274-291)."""
    r, H, BH = box_mesh_3d(L, L, L, dh)
    ne, nb = len(H), len(BH)
    bct = np.full(nb, ord("a"), np.uint8)
    top = np.nonzero(top_face_mask(r, BH))[0]
    px, py = point
    tri = None
    for ib in top:
        a, b, c = r[BH[ib]][:, :2]
        v0, v1, v2 = b - a, c - a, np.array([px, py]) - a
        den = v0[0] * v1[1] - v1[0] * v0[1]
        u = (v2[0] * v1[1] - v1[0] * v2[1]) / den
        v = (v0[0] * v2[1] - v2[0] * v0[1]) / den
        if u >= 0 and v >= 0 and u + v <= 1:
            tri = ib
            break
    assert tri is not None
    bct[tri] = ord("p")
    bcln = np.zeros((nb, 3))
    bcln[tri] = [px, py, 0.0]
    dt = np.full(nb, ord("n"), np.uint8)
    dt[tri] = ord("p")
    return Problem(dim=3, H=H, BH=BH, r=r, mua=np.full(ne, mua), mus=np.full(ne, mus), g=np.full(ne, g),
                   n=np.full(ne, n), BCType=bct, BCn=np.ones(nb), BCLNormal=bcln, BCLightDirectionType=dt,
                   Nphoton=int(nphoton), seed=seed, seedflag=1)


def config_batch(count=64, gen_seed=4, lmin=20, lmax=80, pmin=1e5, pmax=1e7, photon_scale=1.0):
    """64 cubes with edge L ~ log-uniform[20, 80] mm (1 mm grid, 6 L^3 tets), homogeneous
    optics mua U[0.005, 0.1], mus U[5, 20], g U[0.8, 0.95], n U[1.33, 1.45], BCn = 1, a pencil
    source at a uniform random top-face point, photons log-uniform[1e5, 1e7]."""
    rng = np.random.default_rng(gen_seed)
    out = []
    for i in range(count):
        L = int(round(math.exp(rng.uniform(math.log(lmin), math.log(lmax)))))
        mua = rng.uniform(0.005, 0.1)
        mus = rng.uniform(5, 20)
        g = rng.uniform(0.8, 0.95)
        n = rng.uniform(1.33, 1.45)
        pt = (rng.uniform(0.05, L - 0.05), rng.uniform(0.05, L - 0.05))
        nph = int(math.exp(rng.uniform(math.log(pmin), math.log(pmax))) * photon_scale)
        out.append(pencil_box(L, mua, mus, g, n, pt, max(nph, 1), seed=1000 + i))
    return out


def cosinic_disk(r, BH, cx, cy, radius=1.0, z0=0.0):
    """'c' (cosinic) on the top-face triangles whose centroid lies within ``radius`` of (cx, cy)."""
    c = r[BH].mean(axis=1)
    sel = top_face_mask(r, BH, z0) & (((c[:, 0] - cx) ** 2 + (c[:, 1] - cy) ** 2) <= radius * radius)
    if not sel.any():  # at least the nearest top triangle
        d = np.where(top_face_mask(r, BH, z0), (c[:, 0] - cx) ** 2 + (c[:, 1] - cy) ** 2, np.inf)
        sel[np.argmin(d)] = True
    return np.where(sel, ord("c"), ord("a")).astype(np.uint8)


class ServingMix:
    """The serving workload: 8 resident cubes with tet counts log-uniform in [50k, 2M]
    (1 mm grid), requests choosing a mesh, a source (cosinic disk r = 1 mm, or a Gaussian
    sigma = 1 mm direct footprint) at a uniform random top-face point, homogeneous optics as
    in the batch workload, and photons log-uniform in [1e5, 1e7]."""

    def __init__(self, seed=5, meshes=8, tmin=50_000, tmax=2_000_000, pmin=1e5, pmax=1e7):
        self.rng = np.random.default_rng(seed)
        self.pmin, self.pmax = pmin, pmax
        self.base = []
        for _ in range(meshes):
            ntet = math.exp(self.rng.uniform(math.log(tmin), math.log(tmax)))
            L = max(4, int(round((ntet / 6) ** (1 / 3))))
            r, H, BH = box_mesh_3d(L, L, L)
            ne, nb = len(H), len(BH)
            self.base.append(Problem(dim=3, H=H, BH=BH, r=r, mua=np.full(ne, 0.01), mus=np.full(ne, 10.0),
                                     g=np.full(ne, 0.9), n=np.full(ne, 1.4), BCType=np.full(nb, ord("a"), np.uint8),
                                     BCn=np.ones(nb), Nphoton=1, seed=1))
            self.base[-1].L = L

    def request(self):
        rng = self.rng
        k = int(rng.integers(len(self.base)))
        b = self.base[k]
        L = b.L
        cx, cy = rng.uniform(0.5, L - 0.5), rng.uniform(0.5, L - 0.5)
        if rng.random() < 0.5:
            bct, inten = cosinic_disk(b.r, b.BH, cx, cy), None
        else:
            bct, inten = gaussian_footprint(b.r, b.BH, cx, cy, sigma=1.0)
        ne = b.Ne
        p = Problem(dim=3, H=b.H, BH=b.BH, r=b.r, mua=np.full(ne, rng.uniform(0.005, 0.1)),
                    mus=np.full(ne, rng.uniform(5, 20)), g=np.full(ne, rng.uniform(0.8, 0.95)),
                    n=np.full(ne, rng.uniform(1.33, 1.45)), BCType=bct, BCn=np.ones(b.Nb), BCIntensity=inten,
                    Nphoton=int(math.exp(rng.uniform(math.log(self.pmin), math.log(self.pmax)))),
                    seed=int(rng.integers(1 << 31)))
        return k, p


# ---------------------------------------------------------------------------
# text format of the external executables
# ---------------------------------------------------------------------------

def uneven_mesh_2d(n=20, size=10.0, jitter=0.3, seed=6):
    """An unstructured-looking triangle mesh of the square [-size/2, size/2]^2: an n x n grid
    whose interior nodes are moved by up to jitter x h and whose cells are split along a
    random diagonal, so element shapes, sizes and node valences (4-8) vary.  The boundary
    is built by createBH (meshio.create_bh)."""
    from .meshio import create_bh
    rng = np.random.default_rng(seed)
    h = size / n
    g = np.linspace(-size / 2, size / 2, n + 1)
    X, Y = np.meshgrid(g, g, indexing="ij")
    r = np.stack([X.ravel(), Y.ravel()], axis=1)
    inner = (np.abs(r[:, 0]) < size / 2 - 1e-9) & (np.abs(r[:, 1]) < size / 2 - 1e-9)
    r[inner] += rng.uniform(-jitter * h, jitter * h, size=(int(inner.sum()), 2))
    node = lambda i, j: i * (n + 1) + j
    H = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = node(i, j), node(i + 1, j), node(i + 1, j + 1), node(i, j + 1)
            if rng.random() < 0.5:
                H += [[a, b, c], [a, c, d]]
            else:
                H += [[a, b, d], [b, c, d]]
    H = np.asarray(H, np.int64)
    return r, H, create_bh(H)


def circles_2d(nphoton=20000, seed=12345):
    """Two circular inclusions (n 1.5, mua 0.09, g 0.5) in a scattering square (n 1.3,
    mua 0.01, mus 1.3, g 0.9) on an uneven mesh, air outside (Fresnel at the boundary), a
    cosinic source on the left edge -- the optics of the reference's NetGen example
    (examples/netgentest.m) on a mesh made here."""
    r, H, BH = uneven_mesh_2d()
    cen = r[H].mean(axis=1)
    inc = (np.hypot(cen[:, 0] + 2.0, cen[:, 1] + 1.5) < 1.6) | (np.hypot(cen[:, 0] - 2.2, cen[:, 1] - 1.8) < 1.2)
    ne, nb = len(H), len(BH)
    mua = np.where(inc, 0.09, 0.01)
    mus = np.full(ne, 1.3)
    g = np.where(inc, 0.5, 0.9)
    n = np.where(inc, 1.5, 1.3)
    mid = r[BH].mean(axis=1)
    types = np.full(nb, ord("a"), np.uint8)
    types[mid[:, 0] < -5.0 + 1e-9] = ord("c")
    return Problem(dim=2, H=H, BH=BH, r=r, mua=mua, mus=mus, g=g, n=n, BCType=types, BCn=np.ones(nb),
                   Nphoton=nphoton, seed=seed)


def jittered_box_3d(nphoton=3000, seed=12345, gen_seed=8):
    """An 8 x 8 x 6 mm box of tets whose interior nodes are moved by up to 0.25 mm, with a
    spherical inclusion (n 1.5) in n 1.37 tissue, air outside, a direct source on the
    top-face triangles near the centre; boundary built by createBH3 (meshio.create_bh)."""
    from .meshio import create_bh
    r, H, _ = box_mesh_3d(8, 8, 6)
    rng = np.random.default_rng(gen_seed)
    lo, hi = r.min(axis=0), r.max(axis=0)
    inner = np.all((r > lo + 1e-9) & (r < hi - 1e-9), axis=1)
    r = r.copy()
    r[inner] += rng.uniform(-0.25, 0.25, size=(int(inner.sum()), 3))
    BH = create_bh(H)
    cen = r[H].mean(axis=1)
    inc = np.linalg.norm(cen - np.array([4.0, 4.0, 2.5]), axis=1) < 1.5
    ne, nb = len(H), len(BH)
    mid = r[BH].mean(axis=1)
    types = np.full(nb, ord("a"), np.uint8)
    top = (np.abs(mid[:, 2] - lo[2]) < 1e-9) & (np.hypot(mid[:, 0] - 4.0, mid[:, 1] - 4.0) < 1.5)
    types[top] = ord("l")
    return Problem(dim=3, H=H, BH=BH, r=r, mua=np.where(inc, 0.2, 0.02), mus=np.where(inc, 3.0, 6.0),
                   g=np.where(inc, 0.6, 0.85), n=np.where(inc, 1.5, 1.37), BCType=types, BCn=np.ones(nb),
                   Nphoton=nphoton, seed=seed)


def write_input(path, p: Problem, nxyz=None, dirtype_tag=None):
    """The executables' input file (cpp/3d/MC3D.cpp:97-179, cpp/2d/MC2D.cpp:125-203,
    written like ValoMC.m:200-258,293-336)."""
    D = p.dim
    with open(path, "w") as fp:
        fp.write(f"{p.Ne} {p.Nb} {p.Nr} {p.Nphoton}\n")
        fp.write(f"{p.f!r} {p.phase0!r} {p.seed} {p.seedflag}\n")
        nxyz = nxyz or (0,) * D
        fp.write(" ".join(str(v) for v in nxyz) + "\n")

        def block(tag, arr, fmt):
            fp.write(tag + "\n")
            arr = np.asarray(arr)
            if arr.ndim == 1:
                arr = arr[:, None]
            fp.write("\n".join(" ".join(fmt(v) for v in row) for row in arr.tolist()) + "\n")

        ifmt = lambda v: str(int(v))
        ffmt = lambda v: repr(float(v))
        block("H", p.H, ifmt)
        block("BH", p.BH, ifmt)
        block("r", p.r, ffmt)
        block("mua mus g n", np.stack([p.mua, p.mus, p.g, p.n], 1), ffmt)
        fp.write("BCType\n" + "\n".join(chr(c) for c in p.BCType.tolist()) + "\n")
        if p.BCn is not None:
            block("BCn", p.BCn, ffmt)
        if p.BCLNormal is not None:
            block("BCLightDirection", p.BCLNormal, ffmt)
        if p.BCLightDirectionType is not None:
            tag = dirtype_tag or ("BCLDirType" if D == 3 else "BCLightDirectionType")
            fp.write(tag + "\n" + "\n".join(chr(c) for c in p.BCLightDirectionType.tolist()) + "\n")
        if p.BCIntensity is not None:
            block("BCIntensity", p.BCIntensity, ffmt)
        if D == 2 and p.GaussianSigma is not None:
            block("GaussianSigma", p.GaussianSigma, ffmt)


def read_output(path, Ne, Nb):
    """The executables' output file (cpp/3d/MC3D.cpp:186-201): a time line, Ne rows ER EI,
    Nb rows EBR EBI."""
    with open(path) as fp:
        lines = fp.read().split("\n")
    vals = np.array([[float(x) for x in ln.split()] for ln in lines[1:1 + Ne + Nb]])
    return vals[:Ne, 0], vals[:Ne, 1], vals[Ne:, 0], vals[Ne:, 1]
