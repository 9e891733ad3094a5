"""Mesh import for ValoMC problems: NetGen ``.vol`` files and boundary construction.

* ``read_vol`` follows importNetGenMesh.m: the sections ``dimension``,
  ``surfaceelements[gi]``, ``volumeelements[gi]``, ``edgesegmentsgi2`` /
  ``edgesegments``, ``points``, ``materials`` and ``bcnames``; 2D meshes take H from the
  surface elements (columns p1..p3), BH from the edge segments (p1, p2) and regions from
  the surface elements' second column; 3D meshes take H from the volume elements, BH from
  the surface elements and regions from the volume elements' first column.  With
  ``preserve_boundary=False`` the boundary is rebuilt by ``create_bh`` with sorted rows,
  and each named boundary is mapped onto the new rows (importNetGenMesh.m:104-128).
* ``create_bh`` follows createBH.m: in 2D the edges (1,2), (2,3), (3,1) of each triangle
  without a neighbour (createHN.m), listed edge by edge and, within an edge, element by
  element (MATLAB's column-major ``find(HN == 0)``); in 3D the faces (0,1,2), (0,1,3),
  (0,2,3), (1,2,3) that no other tetrahedron shares, element by element
  (cpp/3d/createBH3mex.cpp:34-75).
* ``boundary_mothers`` is findBoundaryElementsFromElements: the element that owns each
  boundary row, which createBoundary.m uses for the default exterior refractive index.

All indices are 0-based (the C ABI's convention); ``regions`` and ``boundaries`` map a
region / boundary number of the file (1-based, as NetGen writes them) to index arrays.
"""
from __future__ import annotations

import dataclasses
from typing import Dict, List, Optional, Union

import numpy as np

FACES_3D = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]])
EDGES_2D = np.array([[0, 1], [1, 2], [2, 0]])


@dataclasses.dataclass
class VolMesh:
    dim: int
    H: np.ndarray                     # (Ne, dim+1) int64, 0-based
    r: np.ndarray                     # (Nr, dim) float64
    BH: np.ndarray                    # (Nb, dim) int64, 0-based
    regions: Dict[int, np.ndarray]    # region number -> element indices
    region_names: Dict[int, str]
    boundaries: Dict[int, np.ndarray]  # boundary number -> BH rows (or node rows, see read_vol)
    boundary_names: Dict[int, str]
    boundary_is_nodes: Dict[int, bool]


def _read_entry(lines, i):
    """A counted section starting at lines[i] (the count); returns (rows, names, next i)."""
    count = int(lines[i].split()[0])
    rows, names = [], {}
    for k in range(count):
        ln = lines[i + 1 + k]
        parts = ln.split()
        try:
            rows.append([float(v) for v in parts])
        except ValueError:
            names[int(parts[0])] = parts[1] if len(parts) > 1 else ""
    return rows, names, i + 1 + count


def read_vol(path: str, preserve_boundary: bool = True) -> VolMesh:
    with open(path) as fp:
        lines = fp.read().split("\n")
    sect = {}
    dim = None
    i = 0
    order = ("surfaceelements", "surfaceelementsgi", "volumeelements", "volumeelementsgi", "materials",
             "bcnames", "edgesegmentsgi2", "edgesegments", "points")
    while i < len(lines):
        t = lines[i].rstrip("\r")
        i += 1
        if t == "dimension" and dim is None:
            dim = int(lines[i].split()[0])
            i += 1
            continue
        if t in order:
            # the first of the alternative names wins, as in the reference's loop
            key = {"surfaceelementsgi": "surfaceelements", "volumeelementsgi": "volumeelements",
                   "edgesegments": "edgesegmentsgi2"}.get(t, t)
            if key in sect:
                continue
            rows, names, i = _read_entry(lines, i)
            sect[key] = (rows, names)
    if dim not in (2, 3):
        raise ValueError("Could not read dimensionality!")
    as_int = lambda rows, cols: np.asarray([[int(round(v)) for v in r] for r in rows], np.int64)[:, cols]
    materials = sect.get("materials", ([], {}))[1]
    bcnames = sect.get("bcnames", ([], {}))[1]
    pts = np.asarray(sect["points"][0], np.float64)
    if dim == 2:
        se = sect["surfaceelements"][0]
        es = sect["edgesegmentsgi2"][0]
        H = as_int(se, slice(5, 8)) - 1
        r = pts[:, 0:2].copy()
        BH = as_int(es, slice(2, 4)) - 1
        bnum = as_int(es, slice(0, 1))[:, 0]
        dnum = as_int(se, slice(1, 2))[:, 0]
    else:
        ve = sect["volumeelements"][0]
        se = sect["surfaceelements"][0]
        H = as_int(ve, slice(2, 6)) - 1
        r = pts[:, 0:3].copy()
        BH = as_int(se, slice(5, 8)) - 1
        bnum = as_int(se, slice(1, 2))[:, 0]
        dnum = as_int(ve, slice(0, 1))[:, 0]
    regions = {k: np.nonzero(dnum == k)[0] for k in range(1, int(dnum.max()) + 1)}
    boundaries = {k: np.nonzero(bnum == k)[0] for k in range(1, int(bnum.max()) + 1)}
    is_nodes = {k: False for k in boundaries}
    bnames = dict(bcnames)
    if not preserve_boundary:
        old = BH
        BH = np.sort(create_bh(H), axis=1)
        for k in list(boundaries):
            cur = np.sort(old[boundaries[k]], axis=1)
            idx = _intersect_rows(cur, BH)
            if len(idx) != cur.shape[0]:
                # the segment is not on the new boundary: keep its node rows
                boundaries[k] = old[boundaries[k]]
                is_nodes[k] = True
            else:
                boundaries[k] = idx
            if len(boundaries[k]) == 0:
                bnames[k] = ""
    return VolMesh(dim, H, r, BH, regions, dict(materials), boundaries, bnames, is_nodes)


def _intersect_rows(A, B):
    """MATLAB's [~, ~, ib] = intersect(A, B, 'rows'): indices into B of the rows common to
    A and B, in the sorted order of those rows (first occurrence in B)."""
    if len(A) == 0 or len(B) == 0:
        return np.zeros(0, np.int64)
    common = {}
    for j, row in enumerate(map(tuple, B.tolist())):
        common.setdefault(row, j)
    rows = sorted({tuple(a) for a in A.tolist()} & common.keys())
    return np.asarray([common[rw] for rw in rows], np.int64)


def create_hn_2d(H: np.ndarray) -> np.ndarray:
    """createHN.m: for edges (1,2), (2,3), (3,1) of each triangle the element sharing both
    nodes, or -1 (MATLAB's 0)."""
    H = np.asarray(H, np.int64)
    Ne = H.shape[0]
    e = np.sort(H[:, EDGES_2D], axis=2).reshape(-1, 2)          # (Ne*3, 2)
    owner = np.repeat(np.arange(Ne), 3)
    _, inv, cnt = np.unique(e, axis=0, return_inverse=True, return_counts=True)
    inv = inv.ravel()
    if np.any(cnt > 2):
        raise ValueError("an edge is shared by more than two elements")
    HN = np.full(Ne * 3, -1, np.int64)
    order = np.argsort(inv, kind="stable")
    s = inv[order]
    pair = np.nonzero(s[1:] == s[:-1])[0]
    a, b = order[pair], order[pair + 1]
    HN[a] = owner[b]
    HN[b] = owner[a]
    return HN.reshape(Ne, 3)


def create_bh(H: np.ndarray) -> np.ndarray:
    """createBH.m (2D) / createBH3mex (3D): the boundary rows of a mesh, 0-based."""
    H = np.asarray(H, np.int64)
    if H.shape[1] == 3:
        HN = create_hn_2d(H)
        rows = []
        for k, (a, b) in enumerate(EDGES_2D):          # column-major find(HN == 0)
            els = np.nonzero(HN[:, k] < 0)[0]
            rows.append(np.stack([H[els, a], H[els, b]], axis=1))
        return np.concatenate(rows, axis=0) if rows else np.zeros((0, 2), np.int64)
    faces = H[:, FACES_3D]                                   # (Ne, 4, 3)
    key = np.sort(faces, axis=2).reshape(-1, 3)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    open_ = (cnt[inv.ravel()] == 1).reshape(H.shape[0], 4)
    return faces[open_]                                      # element by element, faces in order


def boundary_mothers(H: np.ndarray, BH: np.ndarray) -> np.ndarray:
    """findBoundaryElementsFromElements: the element holding each boundary row's nodes."""
    H = np.asarray(H, np.int64)
    BH = np.asarray(BH, np.int64)
    d = BH.shape[1]
    sub = EDGES_2D if d == 2 else FACES_3D
    key = np.sort(H[:, sub], axis=2).reshape(-1, d)
    owner = np.repeat(np.arange(H.shape[0]), sub.shape[0])
    table = {}
    for j, row in enumerate(map(tuple, key.tolist())):
        table.setdefault(row, owner[j])
    out = np.full(BH.shape[0], -1, np.int64)
    for i, row in enumerate(map(tuple, np.sort(BH, axis=1).tolist())):
        out[i] = table.get(row, -1)
    return out


def write_vol(path: str, mesh: VolMesh) -> None:
    """A NetGen .vol file with the sections read_vol reads (for meshes made here)."""
    d = mesh.dim
    with open(path, "w") as fp:
        fp.write("mesh3d\ndimension\n%d\ngeomtype\n0\n\n" % d)
        dom = np.zeros(mesh.H.shape[0], np.int64)
        for k, idx in mesh.regions.items():
            dom[idx] = k
        bnd = np.zeros(mesh.BH.shape[0], np.int64)
        for k, idx in mesh.boundaries.items():
            if not mesh.boundary_is_nodes.get(k, False):
                bnd[idx] = k
        if d == 2:
            fp.write("surfaceelements\n%d\n" % mesh.H.shape[0])
            for t, e in zip(mesh.H + 1, dom):
                fp.write(" 2 %d 0 0 3 %d %d %d\n" % (e, t[0], t[1], t[2]))
            fp.write("\nedgesegmentsgi2\n%d\n" % mesh.BH.shape[0])
            for s, b in zip(mesh.BH + 1, bnd):
                fp.write(" %d 0 %d %d 0 0 1 0 1 0 1 0\n" % (b, s[0], s[1]))
        else:
            fp.write("surfaceelements\n%d\n" % mesh.BH.shape[0])
            for s, b in zip(mesh.BH + 1, bnd):
                fp.write(" 1 %d 1 0 3 %d %d %d\n" % (b, s[0], s[1], s[2]))
            fp.write("\nvolumeelements\n%d\n" % mesh.H.shape[0])
            for t, e in zip(mesh.H + 1, dom):
                fp.write(" %d 4 %d %d %d %d\n" % (e, t[0], t[1], t[2], t[3]))
        fp.write("\npoints\n%d\n" % mesh.r.shape[0])
        for p in mesh.r:
            q = list(p) + [0.0] * (3 - d)
            fp.write("  %.17g %.17g %.17g\n" % tuple(q))
        fp.write("materials\n%d\n" % len(mesh.region_names))
        for k, nm in sorted(mesh.region_names.items()):
            fp.write("%d %s\n" % (k, nm))
        fp.write("\nbcnames\n%d\n" % len(mesh.boundary_names))
        for k, nm in sorted(mesh.boundary_names.items()):
            fp.write("%d\t%s\n" % (k, nm))
        fp.write("\nendmesh\n")
