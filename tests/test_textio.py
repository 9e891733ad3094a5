"""The executables' text reader (valomc_gb300/csrc/app/textio.hpp), through vmc_textdump:

* files written like ValoMC.m writes them are read exactly (every array, every value);
* on malformed rows -- stray characters, numbers a stream cannot take, short rows, long
  lines, CRLF, misnamed or absent tags, truncated blocks -- it reads what the reference's
  reader (cpp/fileio.hpp, built into oracle/_ref/ref_textio) reads, value for value.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from golden.make_golden import cases
from valomc_gb300 import build as vbuild
from valomc_gb300 import meshgen as mg

TEXTDUMP = os.path.join(vbuild.BUILD, "vmc_textdump")
REF_TEXTIO = os.path.join(oracle.REF_DIR, "ref_textio")


def read_dump(path):
    out = {}
    with open(path) as fp:
        head = fp.readline().split()
        out["head"] = head
        while True:
            ln = fp.readline()
            if not ln:
                break
            name, rows, size = ln.split()
            vals = [fp.readline() for _ in range(int(size))]
            out[name] = (int(rows), np.array([float(v) for v in vals]))
    return out


def dump(binary, dim, path, td, tag):
    out = os.path.join(td, f"{tag}.dump")
    r = subprocess.run([binary, str(dim), path, out], capture_output=True, text=True, timeout=120)
    return r.returncode, (read_dump(out) if r.returncode == 0 else None)


@pytest.mark.parametrize("name", ["phantom3d", "mixed3d", "square2d", "mixed2d"])
def test_files_written_like_valomc_are_read_exactly(built, name):
    p = cases()[name][0]
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.txt")
        mg.write_input(fin, p)
        rc, d = dump(TEXTDUMP, p.dim, fin, td, "ours")
    assert rc == 0
    colmajor = lambda a: np.asarray(a, dtype=float).T.ravel() if np.ndim(a) == 2 else np.asarray(a, dtype=float)
    assert d["H"][0] == p.Ne and np.array_equal(d["H"][1], colmajor(p.H))
    assert np.array_equal(d["BH"][1], colmajor(p.BH))
    assert np.array_equal(d["r"][1], colmajor(p.r))
    for k in ("mua", "mus", "g", "n"):
        assert np.array_equal(d[k][1], np.asarray(getattr(p, k), float))
    assert np.array_equal(d["BCType"][1], np.asarray(p.BCType, float))
    if p.BCn is not None:
        assert np.array_equal(d["BCn"][1], np.asarray(p.BCn, float))
    if p.BCIntensity is not None:
        assert np.array_equal(d["BCIntensity"][1], np.asarray(p.BCIntensity, float))


def _edit(lines, tag, offset, new):
    i = lines.index(tag) + offset
    lines[i] = new(lines[i]) if callable(new) else new
    return lines


MALFORMED = {
    "int_given_as_float": (3, lambda L: _edit(L, "H", 2, "1.5 2 3 4")),
    "int_signs_and_overflow": (3, lambda L: _edit(L, "H", 3, "+1 -0 99999999999999999999 4")),
    "int_limits": (3, lambda L: _edit(L, "H", 4, "9223372036854775807 -9223372036854775808 0 1")),
    "int_bare_sign": (3, lambda L: _edit(L, "BH", 1, "- 2 3")),
    "int_hex": (2, lambda L: _edit(L, "H", 1, "0x10 1 2")),
    "double_garbage": (3, lambda L: _edit(L, "r", 1, "abc 1e5x -inf")),
    "double_exponent_forms": (3, lambda L: _edit(L, "r", 2, "1e 2.5E+3 -.5")),
    "double_two_points": (3, lambda L: _edit(L, "r", 3, "1.2.3 4 5")),
    "double_overflow": (3, lambda L: _edit(L, "r", 4, "1e999 -1e999 1e-400")),
    "double_hex_nan": (2, lambda L: _edit(L, "r", 1, "0x1p3 nan")),
    "double_short_row": (3, lambda L: _edit(L, "r", 5, "1.0")),
    "double_tabs_and_extra": (3, lambda L: _edit(L, "r", 6, "\t 2.5\t\t3.5 \t 4.5e-3 extra")),
    "optics_row_garbage": (3, lambda L: _edit(L, "mua mus g n", 1, "0.01 x 0.9 1.4")),
    "chars_with_spaces": (3, lambda L: _edit(L, "BCType", 1, "  l  x")),
    "long_line": (3, lambda L: _edit(L, "H", 1, lambda s: s + " " * 6000 + "7")),
    "crlf": (3, lambda L: [x + "\r" for x in L]),
    "no_final_newline": (3, lambda L: L[:-1] if L[-1] == "" else L),
    "empty_skip_line": (3, lambda L: L[:2] + [""] + L[3:]),
    "misnamed_optional_tag": (3, lambda L: _edit(L, "BCn", 0, "BCN")),
    "tag_with_spaces": (3, lambda L: _edit(L, "mua mus g n", 0, "mua  mus g   n ")),
    "truncated_required_block": (3, lambda L: L[:L.index("BH") + 3]),
}


@pytest.mark.skipif(not os.path.exists(REF_TEXTIO), reason="reference reader not built (no reference tree)")
@pytest.mark.parametrize("case", sorted(MALFORMED))
def test_malformed_rows_read_as_the_reference_reads_them(built, case):
    dim, mutate = MALFORMED[case]
    p = cases()["phantom3d" if dim == 3 else "mixed2d"][0]
    with tempfile.TemporaryDirectory() as td:
        base = os.path.join(td, "base.txt")
        mg.write_input(base, p)
        lines = mutate(open(base).read().split("\n"))
        fin = os.path.join(td, "in.txt")
        with open(fin, "w", newline="") as fp:
            fp.write("\n".join(lines))
        rc_o, ours = dump(TEXTDUMP, dim, fin, td, "ours")
        rc_r, ref = dump(REF_TEXTIO, dim, fin, td, "ref")
    assert rc_o == rc_r
    if rc_o == 0:
        assert ours.keys() == ref.keys()
        assert ours["head"] == ref["head"]
        for k in ours:
            if k == "head":
                continue
            assert ours[k][0] == ref[k][0], k
            np.testing.assert_array_equal(ours[k][1], ref[k][1], err_msg=k)
