"""The drop-in boundary is plain C: a C99 program compiled with -pedantic -Werror against
include/valomc_gb300.h links the library and calls its host-only entry points (no GPU)."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "valomc_gb300", "_build")

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "valomc_gb300.h"

int main(void) {
  /* the unit square as two triangles sharing the edge (1, 2); arrays column-major, 0-based */
  const int64_t H[6] = {0, 1, 1, 3, 2, 2};
  const int64_t BH[8] = {0, 1, 3, 2, 1, 3, 2, 0};
  const double r[8] = {0.0, 1.0, 0.0, 1.0, 0.0, 0.0, 1.0, 1.0};
  vmc_input in;
  vmc_options opt;
  int64_t HN[6];
  int i, s;
  memset(&in, 0, sizeof in);
  in.dim = 2;
  in.Ne = 2;
  in.Nb = 4;
  in.Nr = 4;
  in.H = H;
  in.BH = BH;
  in.r = r;
  s = vmc_build_neighbourhood(&in, HN);
  vmc_default_options(&opt);
  printf("abi %d status %d precision %d rng %d normalize %d ok \"%s\"\n", vmc_abi_version(), s, opt.precision,
         opt.rng, opt.normalize, vmc_status_string(VMC_OK));
  printf("HN");
  for (i = 0; i < 6; i++) printf(" %lld", (long long)HN[i]);
  printf("\n");
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_is_c99_and_the_library_links(built):
    with tempfile.TemporaryDirectory() as td:
        src, exe = os.path.join(td, "abi.c"), os.path.join(td, "abi")
        with open(src, "w") as fp:
            fp.write(PROGRAM)
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        src, "-o", exe, "-L" + BUILD, "-lvalomc_gb300", "-Wl,-rpath," + BUILD],
                       check=True, capture_output=True, text=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=60).stdout.split("\n")
    head = out[0].split()
    assert head[1] == "1" and head[3] == "0"  # ABI version, status OK
    assert head[5] == "1" and head[7] == "0" and head[9] == "1"  # FP32 tracking, Philox, normalised
    hn = [int(x) for x in out[1].split()[1:]]
    # column-major [2 x 3]: element 0's row is hn[0::2], element 1's is hn[1::2]
    e0, e1 = hn[0::2], hn[1::2]
    assert e0.count(1) == 1 and e1.count(0) == 1  # the shared edge, seen from both sides
    boundary = sorted(-1 - x for x in hn if x < 0)
    assert boundary == [0, 1, 2, 3]  # each boundary edge once, as -1 - ib


LAYOUT = r"""
#include <stddef.h>
#include <stdio.h>
#include "valomc_gb300.h"
#define F(T, m) printf(#T " " #m " %zu\n", offsetof(T, m))
#define S(T) printf(#T " sizeof %zu\n", sizeof(T))
int main(void) {
%BODY%
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_python_structs_have_the_headers_layout(built):
    """Every ctypes mirror of a header struct (valomc_gb300/api.py) has the C compiler's size
    and field offsets, so no field is missing, added or misplaced on either side."""
    from valomc_gb300 import api
    pairs = {"vmc_input": api.VmcInput, "vmc_output": api.VmcOutput, "vmc_options": api.VmcOptions,
             "vmc_stats": api.VmcStats, "vmc_server_config": api.VmcServerConfig,
             "vmc_noalloc_buffers": api.VmcNoallocBuffers}
    body = []
    for cname, py in pairs.items():
        body.append(f"  S({cname});")
        body += [f"  F({cname}, {f[0]});" for f in py._fields_]
    with tempfile.TemporaryDirectory() as td:
        src, exe = os.path.join(td, "layout.c"), os.path.join(td, "layout")
        with open(src, "w") as fp:
            fp.write(LAYOUT.replace("%BODY%", "\n".join(body)))
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                       check=True, capture_output=True, text=True)
        lines = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=60).stdout.split("\n")
    c = {}
    for ln in lines:
        if ln.strip():
            t, m, v = ln.split()
            c[(t, m)] = int(v)
    import ctypes
    for cname, py in pairs.items():
        assert c[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert c[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])


@pytest.mark.parametrize("bad", [dict(slicing=3), dict(slicing=-1), dict(epoch_max_ms=-5), dict(epoch_max_ms=20),
                                 dict(max_slots=0), dict(memory_budget=0), dict(precision=7)])
def test_server_config_is_checked_before_any_device_work(built, bad):
    """vmc_server_create refuses an invalid configuration with VMC_ERR_INVALID_ARGUMENT
    before it selects a device, so these run without a GPU."""
    from valomc_gb300 import api
    with pytest.raises(api.VmcError) as e:
        api.Server(**bad)
    assert api.STATUS[e.value.status] == "VMC_ERR_INVALID_ARGUMENT"
