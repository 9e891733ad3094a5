"""The drop-in MC3D / MC2D executables on any host: usage, exit codes, the text reader's
tag handling and the ErrorChecks messages, compared with the reference executables where
they were built (oracle/_ref/)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from golden.make_golden import cases
from valomc_gb300 import build as vbuild
from valomc_gb300 import meshgen as mg


def exe(dim):
    return os.path.join(vbuild.BUILD, f"MC{dim}D")


def run(cmd):
    return subprocess.run(cmd, capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("dim", [3, 2])
def test_usage(built, dim):
    r = run([exe(dim)])
    assert r.returncode == 0 and "Use syntax:" in r.stdout


def test_missing_input_file(built):
    r = run([exe(3), "/nonexistent/in.txt", "/tmp/out.txt"])
    assert r.returncode == 1 and "Error while loading!" in r.stdout


def message(stdout):
    return [ln for ln in stdout.splitlines() if ln.startswith("MC Initialization failed!")]


@pytest.mark.parametrize("case,mutate", [
    ("phantom3d", lambda p: p.copy(BCn=None)),                                  # MISSING_BCN
    ("phantom3d", lambda p: p.copy(BCType=np.full(p.Nb, ord("a"), np.uint8))),  # NO_LIGHTSOURCE
    ("mixed2d", lambda p: p.copy(GaussianSigma=None)),                          # NO_GAUSSIAN_SIGMA
    ("square2d", lambda p: p.copy(BH=p.BH[1:], BCType=p.BCType[1:], BCn=p.BCn[1:])),  # MISSING_BOUNDARY
])
def test_initialisation_errors_print_the_reference_message(built, case, mutate):
    p = mutate(cases()[case][0])
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
        mg.write_input(fin, p)
        r = run([exe(p.dim), fin, fout])
        assert r.returncode == 1
        ours = message(r.stdout)
        assert len(ours) == 1
        if oracle.have_reference_binaries():
            ref = run([os.path.join(oracle.REF_DIR, f"MC{p.dim}D"), fin, fout])
            assert ref.returncode == 1
            assert message(ref.stdout) == ours


def test_misnamed_optional_tag_is_skipped_like_the_reference(built):
    """ValoMC.m writes 'BCLightDirectionType' where the 3D reader expects 'BCLDirType':
    the block is not read and, because tags are order-sensitive, neither is anything after
    it -- so the missing BCIntensity row count stays 0 and no size error follows."""
    p = cases()["phantom3d"][0].copy(BCLightDirectionType=np.full(cases()["phantom3d"][0].Nb, ord("n"), np.uint8))
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.txt"), os.path.join(td, "out.txt")
        mg.write_input(fin, p, dirtype_tag="BCLightDirectionType")
        r = run([exe(3), fin, fout])
        assert "BCIntensity" not in r.stdout and "BCLDirType" not in r.stdout
        assert "BCn" in r.stdout
