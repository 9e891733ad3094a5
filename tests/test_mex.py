"""The MC3Dmex / MC2Dmex gateways, driven through the mex stand-in: argument checks and
error messages on any host; a full call on the GPU equals vmc_run on the same seed."""
import numpy as np
import pytest

from golden.make_golden import cases
from mexshim import driver
from valomc_gb300 import meshgen as mg


@pytest.fixture(scope="module")
def mex3(built):
    return driver.build(3)


@pytest.fixture(scope="module")
def mex2(built):
    return driver.build(2)


def test_wrong_arity_gives_the_syntax_message(mex3):
    p = mg.config_3d_phantom(nphoton=10, scale=0.1)
    args = driver.args_for(mex3, p)[:-1]
    out, err = driver.call(mex3, args)
    assert out is None and err.startswith("Syntax:")


def test_type_error(mex3):
    p = mg.config_3d_phantom(nphoton=10, scale=0.1)
    args = driver.args_for(mex3, p)
    args[0] = driver.mx(mex3, p.H.astype(np.float64), "double")  # H must be int64
    out, err = driver.call(mex3, args)
    assert err == "mxArray type error! Incorrect type received!\n"


def test_errorchecks_message(mex3, mex2):
    p = mg.config_3d_phantom(nphoton=10, scale=0.1)
    q = p.copy(g=p.g[:-1])
    out, err = driver.call(mex3, driver.args_for(mex3, q))
    assert err == ("Error in initializing MC3D: Scattering anisotropy array is not equal in size to the number "
                   "of elements\n")
    p2 = mg.config_2d_square(nphoton=10)
    p2.BCType[:] = ord("g")  # gaussian source without sigma
    p2.GaussianSigma = np.ones(3)
    out, err = driver.call(mex2, driver.args_for(mex2, p2))
    assert err == "Error in initializing MC2D: A gaussian light source exists but no sigma parameter was provided\n"


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [3, 2])
def test_gateway_matches_vmc_run(dim, mex3, mex2):
    import valomc_gb300 as V
    L = mex3 if dim == 3 else mex2
    p = cases()["phantom3d" if dim == 3 else "mixed2d"][0].copy(Nphoton=20000)
    outs, err = driver.call(L, driver.args_for(L, p, seed=99), nlhs=6)
    assert err is None, err
    vsol, bsol, ebsol, t, seed, hn = outs
    assert vsol.shape == (p.Ne, 1) and bsol.shape == (p.Nb, 1) and ebsol.shape == (p.Nb, 1)
    assert int(seed[0, 0]) == 99 and hn.shape == (p.Ne, dim + 1)
    r = V.run(p, seed=99, want_hn=True)
    np.testing.assert_allclose(vsol[:, 0].real, r.ER, rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(bsol[:, 0].real, r.EBR, rtol=1e-9, atol=1e-300)
    np.testing.assert_array_equal(hn, r.HN)


@pytest.mark.gpu
def test_gateway_waitbar_abort(mex3):
    """abort_photonMC set while the run is in progress ends it with the reference's warning."""
    p = mg.config_3d_phantom(nphoton=50_000_000, seed=3)
    mex3.shim_set_abort_after(1)
    outs, err = driver.call(mex3, driver.args_for(mex3, p, disable_pbar=0))
    mex3.shim_set_abort_after(-1)
    assert err is None
    assert "WARNING: RUN WAS ABORTED" in mex3.shim_log().decode()
    assert mex3.shim_eval_count() >= 3  # assignin, waitbar create, delete
