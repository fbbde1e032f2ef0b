"""Reconstruction (include/mrl_recon.h): the Cartesian / EPI transform of
DoCartRecon.m / DoEPIRecon.m (mrl_recon_cart) and the gridding mex
DoGridding (mrl_grid2d) on the GPU.

CPU tests pin the gridding oracle to golden vectors recorded from the
reference mex compiled from its source; GPU tests compare the engine with the
oracles (FP64 throughout: relative L2 within 1e-12)."""
import ast
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from mrilab_gb300 import mexsim
from mrilab_gb300 import recon as mrec
from oracle import recon as orc

GRID = ["grid2d_n400_g32_seed0", "grid2d_n900_g48_seed1"]
TOL = 1e-12


def _grid_case(name):
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden",
                                                                              "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    z = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    return mg.grid_inputs(**ast.literal_eval(str(z["kwargs"]))), z


@pytest.mark.parametrize("name", GRID)
def test_grid_oracle_matches_reference_mex(name):
    args, z = _grid_case(name)
    gx, gy = orc.grid2d_port(*args)
    np.testing.assert_array_equal(gx, z["ref_gx"])
    np.testing.assert_array_equal(gy, z["ref_gy"])


def test_cart_oracle_inverts_a_centred_fft():
    """The restated transform undoes the forward transform it inverts: a
    k-space made as fftshift(fftn(fftshift(image))) (even sizes) comes back as
    the image, with the readout point MATLAB drops appended and zero."""
    rng = np.random.default_rng(3)
    img = rng.normal(size=(16, 12, 4)) + 1j * rng.normal(size=(16, 12, 4))
    k = np.fft.fftshift(np.fft.fftn(np.fft.fftshift(img)))  # [phase, readout, slice] after the permute
    kr = np.concatenate([k.transpose(1, 0, 2), np.zeros((1, 16, 4))], 0)  # [readout + 1, lines, slices]
    out = orc.cart_recon(kr.real.ravel(order="F"), kr.imag.ravel(order="F"), 13, 16, 4, 1, 1)
    np.testing.assert_allclose(out[..., 0, 0], img, atol=1e-12)


CASES = {
    "cart2d": dict(res_freq=33, lines=32, slices=1, rx=2, pools=1),
    "cart3d_multiecho_pools": dict(res_freq=17, lines=12, slices=6, rx=3, pools=2, echoes=3),
    "cart_zero_filled": dict(res_freq=17, lines=10, slices=3, rx=2, pools=1, zf=(32, 16, 2)),
    "cart_readout_first_odd": dict(res_freq=16, lines=9, slices=5, rx=1, pools=3, readout_first=True),
    "epi": dict(res_freq=33, lines=4, slices=2, rx=2, pools=2, epi_etl=8),
    "epi_zero_filled_readout_first": dict(res_freq=17, lines=2, slices=1, rx=4, pools=1, epi_etl=6, zf=(24, 16, 1),
                                          readout_first=True),
}


def _signal(kw, seed):
    rows = kw["res_freq"] * (kw.get("epi_etl") or kw.get("echoes", 1))
    n = rows * kw["lines"] * kw["slices"] * kw["rx"] * kw["pools"]
    rng = np.random.default_rng(seed)
    return rng.normal(size=n), rng.normal(size=n)


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_cart_recon_matches_oracle(built, case):
    kw = CASES[case]
    sx, sy = _signal(kw, 7)
    ref = orc.cart_recon(sx, sy, **kw)
    out = mrec.cart_recon(sx, sy, **kw)
    got = out["Real"] + 1j * out["Imag"]
    assert got.shape == ref.shape
    err = rel_l2(got, ref)
    print(f"{case}: {err:.2e}")
    assert err <= TOL
    np.testing.assert_allclose(out["Mag"], np.abs(ref), rtol=0, atol=1e-12 * np.abs(ref).max())
    m = np.abs(ref) > 1e-9 * np.abs(ref).max()
    np.testing.assert_allclose(out["Phase"][m], np.angle(ref)[m], rtol=0, atol=1e-9)


@pytest.mark.gpu
def test_cart_recon_of_a_scan_shows_the_phantom(built):
    """A 32 x 32 GRE scanned on the GPU and reconstructed there: the image's
    magnitude follows the phantom's proton density (disk inside, empty
    outside)."""
    from mrilab_gb300 import engine, phantoms

    sc = phantoms.config1_gre(seed=5, n=32)
    out = engine.scan(sc)
    img = mrec.cart_recon(out["Sx"], out["Sy"], res_freq=32, lines=32, slices=1, rx=1, pools=1)["Mag"][..., 0, 0, 0]
    ref = orc.cart_recon(out["Sx"], out["Sy"], res_freq=32, lines=32, slices=1, rx=1, pools=1)[..., 0, 0, 0]
    assert rel_l2(img, np.abs(ref)) <= TOL
    rho = sc.VObj["Rho"][..., 0]
    inside = img[8:24, 8:24].mean()
    corner = img[:3, :3].mean()
    assert inside > 3 * corner and rho[16, 16] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", GRID)
def test_grid2d_matches_reference_mex(built, name):
    args, z = _grid_case(name)
    gx, gy = mrec.grid2d(*args)
    assert rel_l2(gx, z["ref_gx"]) <= TOL and rel_l2(gy, z["ref_gy"]) <= TOL


@pytest.mark.gpu
def test_recon_mex_wrappers(built):
    """DoGridding and DoCartReconGPU through the mex stand-in, arguments in
    and arrays out as MATLAB calls them."""
    ms = mexsim.MexSession()
    args, z = _grid_case(GRID[0])
    a, b = ms.call_args(os.path.join(ROOT, "mrilab_gb300", "mex", "DoGridding.so"),
                        [np.asarray(v, np.float64) for v in args[:6]] + [np.float64(args[6]), np.float64(args[7])], 2)
    assert rel_l2(a.ravel(order="F"), z["ref_gx"]) <= TOL
    kw = CASES["cart3d_multiecho_pools"]
    sx, sy = _signal(kw, 9)
    dims = np.array([kw["res_freq"], kw["lines"], kw["slices"], kw["rx"], kw["pools"], kw["echoes"], 0, 0, 0, 0, 0],
                    np.float64)
    re, im, mag, ph = ms.call_args(os.path.join(ROOT, "mrilab_gb300", "mex", "DoCartReconGPU.so"), [sx, sy, dims], 4)
    ref = orc.cart_recon(sx, sy, **kw)
    assert rel_l2(re + 1j * im, ref.reshape(re.shape, order="F")) <= TOL


def test_recon_argument_errors_are_status_codes(built):
    from mrilab_gb300 import engine

    with pytest.raises(engine.ScanError) as e:
        mrec.cart_recon(np.zeros(10), np.zeros(10), res_freq=1, lines=1, slices=1, rx=1, pools=1)
    assert e.value.status == -1
    kw = dict(res_freq=16, lines=8, slices=1, rx=1, pools=1, zf=(32, 16, 1))  # 15 readout points: odd split
    sx, sy = _signal(kw, 1)
    with pytest.raises(engine.ScanError) as e:
        mrec.cart_recon(sx, sy, **kw)
    assert e.value.status == -1
