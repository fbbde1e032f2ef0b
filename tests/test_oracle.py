"""The CPU oracle, pinned against the reference engine (CPU only)."""
import numpy as np
import pytest

import oracle
from mrilab_gb300 import phantoms
from conftest import load_golden, rel_l2, signal

GOLDEN = ["gre2d_n16_tr4_seed1", "gre2d_n32_tr8_seed2", "gre2d_n64_full_seed0"]


@pytest.mark.parametrize("name", GOLDEN)
def test_port_matches_reference_cpu_engine_golden(built, name):
    """The single-precision port reproduces the reference CPU engine's
    signal (golden vectors recorded from DoScanAtCPU on the stand-ins)."""
    sc, g = load_golden(name)
    out = oracle.run_port(sc, "f32", threads=2)
    ref = g["ref_Sx"] + 1j * g["ref_Sy"]
    assert rel_l2(signal(out), ref) <= 1e-6
    np.testing.assert_allclose(out["Kx"], g["ref_Kx"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(out["Ky"], g["ref_Ky"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(out["Mz"], g["ref_Mz"], rtol=0, atol=2e-6)


@pytest.mark.parametrize("name", GOLDEN)
def test_fp64_oracle_is_stable_against_golden(built, name):
    """The all-FP64 oracle reproduces its recorded output on this machine,
    and the reference's own FP32 error against it is at its known level."""
    sc, g = load_golden(name)
    out = oracle.run_port(sc, "f64", threads=2)
    f64 = g["f64_Sx"] + 1j * g["f64_Sy"]
    assert rel_l2(signal(out), f64) <= 1e-12
    ref = g["ref_Sx"] + 1j * g["ref_Sy"]
    assert rel_l2(ref, f64) < 1e-3


def test_port_threads_do_not_change_result(built):
    sc = phantoms.config1_gre(seed=5, n=16, n_tr=3)
    a = oracle.run_port(sc, "f32", threads=1)
    b = oracle.run_port(sc, "f32", threads=4)
    assert rel_l2(signal(a), signal(b)) < 1e-12
    np.testing.assert_array_equal(a["Mz"], b["Mz"])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not mounted")
@pytest.mark.parametrize("seed,n,n_tr", [(7, 8, 2), (8, 12, 3)])
def test_port_matches_live_reference_cpu_engine(built, seed, n, n_tr):
    sc = phantoms.config1_gre(seed=seed, n=n, n_tr=n_tr)
    ref = oracle.run_ref_cpu(sc)
    out = oracle.run_port(sc, "f32")
    assert rel_l2(signal(out), signal(ref)) <= 1e-6


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not mounted")
@pytest.mark.parametrize("model,pools,seq", [("me", 2, "gre"), ("me", 3, "gre"), ("gm", 3, "sat"),
                                             ("mt", 2, "sat"), ("cest", 3, "sat"), ("cest", 4, "sat")])
@pytest.mark.parametrize("spins,coils", [(1, 1), (2, 2)])
def test_port_matches_reference_kernels(built, model, pools, seq, spins, coils):
    """Multi-pool models: the port agrees with the reference's own kernels
    (BlochKernel{ME,MT,CEST,GM}.cuh compiled as host C) at float-rounding
    level; a wrong exchange index or update order shows up as >1e-3."""
    sc = phantoms.small_multipool(model, seed=3, pools=pools, spins=spins, coils=coils, seq=seq)
    ref = oracle.run_ref_kernel(sc)
    out = oracle.run_port(sc, "f32")
    assert rel_l2(signal(out), signal(ref)) <= 2e-5
    np.testing.assert_allclose(out["Mz"], ref["Mz"], atol=1e-4)


def test_port_ext_callback_zeroes_transverse(built):
    """Ext events reach the callback with the state written back; an ideal
    spoiler plugin (DoExtPlugin case 6) zeroes Mxy."""
    sc = phantoms.config1_gre(seed=4, n=8, n_tr=3)
    lines, ntr = phantoms.gre_lines(n_read=8, n_pe=3, fov=(0.24,) * 3, tr_ms=20.0, te_ms=(5.0,), flip=30.0,
                                    rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0, ext_every=1)
    sc.VSeq = lines
    calls = []

    def cb(val, out):
        calls.append(val)
        out["Mx"][:] = 0
        out["My"][:] = 0
        return 0

    out = oracle.run_port(sc, "f64", ext_cb=cb)
    assert len(calls) == 3
    base = oracle.run_port(sc, "f64")
    assert rel_l2(signal(out), signal(base)) > 1e-3  # the spoiler changed later echoes


def test_port_history_matches_reference_cpu_engine_golden(built):
    """RunMode 1: the port's per-time-point state history and step times
    equal the reference CPU engine's (recorded from DoScanAtCPU)."""
    sc, g = load_golden("history_gre2d_n4_tr2_seed4")
    out = oracle.run_port(sc, "f32")
    for k in ("Mxs", "Mys", "Mzs"):
        np.testing.assert_allclose(out[k], g["ref_" + k], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(out["Muts"].ravel(), g["ref_Muts"].ravel())
    f64 = oracle.run_port(sc, "f64")
    for k in ("Mxs", "Mys", "Mzs"):
        np.testing.assert_allclose(f64[k], g["f64_" + k], rtol=0, atol=1e-12)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not mounted")
def test_port_history_matches_live_reference_cpu_engine(built):
    sc = phantoms.with_history(phantoms.config1_gre(seed=9, n=4, n_tr=3))
    ref = oracle.run_ref_cpu(sc)
    out = oracle.run_port(sc, "f32")
    for k in ("Mxs", "Mys", "Mzs"):
        np.testing.assert_allclose(out[k], ref[k], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(out["Muts"], ref["Muts"])
