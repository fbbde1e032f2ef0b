"""Local SAR engine (mrl_sar, include/mrl_sar.h): the reference's SAR engine
DoCalSARAtCPU (Lib/src/engine/CPUEngine/DoCalSARAtCPU.cpp) on the GPU.

CPU tests pin the oracle (oracle/sar.py) to golden vectors recorded from the
reference engine compiled from its source, and check the boundary's argument
errors; GPU tests compare the engine with both."""
import os

import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_l2
from mrilab_gb300 import mexsim, phantoms
from mrilab_gb300 import sar as msar
from oracle import sar as osar

GOLDEN = ["sar_tx1_n6_seed2", "sar_tx2_n8_seed1", "sar_tx3_n6_seed3"]
# accurate numerics (segments folded into FP64 Tx x Tx matrices) against the
# all-FP64 oracle: relative L2 over every sample of every voxel
TOL_F64 = 1e-6


def _cursor(o):
    return [o["SARi"], o["utsi"], o["rfi"], o["TRCount"]]


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_matches_reference_sar_engine(name):
    """The single-precision restatement reproduces the reference engine bit
    for bit (same rounding order), and the walk's cursor and times."""
    sc, g = load_golden(name)
    p = osar.run_sar_port(sc, "f32")
    np.testing.assert_array_equal(p["SAR"].astype(np.float32), g["ref_SAR"])
    np.testing.assert_array_equal(p["SARacc"].astype(np.float32), g["ref_SARacc"])
    np.testing.assert_array_equal(p["Muts"], g["ref_Muts"])
    np.testing.assert_array_equal(p["tRealSample"], g["ref_tRealSample"])
    assert _cursor(p) == list(g["ref_cursor"])
    p64 = osar.run_sar_port(sc, "f64")
    assert rel_l2(p64["SAR"], g["f64_SAR"]) <= 1e-14


@pytest.mark.skipif(not osar.ref_sar_available(), reason="reference tree not built")
def test_oracle_matches_live_reference_engine_with_stops():
    """Sample times that stop the walk early (the engine returns once every
    sample is taken) and a case with one sample at the start."""
    for kw in (dict(seed=7, n=5, nz=1, tx_coils=2, n_tr=3, sample_fracs=(0.0, 0.25)),
               dict(seed=8, n=4, nz=2, tx_coils=1, n_tr=2, sample_fracs=(0.0,))):
        sc = phantoms.sar_case(**kw)
        r = osar.run_ref_sar(sc)
        p = osar.run_sar_port(sc, "f32")
        np.testing.assert_array_equal(p["SAR"], r["SAR"])
        np.testing.assert_array_equal(p["SARacc"], r["SARacc"])
        assert _cursor(p) == _cursor(r)


def test_sar_argument_errors_are_status_codes(built):
    import ctypes

    from mrilab_gb300 import engine

    sc = phantoms.sar_case(seed=1, n=4, nz=1, tx_coils=2, n_tr=1)
    hs = msar.HostSar(sc)
    hs.args.abi_version = 999
    assert msar._lib().mrl_sar(ctypes.byref(hs.args)) == -1
    hs = msar.HostSar(sc)
    hs.args.tx_num = 9
    assert msar._lib().mrl_sar(ctypes.byref(hs.args)) == -6
    hs = msar.HostSar(sc)
    hs.args.econ = ctypes.cast(None, type(hs.args.econ))
    assert msar._lib().mrl_sar(ctypes.byref(hs.args)) == -1
    assert b"missing" in engine.library().mrl_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN)
def test_sar_reference_numerics_equal_reference_engine(built, name):
    """MRL_NUMERICS_REFERENCE: the reference's operation order on the GPU,
    bit for bit equal to the reference engine's VSig.SAR and VVar.SAR."""
    sc, g = load_golden(name)
    out = msar.sar(sc, numerics="reference")
    np.testing.assert_array_equal(out["SAR"], g["ref_SAR"])
    np.testing.assert_array_equal(out["SARacc"], g["ref_SARacc"])
    np.testing.assert_array_equal(out["Muts"], g["ref_Muts"])
    np.testing.assert_array_equal(out["tRealSample"], g["ref_tRealSample"])
    assert _cursor(out) == list(g["ref_cursor"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN)
def test_sar_accurate_numerics_vs_fp64_oracle(built, name):
    sc, g = load_golden(name)
    out = msar.sar(sc)
    e64 = rel_l2(out["SAR"], g["f64_SAR"])
    eacc = rel_l2(out["SARacc"], g["f64_SARacc"])
    print(f"{name}: accurate SAR vs FP64 {e64:.2e} (accumulator {eacc:.2e}); reference engine vs FP64 "
          f"{rel_l2(g['ref_SAR'], g['f64_SAR']):.2e}")
    assert e64 <= TOL_F64 and eacc <= TOL_F64
    assert _cursor(out) == list(g["ref_cursor"])


@pytest.mark.gpu
def test_sar_larger_case_vs_fp64_oracle(built):
    """A 48 x 48 x 4 object, 4 Tx coils, 6 TRs, samples every sixth of the
    sequence: both numerics against the oracle."""
    sc = phantoms.sar_case(seed=11, n=48, nz=4, tx_coils=4, n_tr=6,
                           sample_fracs=tuple(np.linspace(0.0, 1.0, 7)))
    p64 = osar.run_sar_port(sc, "f64")
    p32 = osar.run_sar_port(sc, "f32")
    acc = msar.sar(sc)
    ref = msar.sar(sc, numerics="reference")
    assert rel_l2(acc["SAR"], p64["SAR"]) <= TOL_F64
    np.testing.assert_array_equal(ref["SAR"], p32["SAR"].astype(np.float32))


@pytest.mark.gpu
def test_sar_mex_wrapper_path(built):
    """DoCalSARAtGPU through the mex stand-in: globals in, globals out."""
    sc, g = load_golden("sar_tx2_n8_seed1")
    ms = mexsim.MexSession()
    for k, v in sc.structs().items():
        if v:
            ms.set_global(k, v)
    ms.set_field("VCtl", "Numerics", np.float64(1.0))
    ms.call(os.path.join(ROOT, "mrilab_gb300", "mex", "DoCalSARAtGPU.so"))
    np.testing.assert_array_equal(ms.get("VSig", "SAR").ravel(order="F"), g["ref_SAR"])
    assert int(ms.get("VVar", "SARi").ravel()[0]) == int(g["ref_cursor"][0])
