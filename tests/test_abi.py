"""The C-ABI boundary: the library loads and exports what include/*.h
declares; argument errors come back as status codes (CPU only)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from mrilab_gb300 import engine, phantoms


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(mrl_[a-z0-9_]+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(engine.LIB_PATH)
    names = declared_functions()
    assert "mrl_scan" in names and "mrl_status_string" in names
    for n in names:
        assert hasattr(lib, n), n


@pytest.mark.parametrize("wrapper", ["DoScanAtGPU", "DoMEScanAtGPU", "DoMTScanAtGPU", "DoCESTScanAtGPU", "DoGridding", "DoCartReconGPU",
                                     "DoGMScanAtGPU", "DoCalSARAtGPU"])
def test_mex_wrappers_export_mexfunction(built, wrapper):
    so = os.path.join(ROOT, "mrilab_gb300", "mex", wrapper + ".so")
    lib = ctypes.CDLL(so)
    assert hasattr(lib, "mexFunction")


def test_status_strings(built):
    lib = engine.library()
    for code in range(0, -8, -1):
        assert lib.mrl_status_string(code)
    assert lib.mrl_status_string(12345) == b"unknown status"


def _small_args():
    sc = phantoms.config1_gre(seed=0, n=8, n_tr=1)
    return engine.HostScan(sc, numerics="reference")


def test_abi_version_mismatch_is_rejected(built):
    hs = _small_args()
    hs.args.abi_version = 999
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs)
    assert e.value.status == -1


def test_bad_sizes_are_rejected(built):
    hs = _small_args()
    hs.args.obj.type_num = 0
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs)
    assert e.value.status == -1
    hs = _small_args()
    hs.args.seq.n_ts = 0
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs)
    assert e.value.status == -1
    hs = _small_args()
    hs.args.model = 17
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs)
    assert e.value.status == -1


def test_unsupported_sizes_are_reported(built):
    hs = _small_args()
    hs.args.ctl.run_mode = 1
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs)
    assert e.value.status == -6


def test_mt_model_needs_two_pools(built):
    sc = phantoms.small_multipool("mt", seed=1, n=4, pools=2, n_tr=1)
    hs = engine.HostScan(sc)
    hs.args.obj.type_num = 3
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs)
    assert e.value.status == -1


def test_no_cpu_fallback_without_gpu(built):
    """On a machine without a usable GPU the engine fails loudly."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    hs = _small_args()
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs)
    assert e.value.status in (-7, -2)


def test_batch_argument_errors_are_status_codes(built):
    lib = engine.library()
    ptr = ctypes.c_void_p()
    lib.mrl_batch_create.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    assert lib.mrl_batch_create(None, 0, ctypes.byref(ptr)) == -1
    hs = engine.HostScan(phantoms.config1_gre(seed=0, n=8, n_tr=1), numerics="reference")
    arr = (ctypes.POINTER(engine.ScanArgs) * 1)(ctypes.pointer(hs.args))
    assert lib.mrl_batch_create(ctypes.cast(arr, ctypes.c_void_p), 1, ctypes.byref(ptr)) == -6
    assert b"ACCURATE" in lib.mrl_last_error()


def test_adjoint_plan_argument_errors_are_status_codes(built):
    """The adjoint plan calls reject NULL plans and outputs with
    MRL_ERR_ARG before touching a device."""
    lib = engine.library()
    buf = (ctypes.c_longlong * 6)()
    for name in ("mrl_adjoint_plan_checkpoints", "mrl_adjoint_plan_work"):
        fn = getattr(lib, name)
        fn.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]
        assert fn(None, buf) == -1
    lib.mrl_adjoint_plan_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    assert lib.mrl_adjoint_plan_forward(None, None) == -1
    lib.mrl_adjoint_plan_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    ptr = ctypes.c_void_p()
    assert lib.mrl_adjoint_plan_create(None, ctypes.byref(ptr)) == -1


def test_adjoint_without_gpu_fails_loudly(built):
    """No CPU fallback for the gradients either."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sc = phantoms.small_multipool("gm", seed=3, n=4, pools=3, spins=1, coils=2, n_tr=1, seq="sat")
    with pytest.raises(engine.ScanError) as e:
        engine.adjoint(sc, np.zeros(1), np.zeros(1))
    assert e.value.status in (-7, -2)


def test_inplace_host_scan_aliases_the_callers_arrays(built):
    """HostScan(inplace=True) binds the caller's own state and signal arrays
    (the engine writes them, as the mex layer writes the MATLAB globals);
    the default binds copies and leaves the caller's arrays alone."""
    sc = phantoms.small_multipool("me", seed=3, n=4, pools=2, spins=2, coils=2, n_tr=1)
    hs = engine.HostScan(sc, inplace=True)
    for key, arr in (("mx", sc.VObj["Mx"]), ("mz", sc.VObj["Mz"]), ("sx", sc.VSig["Sx"]), ("sy", sc.VSig["Sy"])):
        assert np.shares_memory(hs.keep[key], arr), key
    hc = engine.HostScan(sc)
    for key, arr in (("mx", sc.VObj["Mx"]), ("sx", sc.VSig["Sx"])):
        assert not np.shares_memory(hc.keep[key], arr), key
    # read-only inputs alias the caller's arrays either way
    assert np.shares_memory(hc.keep["rho"], sc.VObj["Rho"])
