"""Python binding of the local-SAR engine's C ABI (``include/mrl_sar.h``).

``sar(sc, ...)`` runs the SAR accumulation of a ``phantoms.sar_case`` scan on
the GPU through ``mrl_sar`` -- the call the mex wrapper ``DoCalSARAtGPU``
makes in place of the reference's ``DoCalSARAtCPU``
(``Lib/src/engine/CPUEngine/DoCalSARAtCPU.cpp:85``) -- with the globals
passed as host arrays.  No CPU fallback: a missing library or GPU raises.
"""
from __future__ import annotations

import ctypes
from typing import Dict

import numpy as np

from . import engine

_d = ctypes.POINTER(ctypes.c_double)
_f = ctypes.POINTER(ctypes.c_float)
_i = ctypes.POINTER(ctypes.c_int)


class SarArgs(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_int), ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("nz", ctypes.c_int),
                ("econ", _f), ("tx_num", ctypes.c_int), ("tx_e1x", _f), ("tx_e1y", _f), ("tx_e1z", _f),
                ("tr_num", ctypes.c_int), ("gpu_index", ctypes.c_int), ("numerics", ctypes.c_int),
                ("seq", engine.Sequence), ("var", engine.State), ("sar_acc", _f), ("sari", _i), ("sar", _f),
                ("muts", _d), ("t_sample", _d), ("t_real_sample", _d), ("n_sample", ctypes.c_int)]


def _lib():
    lib = engine.library()
    lib.mrl_sar.argtypes = [ctypes.POINTER(SarArgs)]
    lib.mrl_sar.restype = ctypes.c_int
    return lib


class HostSar:
    """Column-major host copies of a SAR case's arrays, bound into SarArgs."""

    def __init__(self, sc, numerics: str = "accurate", gpu_index: int = 0):
        o, c, ctl, q, v, sig = sc.VObj, sc.VCoi, sc.VCtl, sc.VSeq, sc.VVar, sc.VSig
        K = self.keep = {}
        p = lambda a, t: a.ctypes.data_as(t)
        f32 = lambda k, a: K.setdefault(k, np.asarray(a, np.float32).flatten(order="F"))
        f64 = lambda k, a: K.setdefault(k, np.asarray(a, np.float64).flatten(order="F"))
        i32 = lambda k, a: K.setdefault(k, np.asarray(a, np.int32).flatten(order="F"))
        a = SarArgs()
        a.abi_version = engine.ABI_VERSION
        a.ny, a.nx, a.nz = (o["MassDen"].shape + (1, 1))[:3]
        a.econ = p(f32("econ", o["ECon"]), _f)
        a.tx_num = int(c["TxCoilNum"])
        a.tx_e1x, a.tx_e1y, a.tx_e1z = (p(f32("e1x", c["TxE1x"]), _f), p(f32("e1y", c["TxE1y"]), _f),
                                        p(f32("e1z", c["TxE1z"]), _f))
        a.tr_num = int(ctl["TRNum"])
        a.gpu_index = gpu_index
        a.numerics = engine.NUMERICS[numerics]
        sq = a.seq
        for fld, key in [("uts", "utsLine"), ("ts", "tsLine"), ("rf_amp", "rfAmpLine"), ("rf_phase", "rfPhaseLine"),
                         ("rf_freq", "rfFreqLine"), ("rf_coil", "rfCoilLine"), ("ext", "ExtLine"),
                         ("flags", "flagsLine")]:
            setattr(sq, fld, p(f64("seq_" + fld, q[key]), _d))
        sq.n_uts, sq.n_ts, sq.n_rf, sq.n_ext = (q["utsLine"].size, q["tsLine"].size, q["rfAmpLine"].size,
                                                q["ExtLine"].size)
        st = a.var
        for fld, key in [("t", "t"), ("dt", "dt"), ("rf_amp", "rfAmp"), ("rf_phase", "rfPhase"),
                         ("rf_freq", "rfFreq"), ("rf_coil", "rfCoil"), ("ext", "Ext")]:
            setattr(st, fld, p(f64("var_" + fld, v[key]), _d))
        for fld, key in [("utsi", "utsi"), ("rfi", "rfi"), ("exti", "Exti"), ("tr_count", "TRCount")]:
            setattr(st, fld, p(i32("var_" + fld, v[key]), _i))
        a.sar_acc = p(f32("sar_acc", v["SAR"]), _f)
        a.sari = p(i32("sari", v["SARi"]), _i)
        a.sar = p(f32("sar", sig["SAR"]), _f)
        a.muts = p(f64("muts", sig["Muts"]), _d)
        a.t_sample = p(f64("t_sample", sig["tSample"]), _d)
        a.t_real_sample = p(f64("t_real", sig["tRealSample"]), _d)
        a.n_sample = int(np.size(sig["tSample"]))
        self.args = a

    def outputs(self) -> Dict[str, np.ndarray]:
        K = self.keep
        return dict(SAR=K["sar"], SARacc=K["sar_acc"], Muts=K["muts"], tRealSample=K["t_real"],
                    SARi=int(K["sari"][0]), utsi=int(K["var_utsi"][0]), rfi=int(K["var_rfi"][0]),
                    TRCount=int(K["var_tr_count"][0]), rfAmp=K["var_rf_amp"].copy())


def sar(sc, numerics: str = "accurate", gpu_index: int = 0) -> Dict[str, np.ndarray]:
    """Run mrl_sar on a copy of the case's arrays; returns VSig.SAR
    ([n_sample][V] flattened), VVar.SAR (``SARacc``, [3][V]), VSig.Muts,
    VSig.tRealSample and the VVar cursors."""
    hs = HostSar(sc, numerics=numerics, gpu_index=gpu_index)
    rc = _lib().mrl_sar(ctypes.byref(hs.args))
    if rc != 0:
        raise engine.ScanError(rc, engine.library().mrl_last_error().decode())
    return hs.outputs()
