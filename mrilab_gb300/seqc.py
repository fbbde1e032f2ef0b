"""Python binding of the native sequence compiler (``include/mrl_seq.h``,
``mrl_seq_compile``): TR channels in, VSeq lines out.  Host code only (no
device needed)."""
from __future__ import annotations

import ctypes
from typing import Dict, List

import numpy as np

from . import engine

_d = ctypes.POINTER(ctypes.c_double)


class SeqTR(ctypes.Structure):
    _fields_ = [("t_start", ctypes.c_double), ("t_end", ctypes.c_double), ("n_rf", ctypes.c_int),
                ("rf_t", _d), ("rf_amp", _d), ("rf_phase", _d), ("rf_freq", _d), ("rf_coil", _d),
                ("n_gz", ctypes.c_int), ("n_gy", ctypes.c_int), ("n_gx", ctypes.c_int),
                ("gz_t", _d), ("gz", _d), ("gy_t", _d), ("gy", _d), ("gx_t", _d), ("gx", _d),
                ("n_adc", ctypes.c_int), ("n_ext", ctypes.c_int), ("adc_t", _d), ("adc", _d), ("ext_t", _d),
                ("ext", _d)]


class SeqOpts(ctypes.Structure):
    _fields_ = [("multi_transmit", ctypes.c_int), ("tx_coil_num", ctypes.c_int), ("master_tx_coil", ctypes.c_int),
                ("dummy_trs", ctypes.c_int), ("max_grad", ctypes.c_double), ("max_slew", ctypes.c_double),
                ("min_upd_rate", ctypes.c_double)]


_LINES = ("rf_amp", "rf_phase", "rf_freq", "rf_coil", "gz", "gy", "gx", "adc", "ext", "uts", "ts", "flags")


class SeqLines(ctypes.Structure):
    _fields_ = [(n, _d) for n in _LINES] + \
               [("cap_" + n, ctypes.c_longlong) for n in ("rf", "gz", "gy", "gx", "adc", "ext", "uts", "ts")] + \
               [("n_" + n, ctypes.c_longlong) for n in ("rf", "gz", "gy", "gx", "adc", "ext", "uts", "ts")]


class SeqError(ValueError):
    pass


def compile_lines(trs: List[dict], multi_transmit=False, dummy_trs=0, tx_coil_num=0, master_tx_coil=1,
                  max_grad=0.0, max_slew=0.0, min_upd_rate=0.0) -> Dict[str, np.ndarray]:
    """``trs``: per TR a dict with ``span`` (t_start, t_end) and the channels
    ``rf`` (t, amp, phase, freq, coil), ``gz``, ``gy``, ``gx``, ``adc``,
    ``ext`` (t, value), times in seconds.  Returns the VSeq lines."""
    lib = engine.library()
    lib.mrl_seq_compile.argtypes = [ctypes.POINTER(SeqTR), ctypes.c_int, ctypes.POINTER(SeqOpts),
                                    ctypes.POINTER(SeqLines)]
    lib.mrl_seq_compile.restype = ctypes.c_int
    keep = []
    arr = (SeqTR * len(trs))()
    for i, tr in enumerate(trs):
        r = arr[i]
        r.t_start, r.t_end = tr["span"]

        def p(a):
            a = np.ascontiguousarray(np.asarray(a, np.float64))
            keep.append(a)
            return a.ctypes.data_as(_d)

        rt, ra, rp, rfq, rc = tr["rf"]
        r.n_rf = len(rt)
        r.rf_t, r.rf_amp, r.rf_phase, r.rf_freq, r.rf_coil = p(rt), p(ra), p(rp), p(rfq), p(rc)
        for ch in ("gz", "gy", "gx", "adc", "ext"):
            t, v = tr[ch]
            setattr(r, "n_" + ch, len(t))
            setattr(r, ch + "_t", p(t))
            setattr(r, ch, p(v))
    o = SeqOpts(int(bool(multi_transmit)), int(tx_coil_num), int(master_tx_coil), int(dummy_trs), float(max_grad),
                float(max_slew), float(min_upd_rate))
    out = SeqLines()
    rc = lib.mrl_seq_compile(arr, len(trs), ctypes.byref(o), ctypes.byref(out))  # counts
    if rc != 0 and b"capacity" not in lib.mrl_last_error():
        raise SeqError(lib.mrl_last_error().decode())
    n = {k: int(getattr(out, "n_" + k)) for k in ("rf", "gz", "gy", "gx", "adc", "ext", "uts", "ts")}
    bufs = {k: np.zeros(n[{"rf_amp": "rf", "rf_phase": "rf", "rf_freq": "rf", "rf_coil": "rf"}.get(k, k)]
                        if k != "flags" else 6 * n["ts"]) for k in _LINES}
    for k in _LINES:
        setattr(out, k, bufs[k].ctypes.data_as(_d))
    for k, v in n.items():
        setattr(out, "cap_" + k, v)
    rc = lib.mrl_seq_compile(arr, len(trs), ctypes.byref(o), ctypes.byref(out))
    if rc != 0:
        raise SeqError(lib.mrl_last_error().decode())
    return {"rfAmpLine": bufs["rf_amp"], "rfPhaseLine": bufs["rf_phase"], "rfFreqLine": bufs["rf_freq"],
            "rfCoilLine": bufs["rf_coil"], "GzAmpLine": bufs["gz"], "GyAmpLine": bufs["gy"], "GxAmpLine": bufs["gx"],
            "ADCLine": bufs["adc"], "ExtLine": bufs["ext"], "utsLine": bufs["uts"], "tsLine": bufs["ts"],
            "flagsLine": bufs["flags"].reshape(n["ts"], 6).T.copy()}
