"""CPU oracle of the sequence compiler -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` may use this module, as the reference results; the product
never imports it.  A numpy restatement of how MRiLab turns one TR's
sequence-element samples into its lines (the merge every compiled PSD ends
with, ``Src/Main/DoWriteXML2m.m:263-333``: the span's end points and every
channel's sample times on one stably sorted time line with a 6-row flag
column per entry, the unique times, each channel sorted by its own times,
the first and last value of every channel but rfCoil zeroed) and how
``Src/Main/DoPulseGen.m:20-123`` concatenates the TRs (dummy TRs with their
gradients and ADC zeroed; rfCoil forced to 1 without multi-transmit).  It
works on integer nanoseconds, independently of the native compiler's
doubles; MATLAB is absent here, so this restatement is the pin.
"""
from __future__ import annotations

from typing import Dict, List

import numpy as np

NS = 1e-9


def tr_lines(tr) -> Dict[str, np.ndarray]:
    """One ``mrilab_gb300.seq.TR``'s lines (after ``tr.channels()`` filled
    its empty channels)."""
    tr.channels()
    t0, t1 = 0, int(tr.duration_ns)
    chans = [(tr.rf_t, 0), (tr.g_t["z"], 1), (tr.g_t["y"], 2), (tr.g_t["x"], 3), (tr.adc_t, 4), (tr.ext_t, 5)]
    ts = [t0, t1]
    flags = [np.zeros(6), np.zeros(6)]
    for times, row in chans:
        for t in times:
            ts.append(int(t))
            f = np.zeros(6)
            f[row] = 1
            flags.append(f)
    ts = np.asarray(ts, dtype=np.int64) - t0
    order = np.argsort(ts, kind="stable")
    ts = ts[order]
    flags = np.stack(flags, axis=1)[:, order]
    uts = np.unique(ts)

    def sort_by(times, *vals):
        o = np.argsort(np.asarray(times, dtype=np.int64), kind="stable")
        return [np.asarray(v, dtype=float)[o] for v in vals]

    rf_amp, rf_ph, rf_fr, rf_co = sort_by(tr.rf_t, tr.rf_amp, tr.rf_phase, tr.rf_freq, tr.rf_coil)
    gz, = sort_by(tr.g_t["z"], tr.g_a["z"])
    gy, = sort_by(tr.g_t["y"], tr.g_a["y"])
    gx, = sort_by(tr.g_t["x"], tr.g_a["x"])
    adc, = sort_by(tr.adc_t, tr.adc_v)
    ext, = sort_by(tr.ext_t, tr.ext_v)
    for a in (rf_amp, rf_ph, rf_fr, gz, gy, gx, adc, ext):
        a[0] = 0.0
        a[-1] = 0.0
    return dict(rfAmp=rf_amp, rfPhase=rf_ph, rfFreq=rf_fr, rfCoil=rf_co, GzAmp=gz, GyAmp=gy, GxAmp=gx, ADC=adc,
                Ext=ext, uts=uts.astype(np.float64) * NS, ts=ts.astype(np.float64) * NS, flags=flags)


def concat(trs: List, multi_transmit: bool = False, dummy_trs: int = 0) -> Dict[str, np.ndarray]:
    per = [tr_lines(tr) for tr in trs]
    out = {}
    for key, name in [("rfAmp", "rfAmpLine"), ("rfPhase", "rfPhaseLine"), ("rfFreq", "rfFreqLine"),
                      ("rfCoil", "rfCoilLine"), ("GzAmp", "GzAmpLine"), ("GyAmp", "GyAmpLine"),
                      ("GxAmp", "GxAmpLine"), ("ADC", "ADCLine"), ("Ext", "ExtLine"), ("uts", "utsLine"),
                      ("ts", "tsLine")]:
        out[name] = np.concatenate([p[key] for p in per]).astype(np.float64)
    out["flagsLine"] = np.concatenate([p["flags"] for p in per], axis=1).astype(np.float64)
    if dummy_trs:
        # the dummies' gradients and ADC are zeroed (every line so far, after each dummy TR)
        for name, key in (("GzAmpLine", "GzAmp"), ("GyAmpLine", "GyAmp"), ("GxAmpLine", "GxAmp"), ("ADCLine", "ADC")):
            n = sum(per[i][key].size for i in range(min(dummy_trs, len(per))))
            out[name][:n] = 0.0
    if not multi_transmit:
        out["rfCoilLine"] = np.ones_like(out["rfCoilLine"])
    return out
