"""Build MRiLab ``VSeq`` sequence lines for synthetic scans.

The scan engine consumes the pulse sequence as flat "lines"
(``VSeq.rfAmpLine ... flagsLine, utsLine, tsLine``).  Each TR's events are
merged as MRiLab's compiled PSD functions do
(``PSD/3D/GradientEcho/PSD_GRE3D/PSD_GRE3D.m:317-359``):

* ``ts`` = the TR's start/end pair, then the rf, Gz, Gy, Gx, ADC and Ext
  sample times, stably sorted, with a 6-row ``flags`` column per entry
  marking which channel the entry belongs to;
* ``uts`` = the unique times;
* each channel's values are sorted by their own times and the first and
  last value of every channel (except ``rfCoil``) are forced to zero;

and the TRs are concatenated (``Src/Main/DoPulseGen.m:43-111``), so time
restarts at 0 every TR and ``utsLine`` has a negative step at each TR
boundary.

Shapes are restated from MRiLab's sequence elements: Hamming-windowed sinc
RF with flip-angle scaling (``Macro/SeqElem/rf/rfSinc.m``,
``Src/Main/DoB1Scaling.m``), trapezoids sampled at their corner points
(``Macro/SeqElem/STD/StdTrap.m``) and ADC sample trains.

All times are built on an integer nanosecond grid and converted to seconds
once, so events that should coincide produce bit-identical doubles.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

GAMMA_H = 2 * np.pi * 42.5764e6  # rad/s/T, proton
NS = 1e-9


@dataclass
class TR:
    """Events of one TR, times in integer nanoseconds from the TR start."""

    duration_ns: int
    rf_t: List[int] = field(default_factory=list)
    rf_amp: List[float] = field(default_factory=list)
    rf_phase: List[float] = field(default_factory=list)
    rf_freq: List[float] = field(default_factory=list)
    rf_coil: List[float] = field(default_factory=list)
    g_t: Dict[str, List[int]] = field(default_factory=lambda: {"z": [], "y": [], "x": []})
    g_a: Dict[str, List[float]] = field(default_factory=lambda: {"z": [], "y": [], "x": []})
    adc_t: List[int] = field(default_factory=list)
    adc_v: List[float] = field(default_factory=list)
    ext_t: List[int] = field(default_factory=list)
    ext_v: List[float] = field(default_factory=list)

    # -- elements ---------------------------------------------------------
    def rf(self, t_ns, amp, phase=0.0, freq=0.0, coil=1):
        t_ns = np.asarray(t_ns, dtype=np.int64)
        n = len(t_ns)
        self.rf_t += list(t_ns)
        self.rf_amp += list(np.broadcast_to(np.asarray(amp, float), (n,)))
        self.rf_phase += list(np.broadcast_to(np.asarray(phase, float), (n,)))
        self.rf_freq += list(np.broadcast_to(np.asarray(freq, float), (n,)))
        self.rf_coil += [float(coil)] * n

    def grad(self, axis, t_ns, amp):
        t_ns = np.asarray(t_ns, dtype=np.int64)
        self.g_t[axis] += list(t_ns)
        self.g_a[axis] += list(np.broadcast_to(np.asarray(amp, float), (len(t_ns),)))

    def trap(self, axis, t0_ns, t1_ns, amp, ramp_ns=0):
        """Trapezoid sampled at its corners: 0 at t0, amp on [t0+ramp, t1-ramp],
        0 at t1 (``StdTrap`` with two samples per ramp and flat)."""
        if ramp_ns <= 0:
            ramp_ns = 1000
        pts = [t0_ns, t0_ns + ramp_ns, t1_ns - ramp_ns, t1_ns]
        self.grad(axis, pts, [0.0, amp, amp, 0.0])

    def adc(self, t_ns):
        t_ns = np.asarray(t_ns, dtype=np.int64)
        self.adc_t += list(t_ns)
        self.adc_v += [1.0] * len(t_ns)

    def ext(self, t_ns, value):
        self.ext_t.append(int(t_ns))
        self.ext_v.append(float(value))

    # -- PSD-style merge ----------------------------------------------------
    def lines(self) -> Dict[str, np.ndarray]:
        """One TR's lines exactly as a compiled MRiLab PSD returns them."""
        t0, t1 = 0, int(self.duration_ns)
        chans = [
            (self.rf_t, 0),
            (self.g_t["z"], 1),
            (self.g_t["y"], 2),
            (self.g_t["x"], 3),
            (self.adc_t, 4),
            (self.ext_t, 5),
        ]
        # every channel needs at least one entry (PSD_GRE3D.m:300-317)
        if not self.g_t["z"]:
            self.grad("z", [t0, t1], [0.0, 0.0])
        if not self.g_t["y"]:
            self.grad("y", [t0, t1], [0.0, 0.0])
        if not self.g_t["x"]:
            self.grad("x", [t0, t1], [0.0, 0.0])
        if not self.adc_t:
            self.adc_t += [t0, t1]
            self.adc_v += [0.0, 0.0]
        if not self.ext_t:
            self.ext_t += [t0, t1]
            self.ext_v += [0.0, 0.0]
        if not self.rf_t:
            self.rf([t0, t1], 0.0)
        chans = [
            (self.rf_t, 0),
            (self.g_t["z"], 1),
            (self.g_t["y"], 2),
            (self.g_t["x"], 3),
            (self.adc_t, 4),
            (self.ext_t, 5),
        ]
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

        rf_amp, rf_ph, rf_fr, rf_co = sort_by(self.rf_t, self.rf_amp, self.rf_phase, self.rf_freq, self.rf_coil)
        gz, = sort_by(self.g_t["z"], self.g_a["z"])
        gy, = sort_by(self.g_t["y"], self.g_a["y"])
        gx, = sort_by(self.g_t["x"], self.g_a["x"])
        adc, = sort_by(self.adc_t, self.adc_v)
        ext, = sort_by(self.ext_t, self.ext_v)
        for a in (rf_amp, rf_ph, rf_fr, gz, gy, gx, adc, ext):
            a[0] = 0.0
            a[-1] = 0.0
        return dict(
            rfAmp=rf_amp, rfPhase=rf_ph, rfFreq=rf_fr, rfCoil=rf_co,
            GzAmp=gz, GyAmp=gy, GxAmp=gx, ADC=adc, Ext=ext,
            uts=uts.astype(np.float64) * NS, ts=ts.astype(np.float64) * NS, flags=flags,
        )


def concat(trs: List[TR], multi_transmit: bool = False) -> Dict[str, np.ndarray]:
    """Concatenate TRs into VSeq lines (DoPulseGen.m:43-111,118-123)."""
    per = [tr.lines() for tr in trs]
    out = {}
    for key, name in [
        ("rfAmp", "rfAmpLine"), ("rfPhase", "rfPhaseLine"), ("rfFreq", "rfFreqLine"),
        ("rfCoil", "rfCoilLine"), ("GzAmp", "GzAmpLine"), ("GyAmp", "GyAmpLine"),
        ("GxAmp", "GxAmpLine"), ("ADC", "ADCLine"), ("Ext", "ExtLine"),
        ("uts", "utsLine"), ("ts", "tsLine"),
    ]:
        out[name] = np.concatenate([p[key] for p in per]).astype(np.float64)
    out["flagsLine"] = np.concatenate([p["flags"] for p in per], axis=1).astype(np.float64)
    if not multi_transmit:
        out["rfCoilLine"] = np.ones_like(out["rfCoilLine"])
    return out


# ---------------------------------------------------------------------------
# waveform elements
# ---------------------------------------------------------------------------

def sinc_rf(t0_ns: int, dur_ns: int, raster_ns: int, flip_deg: float, tbw: float,
            apod: str = "Hamming", gamma: float = GAMMA_H):
    """Sinc RF samples (times in ns, amplitudes in T) scaled to ``flip_deg``.

    Samples lie on ``raster_ns``; the amplitude is a windowed sinc with
    ``tbw`` zero crossings over the pulse; the first and last samples are 0.
    The gain makes the engine's minimum-|amplitude| sample-and-hold
    integrate to the requested flip angle (the rule of DoB1Scaling.m).
    """
    n = int(np.ceil(dur_ns / raster_ns)) + 1
    t_ns = t0_ns + np.round(np.linspace(0, dur_ns, n)).astype(np.int64)
    rel = (t_ns - t0_ns) * NS - dur_ns * NS / 2
    tw = dur_ns * NS / tbw
    a = {"Non": 0.0, "Hamming": 0.46, "Hanning": 0.5}[apod]
    with np.errstate(invalid="ignore", divide="ignore"):
        shape = (tw * np.sin(np.pi * rel / tw)) / (np.pi * rel)
    shape = shape * ((1 - a) + a * np.cos(np.pi * rel / (tbw * tw)))
    shape[np.isnan(shape)] = np.nanmax(shape)
    shape[0] = 0.0
    shape[-1] = 0.0
    # sample-and-hold keeps min(|a_i|, |a_i+1|) over each interval
    held = np.minimum(np.abs(shape[:-1]), np.abs(shape[1:]))
    gain = np.deg2rad(flip_deg) / (gamma * held.sum() * raster_ns * NS)
    return t_ns, shape * gain


def hard_rf(t0_ns: int, dur_ns: int, flip_deg: float, gamma: float = GAMMA_H):
    amp = np.deg2rad(flip_deg) / (gamma * dur_ns * NS)
    return np.array([t0_ns, t0_ns, t0_ns + dur_ns, t0_ns + dur_ns], dtype=np.int64), np.array([0.0, amp, amp, 0.0])
