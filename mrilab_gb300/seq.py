"""Build MRiLab ``VSeq`` sequence lines for synthetic scans.

The scan engine consumes the pulse sequence as flat "lines"
(``VSeq.rfAmpLine ... flagsLine, utsLine, tsLine``).  ``TR`` collects one
TR's sequence-element samples; ``concat`` hands them to the native sequence
compiler (``mrl_seq_compile``), which merges each TR as MRiLab's compiled
PSD functions do and concatenates the TRs (``Src/Main/DoPulseGen.m``), so
time restarts at 0 every TR and ``utsLine`` has a negative step at each TR
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

    # -- channels for the compiler -------------------------------------------
    def channels(self):
        """The TR's channels as the sequence compiler takes them, times in
        seconds: every channel gets at least one sample (a zero at the TR's
        start and end), as MRiLab's PSDs require (DoWriteXML2m.m:263-286)."""
        t0, t1 = 0, int(self.duration_ns)
        for axis in ("z", "y", "x"):
            if not self.g_t[axis]:
                self.grad(axis, [t0, t1], [0.0, 0.0])
        if not self.adc_t:
            self.adc_t += [t0, t1]
            self.adc_v += [0.0, 0.0]
        if not self.ext_t:
            self.ext_t += [t0, t1]
            self.ext_v += [0.0, 0.0]
        if not self.rf_t:
            self.rf([t0, t1], 0.0)
        sec = lambda t: np.asarray(t, dtype=np.int64).astype(np.float64) * NS
        f = lambda v: np.asarray(v, dtype=np.float64)
        return dict(span=(t0 * NS, t1 * NS), rf=(sec(self.rf_t), f(self.rf_amp), f(self.rf_phase), f(self.rf_freq),
                                                 f(self.rf_coil)),
                    gz=(sec(self.g_t["z"]), f(self.g_a["z"])), gy=(sec(self.g_t["y"]), f(self.g_a["y"])),
                    gx=(sec(self.g_t["x"]), f(self.g_a["x"])), adc=(sec(self.adc_t), f(self.adc_v)),
                    ext=(sec(self.ext_t), f(self.ext_v)))


def concat(trs: List[TR], multi_transmit: bool = False, dummy_trs: int = 0, tx_coil_num: int = 0,
           master_tx_coil: int = 1, max_grad: float = 0.0, max_slew: float = 0.0,
           min_upd_rate: float = 0.0) -> Dict[str, np.ndarray]:
    """The VSeq lines of the TRs, from the native sequence compiler
    (mrl_seq_compile, ``include/mrl_seq.h``): each TR merged as MRiLab's
    compiled PSDs do, the TRs concatenated with ``dummy_trs`` dummies
    (gradients and ADC zeroed), rfCoil forced to 1 without multi-transmit,
    and the multi-transmit, gradient and update-rate checks (0: skipped)."""
    from . import seqc

    return seqc.compile_lines([tr.channels() for tr in trs], multi_transmit=multi_transmit, dummy_trs=dummy_trs,
                              tx_coil_num=tx_coil_num, master_tx_coil=master_tx_coil, max_grad=max_grad,
                              max_slew=max_slew, min_upd_rate=min_upd_rate)


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
