"""Seeded synthetic scans: MATLAB-style globals for the scan engine.

``Scan`` holds the seven structs an MRiLab engine reads (VObj, VMag, VCoi,
VCtl, VSeq, VVar, VSig) as dicts of numpy arrays with the shapes and dtypes
that ``Src/Main/DoPreScan.m`` builds and ``Src/Main/DoDataTypeConv.m:19-138``
fixes:

* per-voxel maps are ``[Y, X, Z]`` (rows = y, columns = x), pool maps add a
  trailing pool axis, isochromat maps ``[Y, X, Z, Spin, Pool]``;
* magnetisation starts at ``Rho / SpinNum`` along z (DoPreScan.m:409-414);
* intravoxel dephasing ``dWRnd = (1/T2* - 1/T2) * tan(pi (u_i - 1/2))`` with
  ``u = linspace(0.01, 0.99, SpinNum)`` (DoPreScan.m:381-390);
* exchange rates are kept as a canonical per-voxel matrix ``rates[..., t, p]``
  = rate from pool t to pool p and laid out into ``VObj.K`` per model by
  ``k_layout`` (ME: channel t*P+p; GM: channel p*P+t; MT: channels 1 and 2;
  CEST: channels t-1 / t+P-2 -- BlochKernel{ME,GM,MT,CEST}.cuh).

The workloads are the five benchmark configurations, each with a ``scale``
knob so tests can run shrunken copies.
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field
from typing import Dict, Optional

import numpy as np

from . import seq as S

GAMMA = S.GAMMA_H
MODELS = ("normal", "me", "mt", "cest", "gm")


@dataclass
class Scan:
    VObj: Dict[str, np.ndarray]
    VMag: Dict[str, np.ndarray]
    VCoi: Dict[str, np.ndarray]
    VCtl: Dict[str, np.ndarray]
    VSeq: Dict[str, np.ndarray]
    VVar: Dict[str, np.ndarray]
    VSig: Dict[str, np.ndarray]
    model: str = "normal"
    rates: Optional[np.ndarray] = None
    info: Dict[str, object] = field(default_factory=dict)

    def structs(self):
        return dict(VObj=self.VObj, VMag=self.VMag, VCoi=self.VCoi, VCtl=self.VCtl,
                    VSeq=self.VSeq, VVar=self.VVar, VSig=self.VSig)

    def copy(self) -> "Scan":
        return copy.deepcopy(self)

    @property
    def dims(self):
        return self.VObj["Rho"].shape[:3]

    @property
    def signal_num(self) -> int:
        return int(self.VSig["SignalNum"])

    def units(self) -> int:
        """Work units: active isochromats x pools x steps with dt > 0."""
        rho = self.VObj["Rho"]
        t1 = self.VObj["T1"]
        t2 = self.VObj["T2"]
        if self.model in ("mt", "cest"):
            act = (rho[..., 0] != 0) & (t1[..., 0] != 0) & (t2[..., 0] != 0)
            n_iso_pool = int(act.sum()) * rho.shape[3]
        elif self.model == "normal":
            act = (rho != 0) & (t1 != 0) & (t2 != 0)
            n_iso_pool = int(act.sum())
        else:
            act = (rho != 0) & (t1 != 0) & (t2 != 0)
            n_iso_pool = int(act.sum())
        uts = self.VSeq["utsLine"]
        n_steps = int(np.count_nonzero(np.diff(uts) > 0))
        return n_iso_pool * int(self.VObj["SpinNum"]) * n_steps


def k_layout(model: str, rates: np.ndarray) -> np.ndarray:
    """Lay a canonical rate matrix ``rates[Y,X,Z,t,p]`` (t -> p) out as VObj.K."""
    Y, X, Z, P, _ = rates.shape
    if model == "me":
        K = np.zeros((Y, X, Z, P * P), np.float32)
        for t in range(P):
            for p in range(P):
                K[..., t * P + p] = rates[..., t, p]
    elif model == "gm":
        K = np.zeros((Y, X, Z, P * P), np.float32)
        for t in range(P):
            for p in range(P):
                K[..., p * P + t] = rates[..., t, p]
    elif model == "mt":
        K = np.zeros((Y, X, Z, 4), np.float32)
        K[..., 1] = rates[..., 0, 1]  # free -> bound (K12)
        K[..., 2] = rates[..., 1, 0]  # bound -> free (K21)
    elif model == "cest":
        K = np.zeros((Y, X, Z, 2 * (P - 1)), np.float32)
        K[..., 0] = rates[..., 0, 1]          # free -> MT
        K[..., P - 1] = rates[..., 1, 0]      # MT -> free
        for t in range(2, P):
            K[..., t - 1] = rates[..., 0, t]  # free -> CEST t
            K[..., t + P - 2] = rates[..., t, 0]  # CEST t -> free
    else:
        raise ValueError(model)
    return K


def _grids(shape, res):
    Y, X, Z = shape
    x = (np.arange(X) - (X - 1) / 2) * res[0]
    y = (np.arange(Y) - (Y - 1) / 2) * res[1]
    z = (np.arange(Z) - (Z - 1) / 2) * res[2]
    gx, gy, gz = np.meshgrid(x, y, z)  # [Y, X, Z], as DoPreScan's meshgrid
    return gx.astype(np.float32), gy.astype(np.float32), gz.astype(np.float32)


def assemble(rho, t1, t2, *, spin_num=1, t2star=None, db0_hz=None, res=(1e-3, 1e-3, 1e-3),
             cs_hz=None, model="normal", rates=None, type_flag=None, tx_mg=None, tx_pe=None,
             rx=None, seqlines=None, tr_num=1, seed=0) -> Scan:
    """Build the seven structs from pool maps ``[Y, X, Z, P]``."""
    rho = np.asarray(rho, np.float32)
    t1 = np.asarray(t1, np.float32)
    t2 = np.asarray(t2, np.float32)
    if rho.ndim == 3:
        rho, t1, t2 = rho[..., None], t1[..., None], t2[..., None]
    Y, X, Z, P = rho.shape
    Sn = int(spin_num)
    gx, gy, gz = _grids((Y, X, Z), res)

    mz = np.zeros((Y, X, Z, Sn, P), np.float32)
    for t in range(P):
        mz[..., t] = (rho[..., t].astype(np.float64) / Sn)[..., None].astype(np.float32)
    dwrnd = np.zeros((Y, X, Z, Sn, P), np.float32)
    if Sn > 1 and t2star is not None:
        u = np.linspace(0.01, 0.99, Sn)
        for t in range(P):
            with np.errstate(divide="ignore", invalid="ignore"):
                r2p = np.where(t2[..., t] > 0, 1.0 / t2star[..., t] - 1.0 / t2[..., t], 0.0)
            for i in range(Sn):
                dwrnd[..., i, t] = (r2p * np.tan(np.pi * (u[i] - 0.5))).astype(np.float32)
    db0 = np.zeros((Y, X, Z), np.float32) if db0_hz is None else (2 * np.pi * db0_hz / GAMMA).astype(np.float32)

    if tx_mg is None:
        tx_mg = np.ones((Y, X, Z, 1), np.float32)
        tx_pe = np.zeros((Y, X, Z, 1), np.float32)
        tx_default = 1.0
    else:
        tx_default = 0.0
    if rx is None:
        rxx = np.ones((Y, X, Z, 1), np.float32)
        rxy = np.zeros((Y, X, Z, 1), np.float32)
        rx_default = 1.0
    else:
        rxx, rxy = np.asarray(rx[0], np.float32), np.asarray(rx[1], np.float32)
        rx_default = 0.0
    ntx, nrx = tx_mg.shape[3], rxx.shape[3]

    vobj = dict(Gyro=np.float64(GAMMA), Mx=np.zeros_like(mz), My=np.zeros_like(mz), Mz=mz,
                Rho=rho, T1=t1, T2=t2, SpinNum=np.int32(Sn), TypeNum=np.int32(P),
                ChemShift=np.float64(0.0))
    if model != "normal":
        vobj["K"] = k_layout(model, rates)
    if model == "gm":
        vobj["TypeFlag"] = np.asarray(type_flag, np.float64)
    vmag = dict(dB0=db0, dWRnd=dwrnd, Gzgrid=gz, Gygrid=gy, Gxgrid=gx)
    vcoi = dict(TxCoilmg=np.asarray(tx_mg, np.float32), TxCoilpe=np.asarray(tx_pe, np.float32),
                RxCoilx=rxx, RxCoily=rxy, TxCoilNum=np.int32(ntx), RxCoilNum=np.int32(nrx),
                TxCoilDefault=np.float64(tx_default), RxCoilDefault=np.float64(rx_default))
    cs = np.zeros(P) if cs_hz is None else np.asarray(cs_hz, np.float64)
    vctl = dict(CS=cs.astype(np.float64), TRNum=np.int32(tr_num), RunMode=np.int32(0),
                MaxThreadNum=np.int32(1), ActiveThreadNum=np.int32(0), GPUIndex=np.int32(0))
    nsig = int(np.count_nonzero(seqlines["ADCLine"] == 1))
    vvar = dict(t=np.float64(0), dt=np.float64(0), rfAmp=np.zeros(ntx), rfPhase=np.zeros(ntx),
                rfFreq=np.zeros(ntx), rfCoil=np.float64(0), rfRef=np.float64(0),
                GzAmp=np.float64(0), GyAmp=np.float64(0), GxAmp=np.float64(0),
                ADC=np.float64(0), Ext=np.float64(0), Kz=np.float64(0), Ky=np.float64(0),
                Kx=np.float64(0), gpuFetch=np.float64(0),
                utsi=np.int32(0), rfi=np.int32(0), Gzi=np.int32(0), Gyi=np.int32(0),
                Gxi=np.int32(0), ADCi=np.int32(0), Exti=np.int32(0), TRCount=np.int32(1),
                SliceCount=np.int32(1), PhaseCount=np.int32(1))
    vsig = dict(Sx=np.zeros(nsig * P * nrx), Sy=np.zeros(nsig * P * nrx),
                Kz=np.zeros(nsig), Ky=np.zeros(nsig), Kx=np.zeros(nsig),
                Mx=np.zeros_like(mz), My=np.zeros_like(mz), Mz=mz.copy(),
                Muts=np.float64(0), SignalNum=np.int32(nsig))
    # MATLAB's column-major layout, which is what the engine binds
    for d in (vobj, vmag, vcoi, vsig):
        for k, a in d.items():
            if isinstance(a, np.ndarray) and a.ndim > 1:
                d[k] = np.asfortranarray(a)
    return Scan(vobj, vmag, vcoi, vctl, dict(seqlines), vvar, vsig, model=model, rates=rates,
                info=dict(seed=seed))


def with_history(sc: Scan) -> Scan:
    """A copy of ``sc`` set up for RunMode 1 the way the spin watcher does
    (DoSpinWatchExec.m:152-161): VSig.Mx/My/Mz [Y, X, Z, S, P, len(uts)]
    single with slot 0 = the initial magnetisation, VSig.Muts zeros."""
    out = sc.copy()
    n = out.VSeq["utsLine"].size
    for k in ("Mx", "My", "Mz"):
        m = np.asarray(out.VObj[k], np.float32)
        h = np.zeros(m.shape + (n,), np.float32, order="F")
        h[..., 0] = m
        out.VSig[k] = h
    out.VSig["Muts"] = np.zeros((n, 1))
    out.VCtl["RunMode"] = np.int32(1)
    return out


# ---------------------------------------------------------------------------
# sequences
# ---------------------------------------------------------------------------

def gre_lines(*, n_read, n_pe, n_par=1, fov=(0.24, 0.24, 0.24), tr_ms=20.0, te_ms=(5.0,),
              flip=30.0, rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0,
              spoil=True, n_tr=None, ext_every=0, tx_coils=1, gamma=GAMMA):
    """Cartesian (multi-echo) gradient echo, 2D (n_par=1) or 3D.

    RF: windowed sinc (``tx_coils`` > 1: the same pulse on every Tx coil,
    coil c scaled by 1 / c and shifted in phase by 0.7 (c - 1) rad); slab
    gradient on z during RF, rephased after;
    phase encode on y (and partition encode on z); monopolar readouts on x
    centred at each TE (ms, from the RF centre) with a rewinder between
    echoes; a spoiler lobe after the last echo.
    """
    dwell_ns = int(round(1e9 / bw_hz))
    rf_ns = int(round(rf_ms * 1e6))
    raster_ns = int(round(rf_raster_us * 1e3))
    tr_ns = int(round(tr_ms * 1e6))
    ramp = 100_000  # 0.1 ms ramps
    gread = 2 * np.pi / (gamma * fov[0] * dwell_ns * S.NS)
    ro_ns = n_read * dwell_ns
    rf_center = rf_ns // 2
    gslab = 2 * np.pi / (gamma * fov[2] * 4 * raster_ns * S.NS) * 0.05  # mild slab gradient
    trs = []
    total = n_pe * n_par if n_tr is None else n_tr
    for i in range(total):
        ipe = i % n_pe
        ipar = (i // n_pe) % n_par
        tr = S.TR(tr_ns)
        t_rf, a_rf = S.sinc_rf(0, rf_ns, raster_ns, flip, tbw)
        tr.rf(t_rf, a_rf)
        for c in range(2, tx_coils + 1):
            tr.rf(t_rf, np.asarray(a_rf) / c, 0.7 * (c - 1), 0.0, coil=c)
        tr.trap("z", 0, rf_ns, gslab, ramp_ns=raster_ns)
        # encoding window between the RF end and the first readout
        first_ro = rf_center + int(round(te_ms[0] * 1e6)) - ro_ns // 2
        enc0 = rf_ns + 20_000
        enc1 = first_ro - 20_000
        if enc1 - enc0 < 4 * ramp:
            raise ValueError("TE too short for the encoding lobes")
        dur = (enc1 - enc0 - 2 * ramp) * S.NS
        ky = (ipe - n_pe // 2) / fov[1]
        tr.trap("y", enc0, enc1, 2 * np.pi * ky / (gamma * dur), ramp_ns=ramp)
        gz_area = -gslab * (rf_ns - 2 * raster_ns) * S.NS / 2
        if n_par > 1:
            kz = (ipar - n_par // 2) / fov[2]
            gz_area += 2 * np.pi * kz / gamma
        tr.trap("z", enc0, enc1, gz_area / dur, ramp_ns=ramp)
        pre_area = -gread * (n_read // 2) * dwell_ns * S.NS
        tr.trap("x", enc0, enc1, pre_area / dur, ramp_ns=ramp)
        adc_times = []
        prev_end = None
        for e, te in enumerate(te_ms):
            ro_start = rf_center + int(round(te * 1e6)) - (n_read // 2) * dwell_ns
            if prev_end is not None:
                # rewind the full readout lobe before the next echo
                g0, g1 = prev_end + 20_000, ro_start - ramp - 20_000
                if g1 - g0 < 3 * ramp:
                    raise ValueError("echo spacing too short")
                rdur = (g1 - g0 - 2 * ramp) * S.NS
                tr.trap("x", g0, g1, -gread * ro_ns * S.NS / rdur, ramp_ns=ramp)
            tr.trap("x", ro_start - ramp, ro_start + ro_ns + ramp, gread, ramp_ns=ramp)
            adc_times += list(ro_start + dwell_ns * np.arange(n_read))
            prev_end = ro_start + ro_ns + ramp
        tr.adc_t += [0]
        tr.adc_v += [0.0]
        tr.adc(adc_times)
        tr.adc_t += [tr_ns]
        tr.adc_v += [0.0]
        if spoil and prev_end + 2_500_000 < tr_ns:
            tr.trap("x", prev_end + 50_000, prev_end + 2_050_000, 4 * gread, ramp_ns=ramp)
        if ext_every and (i % ext_every == ext_every - 1):
            tr.ext_t += [0]
            tr.ext_v += [0.0]
            tr.ext(prev_end + 10_000, 1.0)
            tr.ext_t += [tr_ns]
            tr.ext_v += [0.0]
        trs.append(tr)
    return S.concat(trs, multi_transmit=tx_coils > 1), total


# ---------------------------------------------------------------------------
# the five workloads
# ---------------------------------------------------------------------------

def config1_gre(seed=0, n=64, n_tr=None) -> Scan:
    """Plain single-pool 2D GRE: n x n x 1, three concentric disks, dB0 ~ N(0, 10 Hz)."""
    rng = np.random.default_rng(seed)
    Y = X = n
    yy, xx = np.mgrid[0:Y, 0:X]
    r = np.hypot((xx - (X - 1) / 2) / (X / 2), (yy - (Y - 1) / 2) / (Y / 2))
    rho = np.zeros((Y, X, 1), np.float32)
    t1 = np.zeros_like(rho)
    t2 = np.zeros_like(rho)
    for rmax, T1, T2, M0 in [(0.9, 0.8, 0.08, 0.7), (0.6, 1.3, 0.11, 0.8), (0.3, 4.0, 2.0, 1.0)]:
        m = (r <= rmax)[..., None]
        rho[m], t1[m], t2[m] = M0, T1, T2
    db0 = rng.normal(0.0, 10.0, (Y, X, 1))
    fov = 0.24
    lines, ntr = gre_lines(n_read=n, n_pe=n, fov=(fov, fov, fov), tr_ms=20.0, te_ms=(5.0,),
                           flip=30.0, rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0,
                           n_tr=n_tr)
    return assemble(rho, t1, t2, db0_hz=db0, res=(fov / X, fov / Y, 0.005), seqlines=lines,
                    tr_num=ntr, seed=seed)


def multi_tx_gre(seed=0, n=8, n_tr=2, tx_coils=2, rx_coils=2) -> Scan:
    """A small single-pool 2D GRE transmitting on ``tx_coils`` coils with
    seeded smooth magnitude / phase maps (the B1 of a step is the complex
    sum over the coils, BlochKernel.h:62-110), ``rx_coils`` receive coils."""
    rng = np.random.default_rng(seed)
    Y = X = n
    yy, xx = np.mgrid[0:Y, 0:X]
    r = np.hypot((xx - (X - 1) / 2) / (X / 2), (yy - (Y - 1) / 2) / (Y / 2))
    inside = (r <= 0.9)[..., None]
    rho = np.where(inside, rng.uniform(0.5, 1.0, (Y, X, 1)), 0).astype(np.float32)
    t1 = np.where(inside, rng.uniform(0.5, 1.5, (Y, X, 1)), 0).astype(np.float32)
    t2 = np.where(inside, rng.uniform(0.04, 0.12, (Y, X, 1)), 0).astype(np.float32)
    db0 = rng.normal(0.0, 10.0, (Y, X, 1))
    fov = 0.24
    res = (fov / X, fov / Y, 0.005)
    tx_mg = np.stack([0.6 + 0.4 * np.cos(np.pi * (xx / X + c / tx_coils))[..., None]
                      for c in range(tx_coils)], -1).astype(np.float32)
    tx_pe = np.stack([(0.5 * c + 0.3 * (yy / Y))[..., None] for c in range(tx_coils)], -1).astype(np.float32)
    rx = _cylinder_coils((Y, X, 1), res, rx_coils, rng) if rx_coils > 1 else None
    lines, ntr = gre_lines(n_read=n, n_pe=n, fov=(fov, fov, fov), tr_ms=20.0, te_ms=(5.0,), flip=30.0,
                           rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0, n_tr=n_tr, tx_coils=tx_coils)
    return assemble(rho, t1, t2, db0_hz=db0, res=res, tx_mg=tx_mg, tx_pe=tx_pe, rx=rx, seqlines=lines,
                    tr_num=ntr, seed=seed)


def _cylinder_coils(shape, res, n_coils, rng):
    Y, X, Z = shape
    gx, gy, gz = _grids(shape, res)
    radius = 0.6 * max(X * res[0], Y * res[1])
    sigma = 0.5 * radius
    mags, phs = [], []
    for c in range(n_coils):
        th = 2 * np.pi * c / n_coils
        cx, cy = radius * np.cos(th), radius * np.sin(th)
        cz = (rng.uniform(-0.3, 0.3)) * Z * res[2]
        d2 = (gx - cx) ** 2 + (gy - cy) ** 2 + (gz - cz) ** 2
        mags.append(np.exp(-d2 / (2 * sigma**2)))
        phs.append(th + 2 * np.pi * (gx * np.cos(th) + gy * np.sin(th)) / (4 * radius))
    mag = np.stack(mags, -1)
    ph = np.stack(phs, -1)
    return (mag * np.cos(ph)).astype(np.float32), (mag * np.sin(ph)).astype(np.float32)


def config2_me_gre(seed=0, nx=128, ny=128, nz=32, n_pe=32, n_par=8, n_read=128, spins=4,
                   n_coils=8, n_tr=None, model="me") -> Scan:
    """Two-pool exchange 3D multi-echo GRE with 8 Rx coils (precision study).

    Free water (T1 1000 / T2 60 ms) and myelin water (T1 400 / T2 12 ms),
    myelin fraction ~ U(0, 0.25), exchange k ~ U(2, 20) 1/s from myelin to
    free water (detailed balance sets the reverse rate), dB0 ~ N(0, 25 Hz),
    4 spins per voxel with intravoxel dephasing, 6 echoes at TE 2..22 ms,
    ``n_pe`` x ``n_par`` phase/partition encodes of ``n_read`` samples.
    """
    rng = np.random.default_rng(seed)
    Y, X, Z = ny, nx, nz
    yy, xx, zz = np.meshgrid(np.arange(Y), np.arange(X), np.arange(Z), indexing="ij")
    r = np.hypot((xx - (X - 1) / 2) / (X / 2), (yy - (Y - 1) / 2) / (Y / 2))
    inside = r <= 0.85
    f = rng.uniform(0.0, 0.25, (Y, X, Z))
    rho = np.zeros((Y, X, Z, 2), np.float32)
    rho[..., 0] = np.where(inside, 1.0 - f, 0.0)
    rho[..., 1] = np.where(inside, f, 0.0)
    t1 = np.zeros_like(rho)
    t2 = np.zeros_like(rho)
    t1[..., 0], t2[..., 0] = np.where(inside, 1.0, 0.0), np.where(inside, 0.060, 0.0)
    t1[..., 1], t2[..., 1] = np.where(inside, 0.4, 0.0), np.where(inside, 0.012, 0.0)
    # a myelin fraction of exactly 0 leaves that pool empty (Rho == 0)
    k = rng.uniform(2.0, 20.0, (Y, X, Z))
    rates = np.zeros((Y, X, Z, 2, 2), np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        rates[..., 1, 0] = np.where(inside, k, 0.0)
        rates[..., 0, 1] = np.where(inside & (f < 1), k * f / np.maximum(1 - f, 1e-6), 0.0)
    db0 = rng.normal(0.0, 25.0, (Y, X, Z))
    t2star = np.stack([np.full((Y, X, Z), 0.040), np.full((Y, X, Z), 0.010)], -1)
    fov = (0.24, 0.24, 0.24 * Z / X)
    res = (fov[0] / X, fov[1] / Y, fov[2] / Z)
    rxx, rxy = _cylinder_coils((Y, X, Z), res, n_coils, rng)
    lines, ntr = gre_lines(n_read=n_read, n_pe=n_pe, n_par=n_par, fov=fov, tr_ms=25.0,
                           te_ms=(2.0, 6.0, 10.0, 14.0, 18.0, 22.0), flip=20.0, rf_ms=0.5,
                           rf_raster_us=10.0, tbw=2.0, bw_hz=64000.0, n_tr=n_tr)
    tf = np.zeros(2) if model == "gm" else None
    return assemble(rho, t1, t2, spin_num=spins, t2star=t2star, db0_hz=db0, res=res,
                    model=model, rates=rates, type_flag=tf, rx=(rxx, rxy), seqlines=lines,
                    tr_num=ntr, seed=seed)


def bssfp_lines(*, n_read=96, n_pe=96, n_par=16, fov=(0.24, 0.24, 0.04), tr_ms=5.0, te_ms=2.0, flip=40.0,
                rf_samples=512, rf_raster_us=2.0, tbw=4.0, bw_hz=125000.0, n_tr=200, gamma=GAMMA):
    """Balanced SSFP, 3D Cartesian: every TR plays the same complex rf
    waveform of ``rf_samples`` samples (a windowed sinc with a slow phase
    modulation) with the phase cycled by pi every other TR, a slab gradient
    under it, phase / partition / readout prephasers, a readout of
    ``n_read`` samples centred ``te_ms`` after the rf centre, and rewinders
    that null every gradient axis's area over the TR.  The areas are those
    the engine's sample-and-hold integrates (trapezoid flats; the ramps hold
    their zero end).  Phase and partition encodes cycle over ``n_tr`` TRs."""
    raster = int(round(rf_raster_us * 1e3))
    rf_ns = (rf_samples - 1) * raster
    dwell = int(round(1e9 / bw_hz))
    ro_ns = n_read * dwell
    tr_ns = int(round(tr_ms * 1e6))
    ramp = 100_000
    rf_center = rf_ns // 2
    ro_start = rf_center + int(round(te_ms * 1e6)) - ro_ns // 2
    enc0, enc1 = rf_ns + 20_000, ro_start - ramp - 20_000
    rw0 = ro_start + ro_ns + ramp + 20_000
    rw1 = rw0 + (enc1 - enc0)
    if enc1 - enc0 < 3 * ramp or rw1 + 20_000 > tr_ns:
        raise ValueError("TR / TE too short for the balanced lobes")
    flat = lambda t0, t1: (t1 - t0 - 2 * ramp) * S.NS  # seconds of flat top
    gread = 2 * np.pi / (gamma * fov[0] * dwell * S.NS)
    slab_area = 2 * np.pi / (gamma * fov[2] * 4 * raster * S.NS) * 0.05 * (rf_ns - 2 * raster) * S.NS
    gslab = slab_area / ((rf_ns - 2 * raster) * S.NS)
    t_rf, a_rf = S.sinc_rf(0, rf_ns, raster, flip, tbw)
    assert t_rf.size == rf_samples
    j = np.arange(rf_samples)
    ph_rf = 0.25 + 0.1 * np.sin(2 * np.pi * j / (rf_samples - 1))
    trs = []
    for i in range(n_tr):
        ipe, ipar = i % n_pe, (i // n_pe) % n_par
        tr = S.TR(tr_ns)
        tr.rf(t_rf, a_rf, ph_rf + np.pi * (i % 2))
        tr.trap("z", 0, rf_ns, gslab, ramp_ns=raster)
        ky = (ipe - n_pe // 2) / fov[1]
        kz = (ipar - n_par // 2) / fov[2]
        a_y = 2 * np.pi * ky / gamma
        a_z = -slab_area / 2 + 2 * np.pi * kz / gamma
        a_x = -gread * (n_read // 2) * dwell * S.NS
        tr.trap("y", enc0, enc1, a_y / flat(enc0, enc1), ramp_ns=ramp)
        tr.trap("z", enc0, enc1, a_z / flat(enc0, enc1), ramp_ns=ramp)
        tr.trap("x", enc0, enc1, a_x / flat(enc0, enc1), ramp_ns=ramp)
        tr.trap("x", ro_start - ramp, ro_start + ro_ns + ramp, gread, ramp_ns=ramp)
        tr.adc_t += [0]
        tr.adc_v += [0.0]
        tr.adc(ro_start + dwell * np.arange(n_read))
        tr.adc_t += [tr_ns]
        tr.adc_v += [0.0]
        tr.trap("y", rw0, rw1, -a_y / flat(rw0, rw1), ramp_ns=ramp)
        tr.trap("z", rw0, rw1, -(slab_area + a_z) / flat(rw0, rw1), ramp_ns=ramp)
        tr.trap("x", rw0, rw1, -(a_x + gread * ro_ns * S.NS) / flat(rw0, rw1), ramp_ns=ramp)
        trs.append(tr)
    return S.concat(trs), n_tr


def epi_lines(*, n_read=128, n_pe=128, fov=(0.24, 0.24, 0.12), bw_hz=250000.0, ramp_us=40.0,
              mt_ms=8.0, mt_offset_hz=1500.0, mt_b1_ut=6.0, mt_raster_us=10.0, ex_ms=2.0, ex_raster_us=10.0,
              flip=90.0, tbw=4.0, gamma=GAMMA):
    """Single-shot EPI with magnetisation-transfer preparation: a Gaussian
    off-resonance MT pulse (``mt_ms`` long, ``mt_offset_hz`` off, peak
    ``mt_b1_ut``), a spoiler, a slab-selective sinc excitation, prephasers
    and ``n_pe`` readout lines of ``n_read`` samples at ``bw_hz`` with
    alternating readout polarity and phase-encode blips between lines."""
    dwell = int(round(1e9 / bw_hz))
    ramp = int(round(ramp_us * 1e3))
    ro_ns = n_read * dwell
    mt_raster = int(round(mt_raster_us * 1e3))
    mt_ns = int(round(mt_ms * 1e6)) // mt_raster * mt_raster
    ex_raster = int(round(ex_raster_us * 1e3))
    ex_ns = int(round(ex_ms * 1e6)) // ex_raster * ex_raster
    flat = lambda t0, t1: (t1 - t0 - 2 * ramp) * S.NS
    gread = 2 * np.pi / (gamma * fov[0] * dwell * S.NS)
    gblip_area = 2 * np.pi / (gamma * fov[1])
    t = 0
    tr = None
    # MT preparation: Gaussian envelope, sigma = duration / 6
    t_mt = np.arange(mt_ns // mt_raster + 1, dtype=np.int64) * mt_raster
    env = np.exp(-0.5 * ((t_mt - mt_ns / 2) / (mt_ns / 6)) ** 2)
    env[0] = env[-1] = 0.0
    t = mt_ns
    spoil0, spoil1 = t + 20_000, t + 1_020_000
    ex0 = spoil1 + 20_000
    t_ex, a_ex = S.sinc_rf(ex0, ex_ns, ex_raster, flip, tbw)
    gslab = 2 * np.pi / (gamma * fov[2] * 4 * ex_raster * S.NS) * 0.05
    slab_area = gslab * (ex_ns - 2 * ex_raster) * S.NS
    pre0 = ex0 + ex_ns + 20_000
    pre1 = pre0 + 400_000
    lines0 = pre1 + 20_000
    line_ns = ro_ns + 2 * ramp
    tr_ns = lines0 + n_pe * line_ns + 200_000
    tr = S.TR(tr_ns)
    tr.rf(t_mt, mt_b1_ut * 1e-6 * env, 0.0, mt_offset_hz)
    tr.trap("z", spoil0, spoil1, 4 * gread, ramp_ns=100_000)
    tr.rf(t_ex, a_ex)
    tr.trap("z", ex0, ex0 + ex_ns, gslab, ramp_ns=ex_raster)
    tr.trap("z", pre0, pre1, -slab_area / 2 / flat(pre0, pre1), ramp_ns=ramp)
    tr.trap("x", pre0, pre1, -gread * (ro_ns / 2 + ramp) * S.NS / flat(pre0, pre1), ramp_ns=ramp)
    tr.trap("y", pre0, pre1, -gblip_area * (n_pe // 2) / flat(pre0, pre1), ramp_ns=ramp)
    tr.adc_t += [0]
    tr.adc_v += [0.0]
    for i in range(n_pe):
        l0 = lines0 + i * line_ns
        sgn = 1.0 if i % 2 == 0 else -1.0
        tr.trap("x", l0, l0 + line_ns, sgn * gread, ramp_ns=ramp)
        tr.adc(l0 + ramp + dwell * np.arange(n_read))
        if i + 1 < n_pe:  # blip across the ramps between lines
            b0 = l0 + line_ns - ramp
            tr.trap("y", b0, b0 + 2 * ramp, gblip_area / ((2 * ramp - ramp) * S.NS), ramp_ns=ramp // 2)
    tr.adc_t += [tr_ns]
    tr.adc_v += [0.0]
    return S.concat([tr]), 1


def sat_gre_lines(*, n_read=16, n_pe=4, fov=0.2, tr_ms=30.0, sat_offsets_hz=(1500.0,), sat_ms=4.0,
                  sat_b1_ut=2.0, sat_raster_us=20.0, flip=15.0, bw_hz=32000.0, gamma=GAMMA):
    """Saturation-prepared GRE: per TR a block of Gaussian saturation pulses
    at ``sat_offsets_hz`` (one offset per TR, cycled), then a hard
    excitation and one Cartesian readout -- the MT/CEST workloads' shape."""
    dwell = int(round(1e9 / bw_hz))
    raster = int(round(sat_raster_us * 1e3))
    sat_ns = int(round(sat_ms * 1e6))
    tr_ns = int(round(tr_ms * 1e6))
    ramp = 100_000
    gread = 2 * np.pi / (gamma * fov * dwell * S.NS)
    trs = []
    for i in range(n_pe):
        tr = S.TR(tr_ns)
        off = sat_offsets_hz[i % len(sat_offsets_hz)]
        n = sat_ns // raster + 1
        t = np.arange(n, dtype=np.int64) * raster
        env = np.exp(-0.5 * ((t - sat_ns / 2) / (sat_ns / 5)) ** 2)
        env[0] = env[-1] = 0.0
        tr.rf(t, sat_b1_ut * 1e-6 * env, 0.0, off)
        t_ex = sat_ns + 1_000_000
        t_hr, a_hr = S.hard_rf(t_ex, 200_000, flip)
        tr.rf(t_hr, a_hr)
        ro = t_ex + 2_000_000
        ky = (i - n_pe // 2) / fov
        dur = (1_600_000 - 2 * ramp) * S.NS
        tr.trap("y", t_ex + 250_000, t_ex + 1_850_000, 2 * np.pi * ky / (gamma * dur), ramp_ns=ramp)
        tr.trap("x", t_ex + 250_000, t_ex + 1_850_000, -gread * (n_read // 2) * dwell * S.NS / dur, ramp_ns=ramp)
        tr.trap("x", ro - ramp, ro + n_read * dwell + ramp, gread, ramp_ns=ramp)
        tr.adc_t += [0]
        tr.adc_v += [0.0]
        tr.adc(ro + dwell * np.arange(n_read))
        tr.adc_t += [tr_ns]
        tr.adc_v += [0.0]
        trs.append(tr)
    return S.concat(trs), n_pe


def small_multipool(model: str, seed=0, n=8, nz=1, pools=2, spins=1, coils=1, n_tr=3, seq="gre") -> Scan:
    """A small random multi-pool scan for parity tests of the ME/MT/CEST/GM
    models: random tissue per voxel, rates obeying detailed balance."""
    rng = np.random.default_rng(seed)
    Y = X = n
    Z = nz
    P = pools
    yy, xx = np.mgrid[0:Y, 0:X]
    inside2d = np.hypot(xx - (X - 1) / 2, yy - (Y - 1) / 2) <= 0.45 * n
    inside = np.repeat(inside2d[..., None], Z, axis=2)
    frac = rng.uniform(0.02, 0.2, (Y, X, Z, P))
    frac[..., 0] = 1.0
    rho = (frac * inside[..., None]).astype(np.float32)
    t1 = np.where(inside[..., None], rng.uniform(0.3, 1.5, (Y, X, Z, P)), 0).astype(np.float32)
    t2 = np.where(inside[..., None], rng.uniform(0.01, 0.1, (Y, X, Z, P)), 0).astype(np.float32)
    type_flag = None
    if model in ("mt", "cest"):
        t2[..., 1] = np.where(inside, 12e-6, 0)  # bound pool T2 (s)
    if model == "gm":
        type_flag = np.zeros(P)
        type_flag[-1] = 1.0
        t2[..., -1] = np.where(inside, 10e-6, 0)
    rates = np.zeros((Y, X, Z, P, P), np.float32)
    for p in range(1, P):
        k = rng.uniform(10, 500, (Y, X, Z))
        if model in ("me", "gm"):
            rates[..., p, 0] = np.where(inside, k, 0)
            rates[..., 0, p] = np.where(inside, k * rho[..., p] / np.maximum(rho[..., 0], 1e-6), 0)
            if model == "me" and P > 2 and p == P - 1:
                k2 = rng.uniform(5, 50, (Y, X, Z))
                rates[..., p, 1] = np.where(inside, k2, 0)
                rates[..., 1, p] = np.where(inside, k2 * rho[..., p] / np.maximum(rho[..., 1], 1e-6), 0)
        else:  # mt / cest: exchange with free water only
            rates[..., p, 0] = np.where(inside, k, 0)
            rates[..., 0, p] = np.where(inside, k * rho[..., p] / np.maximum(rho[..., 0], 1e-6), 0)
    db0 = rng.normal(0.0, 20.0, (Y, X, Z))
    cs = np.zeros(P)
    if model == "cest":
        cs[2:] = rng.choice([3.5 * 128.0, 2.0 * 128.0, -3.5 * 128.0], P - 2, replace=False)
    elif model in ("me", "gm"):
        cs[1:] = rng.uniform(-50, 50, P - 1)
    fov = 0.2
    res = (fov / X, fov / Y, 0.005)
    rx = _cylinder_coils((Y, X, Z), res, coils, rng) if coils > 1 else None
    if seq == "sat":
        lines, ntr = sat_gre_lines(n_read=n, n_pe=n_tr, fov=fov, sat_offsets_hz=(1500.0, -800.0, 400.0))
    else:
        lines, ntr = gre_lines(n_read=n, n_pe=n_tr, fov=(fov, fov, fov), tr_ms=12.0, te_ms=(4.0,), flip=25.0,
                               rf_ms=1.0, rf_raster_us=10.0, tbw=2.0, bw_hz=32000.0)
    t2s = np.maximum(t2 * 0.5, 1e-6) if spins > 1 else None
    return assemble(rho, t1, t2, spin_num=spins, t2star=t2s, db0_hz=db0, res=res, cs_hz=cs, model=model,
                    rates=rates, type_flag=type_flag, rx=rx, seqlines=lines, tr_num=ntr, seed=seed)


# ---------------------------------------------------------------------------
# batched CEST Z-spectra (many independent instances)
# ---------------------------------------------------------------------------

PPM_3T_HZ = GAMMA / (2 * np.pi) * 3.0 * 1e-6  # Hz per ppm of the 1H resonance at 3 T
CEST_POOLS_PPM = (3.5, 2.0, -3.5)             # amide, amine, NOE


def zspec_lines(*, offset_hz, sat_ms, b1_ut, raster_us=10.0, flip=90.0, gamma=GAMMA):
    """One Z-spectrum point: continuous-wave saturation at ``offset_hz`` and
    ``b1_ut`` for ``sat_ms`` on a ``raster_us`` raster, then a hard
    excitation and one sample of the FID."""
    raster = int(round(raster_us * 1e3))
    sat_ns = int(round(sat_ms * 1e6)) // raster * raster
    t_ex = sat_ns + 200_000
    tr_ns = t_ex + 1_000_000
    tr = S.TR(tr_ns)
    t = np.arange(sat_ns // raster + 1, dtype=np.int64) * raster
    amp = np.full(t.size, b1_ut * 1e-6)
    amp[0] = amp[-1] = 0.0
    tr.rf(t, amp, 0.0, offset_hz)
    t_hr, a_hr = S.hard_rf(t_ex, 100_000, flip, gamma)
    tr.rf(t_hr, a_hr)
    tr.adc_t += [0]
    tr.adc_v += [0.0]
    tr.adc([t_ex + 300_000])
    tr.adc_t += [tr_ns]
    tr.adc_v += [0.0]
    return S.concat([tr]), 1


def cest_instance(seed, n_vox, pools, offset_ppm, b1_ut, sat_ms) -> Scan:
    """One instance of the batched CEST workload: ``n_vox`` voxels of water,
    a semisolid MT pool and ``pools - 2`` CEST pools (amide, amine, NOE),
    fractions U(0.001, 0.1), exchange rates U(10, 5000) /s (pool -> water;
    water -> pool by detailed balance), dB0 N(0, 10 Hz), 3 T."""
    rng = np.random.default_rng(seed)
    P = pools
    shape = (n_vox, 1, 1)
    frac = rng.uniform(0.001, 0.1, shape + (P,))
    frac[..., 0] = 1.0
    rho = frac.astype(np.float32)
    t1 = np.empty(shape + (P,), np.float32)
    t2 = np.empty(shape + (P,), np.float32)
    t1[..., 0] = rng.uniform(0.8, 1.6, shape)
    t2[..., 0] = rng.uniform(0.04, 0.1, shape)
    t1[..., 1] = 1.0
    t2[..., 1] = 10e-6  # semisolid (super-Lorentzian lineshape)
    for p in range(2, P):
        t1[..., p] = 1.0
        t2[..., p] = rng.uniform(0.005, 0.02, shape)
    rates = np.zeros(shape + (P, P), np.float32)
    for p in range(1, P):
        k = rng.uniform(10, 5000, shape)
        rates[..., p, 0] = k
        rates[..., 0, p] = k * rho[..., p] / rho[..., 0]
    cs = np.zeros(P)
    cs[2:] = np.array(CEST_POOLS_PPM[:P - 2]) * PPM_3T_HZ
    lines, ntr = zspec_lines(offset_hz=offset_ppm * PPM_3T_HZ, sat_ms=sat_ms, b1_ut=b1_ut)
    return assemble(rho, t1, t2, db0_hz=rng.normal(0.0, 10.0, shape), res=(1e-3, 1e-3, 1e-3), cs_hz=cs,
                    model="cest", rates=rates, seqlines=lines, tr_num=ntr, seed=seed)


def config3_batch(seed=0, n_inst=256, vox_range=(1000, 262144), sat_s=(1.0, 4.0), sat_scale=1.0 / 40,
                  n_offsets=51, vox_scale=1.0):
    """The batched CEST workload: ``n_inst`` instances with log-uniform voxel
    counts in ``vox_range`` (times ``vox_scale``), 3-5 pools, one of
    ``n_offsets`` offsets in +-6 ppm, B1 U(0.5, 3) uT and a saturation of
    U(``sat_s``) seconds times ``sat_scale`` (the timed subset of the 1-4 s
    trains).  Returns the list of scans and their description."""
    rng = np.random.default_rng(seed)
    offsets = np.linspace(-6.0, 6.0, n_offsets)
    scans, meta = [], []
    for i in range(n_inst):
        nv = int(round(np.exp(rng.uniform(np.log(vox_range[0]), np.log(vox_range[1]))) * vox_scale))
        nv = max(nv, 1)
        pools = int(rng.integers(3, 6))
        off = float(offsets[rng.integers(0, n_offsets)])
        b1 = float(rng.uniform(0.5, 3.0))
        sat_ms = float(rng.uniform(*sat_s)) * sat_scale * 1e3
        scans.append(cest_instance(seed * 100003 + i, nv, pools, off, b1, sat_ms))
        meta.append(dict(voxels=nv, pools=pools, offset_ppm=off, b1_ut=b1, sat_ms=sat_ms))
    return scans, meta


# the four tissue classes of the adjoint workload: T1 (s), T2 (s), M0 and
# the fraction of the second (short-T2, exchanging) water pool
CONFIG4_CLASSES = ((0.83, 0.080, 0.70, 0.15), (1.33, 0.110, 0.80, 0.05), (4.00, 2.000, 1.00, 0.01),
                   (1.40, 0.050, 0.90, 0.10))


def config4_adjoint(seed=0, nx=96, ny=96, nz=16, spins=2, n_tr=200, n_coils=4, rf_samples=512) -> Scan:
    """The adjoint workload: ``ny x nx x nz`` voxels of a seeded 4-class
    phantom (classes ``CONFIG4_CLASSES``, per-voxel values jittered by
    U(0.95, 1.05)), each voxel a free pool and a short-T2 pool (T1 400 ms,
    T2 12 ms) exchanging at k ~ U(2, 20) /s (detailed balance sets the
    reverse rate), dB0 ~ N(0, 15 Hz), ``spins`` spins per voxel with
    intravoxel dephasing (T2* = 0.7 T2), ``n_coils`` Rx coils on a cylinder;
    balanced SSFP with ``n_tr`` TRs of 5 ms, flip 40 degrees and a
    ``rf_samples``-sample complex rf waveform."""
    rng = np.random.default_rng(seed)
    Y, X, Z = ny, nx, nz
    # blocky class map: argmax of four coarse random fields, upsampled
    coarse = rng.normal(size=(max(Y // 8, 1), max(X // 8, 1), max(Z // 4, 1), 4))
    iy = np.minimum(np.arange(Y) * coarse.shape[0] // Y, coarse.shape[0] - 1)
    ix = np.minimum(np.arange(X) * coarse.shape[1] // X, coarse.shape[1] - 1)
    iz = np.minimum(np.arange(Z) * coarse.shape[2] // Z, coarse.shape[2] - 1)
    label = np.argmax(coarse[iy][:, ix][:, :, iz], axis=-1)
    tab = np.asarray(CONFIG4_CLASSES)
    jit = lambda: rng.uniform(0.95, 1.05, (Y, X, Z))
    T1, T2, M0, f2 = (tab[label, c] * jit() for c in range(4))
    rho = np.stack([M0 * (1 - f2), M0 * f2], -1).astype(np.float32)
    t1 = np.stack([T1, np.full_like(T1, 0.4)], -1).astype(np.float32)
    t2 = np.stack([T2, np.full_like(T2, 0.012)], -1).astype(np.float32)
    k = rng.uniform(2.0, 20.0, (Y, X, Z))
    rates = np.zeros((Y, X, Z, 2, 2), np.float32)
    rates[..., 1, 0] = k
    rates[..., 0, 1] = k * f2 / (1 - f2)
    db0 = rng.normal(0.0, 15.0, (Y, X, Z))
    fov = (0.24, 0.24 * Y / X, 0.24 * Z / X)
    res = (fov[0] / X, fov[1] / Y, fov[2] / Z)
    rxx, rxy = _cylinder_coils((Y, X, Z), res, n_coils, rng)
    lines, ntr = bssfp_lines(n_read=X, n_pe=Y, n_par=Z, fov=fov, n_tr=n_tr, rf_samples=rf_samples)
    return assemble(rho, t1, t2, spin_num=spins, t2star=0.7 * t2, db0_hz=db0, res=res, model="me",
                    rates=rates, rx=(rxx, rxy), seqlines=lines, tr_num=ntr, seed=seed)


def config5_mt_epi(seed=0, nx=256, ny=256, nz=128, spins=4, n_coils=32, n_read=128, n_pe=128) -> Scan:
    """The roofline stress case: ``ny x nx x nz`` voxels, ``spins`` spins,
    three pools in the general model -- free water (T1 1.0 s, T2 80 ms),
    myelin water (T1 0.4 s, T2 12 ms, fraction U(0, 0.2)) and a bound
    macromolecular pool (T1 1 s, T2 12 us, super-Lorentzian, fraction
    U(0.05, 0.15)) -- exchanging at U(1, 50) /s (pools -> free water;
    the reverse rates by detailed balance), dB0 ~ N(0, 20 Hz), T2* = 0.7 T2
    for the intravoxel dephasing, ``n_coils`` Rx coils on a cylinder;
    single-shot EPI (``n_pe`` x ``n_read`` at 250 kHz) after an 8 ms
    off-resonance MT pulse."""
    rng = np.random.default_rng(seed)
    Y, X, Z = ny, nx, nz
    yy, xx = np.mgrid[0:Y, 0:X]
    r = np.hypot((xx - (X - 1) / 2) / (X / 2), (yy - (Y - 1) / 2) / (Y / 2))
    inside = np.repeat((r <= 0.9)[..., None], Z, axis=2)
    fm = rng.uniform(0.0, 0.2, (Y, X, Z)).astype(np.float32)
    fb = rng.uniform(0.05, 0.15, (Y, X, Z)).astype(np.float32)
    rho = np.stack([1 - fm - fb, fm, fb], -1) * inside[..., None]
    t1 = np.stack([np.full((Y, X, Z), 1.0), np.full((Y, X, Z), 0.4), np.full((Y, X, Z), 1.0)], -1) * inside[..., None]
    t2 = np.stack([np.full((Y, X, Z), 0.08), np.full((Y, X, Z), 0.012), np.full((Y, X, Z), 12e-6)], -1) * inside[..., None]
    rates = np.zeros((Y, X, Z, 3, 3), np.float32)
    for p in (1, 2):
        k = rng.uniform(1.0, 50.0, (Y, X, Z)).astype(np.float32)
        rates[..., p, 0] = np.where(inside, k, 0.0)
        with np.errstate(divide="ignore", invalid="ignore"):
            rates[..., 0, p] = np.where(inside, k * rho[..., p] / np.maximum(rho[..., 0], 1e-6), 0.0)
    db0 = rng.normal(0.0, 20.0, (Y, X, Z)).astype(np.float32)
    fov = (0.24, 0.24 * Y / X, 0.24 * Z / X)
    res = (fov[0] / X, fov[1] / Y, fov[2] / Z)
    rxx, rxy = _cylinder_coils((Y, X, Z), res, n_coils, rng)
    lines, ntr = epi_lines(n_read=n_read, n_pe=n_pe, fov=fov)
    return assemble(rho.astype(np.float32), t1.astype(np.float32), t2.astype(np.float32), spin_num=spins,
                    t2star=0.7 * t2, db0_hz=db0, res=res, model="gm", rates=rates,
                    type_flag=np.array([0.0, 0.0, 1.0]), rx=(rxx, rxy), seqlines=lines, tr_num=ntr, seed=seed)


def crop(sc: Scan, ys, xs, zs) -> Scan:
    """The scan restricted to the voxels at rows ``ys``, columns ``xs`` and
    slices ``zs`` (index arrays or slices), each keeping its position, maps,
    coil sensitivities and state.  Voxels are independent in the engine
    (pool exchange is within a voxel), so the cropped scan's signal is the
    full scan's signal minus the other voxels' contributions: a subset of
    the same workload, for checks at full sequence length."""
    out = sc.copy()
    ix = np.ix_(np.arange(sc.dims[0])[ys], np.arange(sc.dims[1])[xs], np.arange(sc.dims[2])[zs])

    def cut(a):
        a = np.asarray(a)
        return np.asfortranarray(a[ix]) if a.ndim >= 3 else a

    for d, keys in ((out.VObj, ("Rho", "T1", "T2", "K", "Mx", "My", "Mz")),
                    (out.VMag, ("dB0", "dWRnd", "Gzgrid", "Gygrid", "Gxgrid")),
                    (out.VCoi, ("TxCoilmg", "TxCoilpe", "RxCoilx", "RxCoily")),
                    (out.VSig, ("Mx", "My", "Mz"))):
        for k in keys:
            if k in d:
                d[k] = cut(d[k])
    if out.rates is not None:
        out.rates = out.rates[ix]
    out.info = dict(sc.info, crop=True)
    return out


def config2_subset(seed=0, step=8, offset=4, n_tr=None) -> Scan:
    """The two-pool multi-echo GRE benchmark scan (config2_me_gre at its
    full 128 x 128 x 32 size and full sequence length) restricted to every
    ``step``-th row and column from ``offset``, all slices: 16 x 16 x 32
    voxels spread over the field of view by default, the whole 256-TR
    sequence, all 8 Rx coils."""
    sc = config2_me_gre(seed=seed, n_tr=n_tr)
    return crop(sc, slice(offset, None, step), slice(offset, None, step), slice(None))


def sar_case(seed=0, n=16, nz=2, tx_coils=2, n_tr=3, sample_fracs=(0.0, 0.3, 0.5, 0.8, 1.0)) -> Scan:
    """A local-SAR calculation as the SAR watcher sets it up
    (Src/Main/DoSARWatchExec.m:36-105): an n x n x nz object with a mass
    density and per-component conductivity factors (VObj.MassDen, ECon), a
    seeded smooth E-field map per Tx coil and component (VCoi.TxE1x/y/z,
    per unit rf amplitude), a GRE transmitting on ``tx_coils`` coils, and
    sample times at the given fractions of the sequence's length
    (VSig.tSample, unique and sorted; VSig.SAR / tRealSample / Muts and
    VVar.SAR / SARi zeroed)."""
    rng = np.random.default_rng(seed)
    Y = X = n
    Z = nz
    yy, xx, zz = np.meshgrid(np.arange(Y), np.arange(X), np.arange(Z), indexing="ij")
    r = np.hypot((xx - (X - 1) / 2) / (X / 2), (yy - (Y - 1) / 2) / (Y / 2))
    inside = r <= 0.9
    massden = np.where(inside, rng.uniform(900.0, 1100.0, (Y, X, Z)), 0.0).astype(np.float32)
    econ = np.stack([np.where(inside, rng.uniform(0.3, 0.7, (Y, X, Z)), 0.0) for _ in range(3)], -1)
    # E-field per unit rf amplitude (V/m per T): smooth fields, one per coil and component
    e1 = []
    for comp in range(3):
        maps = []
        for c in range(tx_coils):
            ph = 2 * np.pi * rng.uniform()
            kx, ky = rng.uniform(0.5, 1.5, 2)
            maps.append(4e5 * (0.3 + np.cos(np.pi * kx * xx / X + ph) * np.sin(np.pi * ky * yy / Y + 0.4 * c)
                               + 0.1 * zz / max(Z, 1)))
        e1.append(np.stack(maps, -1).astype(np.float32))
    lines, ntr = gre_lines(n_read=16, n_pe=max(n_tr, 1), fov=(0.24, 0.24, 0.24), tr_ms=20.0, te_ms=(5.0,),
                           flip=30.0, rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0, n_tr=n_tr,
                           tx_coils=tx_coils)
    uts = lines["utsLine"]
    d = np.diff(uts)
    t_end = float(np.sum(d[d > 0]))
    t_sample = np.unique(np.asarray(sample_fracs, np.float64) * t_end)
    vobj = dict(MassDen=np.asfortranarray(massden), ECon=np.asfortranarray(econ.astype(np.float32)))
    vcoi = dict(TxE1x=np.asfortranarray(e1[0]), TxE1y=np.asfortranarray(e1[1]), TxE1z=np.asfortranarray(e1[2]),
                TxCoilNum=np.int32(tx_coils))
    vctl = dict(TRNum=np.int32(ntr), MaxThreadNum=np.int32(1))
    vvar = dict(t=np.float64(0), dt=np.float64(0), rfAmp=np.zeros(tx_coils), rfPhase=np.zeros(tx_coils),
                rfFreq=np.zeros(tx_coils), rfCoil=np.float64(0), Ext=np.float64(0),
                SAR=np.asfortranarray(np.zeros((Y, X, Z, 3), np.float32)), SARi=np.int32(0), utsi=np.int32(0),
                rfi=np.int32(0), Exti=np.int32(0), TRCount=np.int32(1))
    vsig = dict(SAR=np.asfortranarray(np.zeros((Y, X, Z, t_sample.size), np.float32)), Muts=np.zeros(uts.size),
                tSample=t_sample, tRealSample=np.zeros(t_sample.size))
    return Scan(vobj, {}, vcoi, vctl, dict(lines), vvar, vsig, model="sar", info=dict(seed=seed))
