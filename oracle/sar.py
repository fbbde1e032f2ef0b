"""CPU oracle of the local-SAR engine -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm may use this module, and only as the reference
results or the timed CPU baseline; the product never imports it.

``run_sar_port`` restates the reference's SAR engine,
``Lib/src/engine/CPUEngine/DoCalSARAtCPU.cpp:185-353`` (the sequence walk:
equal-time flag merge, sample checks before and after every step, rf hold,
packet reset, TR boundaries, early return) with its power kernel
``SARKernel.h:17-56`` as numpy arithmetic over the voxels: ``"f32"`` in the
reference's single-precision operation order, ``"f64"`` in double precision.
``run_ref_sar`` runs the reference engine itself, compiled unmodified from
the reference tree into ``_ref/DoCalSARAtCPU.so`` against the project's
mex / IPP stand-ins (available where the reference tree is mounted).
"""
from __future__ import annotations

import os
from typing import Dict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SAR_SO = os.path.join(HERE, "_ref", "DoCalSARAtCPU.so")


def ref_sar_available() -> bool:
    return os.path.exists(REF_SAR_SO)


def run_sar_port(sc, precision: str = "f32") -> Dict[str, np.ndarray]:
    """The reference SAR engine on the host; outputs as mrilab_gb300.sar.sar."""
    ft = np.float32 if precision == "f32" else np.float64
    o, c, q, v, sig = sc.VObj, sc.VCoi, sc.VSeq, sc.VVar, sc.VSig
    tx = int(c["TxCoilNum"])
    V = int(np.prod(o["MassDen"].shape))
    E = [np.asarray(c[k], np.float32).reshape(V, tx, order="F").T.astype(ft) for k in ("TxE1x", "TxE1y", "TxE1z")]
    econ = np.asarray(o["ECon"], np.float32).reshape(V, 3, order="F").T.astype(ft)
    acc = np.asarray(v["SAR"], np.float32).reshape(V, 3, order="F").T.astype(ft).copy()
    ns = int(np.size(sig["tSample"]))
    sar = np.asarray(sig["SAR"], np.float32).reshape(V, ns, order="F").T.astype(ft).copy()
    muts = np.asarray(sig["Muts"], np.float64).ravel().copy()
    t_sample = np.asarray(sig["tSample"], np.float64).ravel()
    t_real = np.asarray(sig["tRealSample"], np.float64).ravel().copy()
    ts, uts, flags = q["tsLine"].ravel(), q["utsLine"].ravel(), np.asarray(q["flagsLine"]).ravel(order="F")
    rf_amp, rf_ph, rf_fr, rf_coil = (q["rfAmpLine"].ravel(), q["rfPhaseLine"].ravel(), q["rfFreqLine"].ravel(),
                                     q["rfCoilLine"].ravel())
    n_ts, n_uts, n_rf = ts.size, uts.size, rf_amp.size
    utsi, rfi, trc, sari = int(v["utsi"]), int(v["rfi"]), int(v["TRCount"]), int(v["SARi"])
    amp = np.asarray(v["rfAmp"], np.float64).ravel().copy()

    def sample():
        nonlocal sari
        if sari < ns:
            if muts[utsi] >= t_sample[sari]:
                s = sar[sari]
                for k in range(3):  # rounded product, then rounded sum
                    s += (acc[k] * econ[k]).astype(ft)
                t_real[sari] = muts[utsi]
                sari += 1
            if sari == ns:
                return False
        return True

    i = 0
    while i < n_ts - 1:
        flag = np.zeros(6)
        if ts[i] != ts[i + 1]:
            flag += flags[i * 6:i * 6 + 6]
            i += 1
        else:
            flag += flags[i * 6:i * 6 + 6]
            while ts[i] == ts[i + 1]:
                flag += flags[(i + 1) * 6:(i + 1) * 6 + 6]
                i += 1
                if i == n_ts - 1:
                    break
            i += 1
        if not sample():
            break
        nxt = min(utsi + 1, n_uts - 1)
        dt = uts[nxt] - uts[utsi]
        utsi = nxt
        if flag[0] >= 1:
            for _ in range(int(np.ceil(flag[0]))):
                if rfi >= n_rf:
                    break
                coil = rf_coil[rfi]
                for s in range(rfi + 1, n_rf):
                    if rf_coil[s] == coil:
                        txi = int(coil)
                        if 1 <= txi <= tx:
                            amp[txi - 1] = rf_amp[rfi] if abs(rf_amp[rfi]) <= abs(rf_amp[s]) else rf_amp[s]
                        break
                rfi += 1
        if flag.sum() == 0:
            amp[:] = 0
        if dt == 0:
            continue
        if dt < 0:
            trc += 1
            muts[utsi] = muts[utsi - 1]
            continue
        if np.sum(np.abs(amp.astype(np.float32))) != 0:
            for k in range(3):
                b = np.zeros(V, ft)
                for cc in range(tx):
                    a = ft(np.float32(amp[cc])) if precision == "f32" else amp[cc]
                    if a != 0:
                        b += (E[k][cc] * a).astype(ft)
                sq = (b * b).astype(ft)
                acc[k] += (sq * (ft(np.float32(dt)) if precision == "f32" else dt)).astype(ft)
        muts[utsi] = muts[utsi - 1] + dt
        if not sample():
            break
    return dict(SAR=sar.ravel().astype(np.float64), SARacc=acc.ravel().astype(np.float64), Muts=muts,
                tRealSample=t_real, SARi=sari, utsi=utsi, rfi=rfi, TRCount=trc)


def run_ref_sar(sc) -> Dict[str, np.ndarray]:
    """The reference SAR engine (DoCalSARAtCPU), compiled from its source,
    through the mex stand-in; outputs as run_sar_port."""
    from mrilab_gb300 import mexsim

    ms = mexsim.MexSession()
    for name, fields in sc.structs().items():
        if fields:
            ms.set_global(name, fields)
    ms.call(REF_SAR_SO)
    V = int(np.prod(sc.VObj["MassDen"].shape))
    ns = int(np.size(sc.VSig["tSample"]))
    sar = ms.get("VSig", "SAR").ravel(order="F").reshape(ns, V)
    acc = ms.get("VVar", "SAR").ravel(order="F").reshape(3, V)
    return dict(SAR=sar.ravel().astype(np.float64), SARacc=acc.ravel().astype(np.float64),
                Muts=ms.get("VSig", "Muts").ravel(order="F").copy(),
                tRealSample=ms.get("VSig", "tRealSample").ravel(order="F").copy(),
                SARi=int(ms.get("VVar", "SARi").ravel()[0]), utsi=int(ms.get("VVar", "utsi").ravel()[0]),
                rfi=int(ms.get("VVar", "rfi").ravel()[0]), TRCount=int(ms.get("VVar", "TRCount").ravel()[0]))
