"""FP64 reference gradient of the scan -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` use this module, as the reference the adjoint kernel is
compared with.  The
C oracle's discrete map (``port/mrl_port_impl.h``, the reference's
algorithm: ``BlochKernel.h:38-368`` for the normal model,
``BlochKernelME.cuh:154-343`` and ``BlochKernelGM.cuh:159-471`` for the
exchange models, receive ``DoScanAtCPU.cpp:445-491``) is restated step by
step in float64 PyTorch on the CPU, vectorised over isochromats, and
differentiated by reverse-mode automatic differentiation: a double-precision
gradient derived independently of the hand-written adjoint.  The steps are
the C oracle's own decode (``run_port(..., step_records=N)``), so both walk
the same step list.  The autograd graph holds every step: small cases only.

Models: normal, ME and GM (GM pools of TypeFlag 0 and 1) as the adjoint
kernel covers them, and MT and CEST (``BlochKernelMT.cuh:180-411``,
``BlochKernelCEST.cuh:280-606``: pool 0 free water, pool 1 the bound pool,
CEST pools exchanging with pool 0).  Several transmit coils (free-pool
models): an rf step's field is the sum over the coils that are on of
TxCoil_c A_c and its frequency term the sum of their frequencies
(``BlochKernel.h:57-122``; the port's ``rotate``); the rf gradient is per
step and coil.
"""
from __future__ import annotations

from typing import Dict

import numpy as np
import torch

from . import run_port

PI = 3.14159265359  # the reference's constant


def _flat(arr) -> np.ndarray:
    return np.asarray(arr).ravel(order="F").astype(np.float32).astype(np.float64)


def _lineshape(freq: float, db0: torch.Tensor, gyro: float, t2b: torch.Tensor) -> torch.Tensor:
    """Super-Lorentzian lineshape of a bound pool, the oracle's 1000-point
    rule (BlochKernelMT.cuh:348-358), per voxel."""
    u = torch.arange(1000, dtype=torch.float64) * 0.001
    den = 3 * u * u - 1
    x = ((2 * PI * freq + db0 * gyro) * t2b)[:, None] / den
    return (np.sqrt(2 / PI) * t2b[:, None] / den.abs() * torch.exp(-2 * x * x) * 0.001).sum(-1)


def _rotate(x, y, z, vx, vy, vz):
    """exp([v]x) m by Rodrigues' formula, with the series of sin a / a and
    (1 - cos a) / a^2 near a = 0 (kept off the division there, so the
    gradient stays finite)."""
    a2 = vx * vx + vy * vy + vz * vz
    small = a2 < 1e-8
    a2s = torch.where(small, torch.ones_like(a2), a2)
    a = torch.sqrt(a2s)
    s1 = torch.where(small, 1 - a2 / 6, torch.sin(a) / a)
    s2 = torch.where(small, 0.5 - a2 / 24, (1 - torch.cos(a)) / a2s)
    cx, cy, cz = vy * z - vz * y, vz * x - vx * z, vx * y - vy * x  # v x m
    dx, dy, dz = vy * cz - vz * cy, vz * cx - vx * cz, vx * cy - vy * cx  # v x (v x m)
    return x + s1 * cx + s2 * dx, y + s1 * cy + s2 * dy, z + s1 * cz + s2 * dz


def _mt_cest_step(model, P, S, dt, rf, X, Y, Z, xr, yr, zr, T1, T2, Rho, K, on, b1, freq, dB0, gyro):
    """One step of the MT / CEST maps (the oracle's, BlochKernelMT.cuh:324-407,
    BlochKernelCEST.cuh:364-600): pool 0 free water exchanging with the
    bound pool 1 (K12 free -> bound, K21 back) and, for CEST, with pools
    2..P-1, each rotated at its own frequency; the bound pool saturated by
    rf (W = pi (gamma b1)^2 G), then relaxed.  An isochromat whose pool 0 is
    empty is left alone.  (xr, yr, zr): every pool's rotated state."""
    ex = torch.exp
    if model == "mt":
        K12, K21 = K[1], K[2]
    else:
        K12, K21 = K[0], K[P - 1]
    x0, y0, z0, zb0 = X[0], Y[0], Z[0], Z[1]
    e2 = ex(-dt / T2[0])
    e1k = ex(-dt / T1[0] - dt * K12)
    m0 = Rho[0] * (1 - ex(-dt / T1[0])) / S
    ek = 1 - ex(-dt * K21)
    nx, ny, nz = [None] * P, [None] * P, [None] * P
    if model == "mt":
        nx[0], ny[0], nz[0] = xr[0] * e2, yr[0] * e2, zr[0] * e1k + m0 + zb0 * ek
    else:
        kout = torch.ones_like(e2)
        kx, ky, kz = torch.zeros_like(x0), torch.zeros_like(x0), torch.zeros_like(x0)
        for t in range(2, P):
            kout = kout * ex(-dt * K[t - 1])
            f = 1 - ex(-dt * K[t + P - 2])
            kx, ky, kz = kx + f * X[t], ky + f * Y[t], kz + f * Z[t]
        nx[0] = xr[0] * e2 * kout + kx
        ny[0] = yr[0] * e2 * kout + ky
        nz[0] = zr[0] * e1k * kout + kz + zb0 * ek + m0
        for t in range(2, P):
            c2, c1 = ex(-dt / T2[t]), ex(-dt / T1[t])
            ko = ex(-dt * K[t + P - 2])
            f = 1 - ex(-dt * K[t - 1])
            nx[t] = xr[t] * c2 * ko + f * x0
            ny[t] = yr[t] * c2 * ko + f * y0
            nz[t] = zr[t] * c1 * ko + f * z0 + Rho[t] * (1 - c1) / S
    bz = Z[1]
    if rf:
        W = PI * (b1 * gyro) ** 2 * _lineshape(freq, dB0, gyro, T2[1])
        bz = bz * ex(-W * dt)
    nz[1] = bz * ex(-dt / T1[1] - dt * K21) + Rho[1] * (1 - ex(-dt / T1[1])) / S + z0 * (1 - ex(-dt * K12))
    nx[1], ny[1] = X[1], Y[1]
    act = on[0][None].expand_as(x0)
    return (torch.stack([torch.where(act, a, b) for a, b in zip(nx, X)]),
            torch.stack([torch.where(act, a, b) for a, b in zip(ny, Y)]),
            torch.stack([torch.where(act, a, b) for a, b in zip(nz, Z)]))


def gradients(sc, grad_sx, grad_sy) -> Dict[str, np.ndarray]:
    """dL/dtheta of L = sum(grad_sx * Sx + grad_sy * Sy) over the scan's
    signal (so its gradient is the adjoint's for those dL/dS), in the
    adjoint's layouts: T1, T2, Rho [P*V], dB0 [V], K [nK*V], Mx0, My0, Mz0
    [P*S*V], rf [n_rf, 2] (dL/dRe A, dL/dIm A of each rf-on step; [n_rf,
    Tx, 2] with several Tx coils), plus Sx, Sy (the signal of the restated
    map)."""
    o, mag, coil, ctl = sc.VObj, sc.VMag, sc.VCoi, sc.VCtl
    model = sc.model
    if model not in ("normal", "me", "gm", "mt", "cest"):
        raise ValueError("unknown model")
    P, S = int(o["TypeNum"]), int(o["SpinNum"])
    TX, RX = int(coil["TxCoilNum"]), int(coil["RxCoilNum"])
    if TX > 1 and (model in ("mt", "cest") or
                   (model == "gm" and np.any(np.asarray(o["TypeFlag"], np.float64).ravel() == 1))):
        raise ValueError("several transmit coils: free-pool models only")
    A = int(sc.VSig["SignalNum"])
    V = int(np.asarray(o["Rho"]).size // P)
    gyro = float(o["Gyro"])
    n = run_port(sc, "f64")["steps"]
    rec = run_port(sc, "f64", step_records=max(n, 1))["records"]

    def leaf(a):
        return torch.tensor(a, dtype=torch.float64, requires_grad=True)

    T1 = leaf(_flat(o["T1"]).reshape(P, V))
    T2 = leaf(_flat(o["T2"]).reshape(P, V))
    Rho = leaf(_flat(o["Rho"]).reshape(P, V))
    dB0 = leaf(_flat(mag["dB0"]))
    has_k = model != "normal"
    K = leaf(_flat(o["K"]).reshape(-1, V)) if has_k else None
    Mx0 = leaf(_flat(o["Mx"]).reshape(P, S, V))
    My0 = leaf(_flat(o["My"]).reshape(P, S, V))
    Mz0 = leaf(_flat(o["Mz"]).reshape(P, S, V))
    rf_on = rec[:, 7] != 0
    # per rf step and coil: amplitude, phase, frequency (coil 0 in columns
    # 4-6, coil c >= 1 in 10 + 3 (c - 1) ...)
    cols = [(4, 5, 6)] + [(10 + 3 * (c - 1), 11 + 3 * (c - 1), 12 + 3 * (c - 1)) for c in range(1, TX)]
    amp = np.stack([rec[rf_on, ca] for ca, _, _ in cols], 1)  # [n_rf, TX]
    ph = np.stack([rec[rf_on, cp] for _, cp, _ in cols], 1)
    frq = np.stack([rec[rf_on, cf] for _, _, cf in cols], 1)
    rfa = leaf(np.stack([amp * np.cos(ph), amp * np.sin(ph)], 2))  # [n_rf, TX, 2]

    t = lambda a: torch.tensor(a, dtype=torch.float64)
    dwr = t(_flat(mag["dWRnd"]).reshape(P, S, V))
    gzg, gyg, gxg = (t(_flat(mag[k])) for k in ("Gzgrid", "Gygrid", "Gxgrid"))
    mg_all, pe_all = t(_flat(coil["TxCoilmg"]).reshape(-1, V)), t(_flat(coil["TxCoilpe"]).reshape(-1, V))
    mg, pe = mg_all[0], pe_all[0]
    txc_re_all, txc_im_all = mg_all * torch.cos(pe_all), mg_all * torch.sin(pe_all)  # [TX, V]
    if float(coil["RxCoilDefault"]) == 0:
        rxr, rxi = t(_flat(coil["RxCoilx"]).reshape(RX, V)), t(_flat(coil["RxCoily"]).reshape(RX, V))
    else:
        rxr, rxi = torch.ones(RX, V, dtype=torch.float64), torch.zeros(RX, V, dtype=torch.float64)
    cs = np.asarray(ctl["CS"], np.float64).ravel()
    kind = np.zeros(P, int) if model != "gm" else np.asarray(o["TypeFlag"], np.float64).ravel().astype(int)
    mtc = model in ("mt", "cest")
    # pools the receiver samples: the free pools; MT / CEST: pool 0 only
    sampled = [(tp == 0) if mtc else kind[tp] == 0 for tp in range(P)]
    rf_ref = float(sc.VVar["rfRef"])
    gx_t = t(np.asarray(grad_sx, np.float64).reshape(P, RX, A))
    gy_t = t(np.asarray(grad_sy, np.float64).reshape(P, RX, A))

    on = ((T1 != 0) & (T2 != 0) & (Rho != 0)).detach()  # [P, V]
    T1s = torch.where(on, T1, torch.ones_like(T1))
    T2s = torch.where(on, T2, torch.ones_like(T2))
    if has_k:
        def kgo(a, b):  # rate a -> b (ME channel a*P+b, GM b*P+a)
            return K[a * P + b] if model == "me" else K[b * P + a]

    X, Y, Z = Mx0, My0, Mz0
    loss = torch.zeros((), dtype=torch.float64)
    sig_x = torch.zeros(P, RX, A, dtype=torch.float64)
    sig_y = torch.zeros(P, RX, A, dtype=torch.float64)
    cr, sr = np.cos(-rf_ref), np.sin(-rf_ref)
    ri = 0
    for r in rec:
        dt, gz, gy, gx, _, _, freq, rf_sum, adc, sidx = (float(q) for q in r[:10])
        if adc and int(sidx) < A:
            # receive before the step: sum over spins and voxels of m conj(R_c)
            for tp in range(P):
                if not sampled[tp]:
                    continue
                mx, my = X[tp].sum(0), Y[tp].sum(0)  # [V]
                b1 = (mx[None] * rxr + my[None] * rxi).sum(1)  # [RX]
                b3 = (my[None] * rxr - mx[None] * rxi).sum(1)
                if rf_ref != 0:
                    b1, b3 = b1 * cr - b3 * sr, b1 * sr + b3 * cr
                a = int(sidx)
                loss = loss + (gx_t[tp, :, a] * b1).sum() + (gy_t[tp, :, a] * b3).sum()
                sig_x[tp, :, a] = b1.detach()
                sig_y[tp, :, a] = b3.detach()
        w = (dB0 * gyro)[None, None] + dwr + t(2 * PI * cs)[:, None, None] \
            + (gzg * (gz * gyro) + gyg * (gy * gyro) + gxg * (gx * gyro))[None, None]
        rf = rf_sum != 0
        if rf:
            # the field of the coils that are on (TX = 1: coil 0, on whenever rf is)
            bre = torch.zeros(V, dtype=torch.float64)
            bim = torch.zeros(V, dtype=torch.float64)
            fsum = 0.0
            for c in range(TX):
                if TX > 1 and amp[ri, c] == 0:
                    continue
                Arc, Aic = rfa[ri, c, 0], rfa[ri, c, 1]
                bre = bre + txc_re_all[c] * Arc - txc_im_all[c] * Aic
                bim = bim + txc_re_all[c] * Aic + txc_im_all[c] * Arc
                fsum += float(frq[ri, c])
            Ar, Ai = rfa[ri, 0, 0], rfa[ri, 0, 1]
            ri += 1
            vx = (-dt * gyro) * bre
            vy = (-dt * gyro) * bim
            vz = -dt * (w + 2 * PI * fsum)
            xr, yr, zr = _rotate(X, Y, Z, vx[None, None].expand_as(X), vy[None, None].expand_as(X), vz)
        else:
            zero = torch.zeros_like(X)
            xr, yr, zr = _rotate(X, Y, Z, zero, zero, -dt * w)
        if mtc:
            X, Y, Z = _mt_cest_step(model, P, S, dt, rf, X, Y, Z, xr, yr, zr, T1s, T2s, Rho, K, on,
                                    (mg * torch.sqrt(Ar * Ar + Ai * Ai)) if rf else None, freq, dB0, gyro)
            continue
        nx, ny, nz = [], [], []
        for tp in range(P):
            e1 = torch.exp(torch.clamp(-dt / T1s[tp], min=-200.0))[None]
            e2 = torch.exp(torch.clamp(-dt / T2s[tp], min=-200.0))[None]
            m0 = (Rho[tp] * (1 - e1[0]) / S)[None]
            act = on[tp][None].expand(S, V)
            if model == "normal":
                x1, y1, z1 = xr[tp] * e2, yr[tp] * e2, zr[tp] * e1 + m0
            elif kind[tp] not in (0, 1):
                x1, y1, z1 = X[tp], Y[tp], Z[tp]
            else:
                ksum = torch.zeros(V, dtype=torch.float64)
                ix = torch.zeros(S, V, dtype=torch.float64)
                iy = torch.zeros(S, V, dtype=torch.float64)
                iz = torch.zeros(S, V, dtype=torch.float64)
                for p in range(P):
                    if model == "gm" and p == tp:
                        continue
                    ksum = ksum + kgo(tp, p)
                    f = 1 - torch.exp(-dt * kgo(p, tp))[None]
                    if kind[tp] == 0:
                        ix = ix + f * X[p]
                        iy = iy + f * Y[p]
                    iz = iz + f * Z[p]
                kout = torch.exp(-dt * ksum)[None]
                if kind[tp] == 0:
                    x1, y1 = xr[tp] * e2 * kout + ix, yr[tp] * e2 * kout + iy
                    zb = zr[tp]
                else:
                    x1, y1 = X[tp], Y[tp]
                    zb = Z[tp]
                    if rf:
                        b1 = mg * torch.sqrt(Ar * Ar + Ai * Ai)
                        W = PI * (b1 * gyro) ** 2 * _lineshape(freq, dB0, gyro, T2s[tp])
                        zb = zb * torch.exp(-W * dt)[None]
                z1 = zb * e1 * kout + iz + m0
            nx.append(torch.where(act, x1, X[tp]))
            ny.append(torch.where(act, y1, Y[tp]))
            nz.append(torch.where(act, z1, Z[tp]))
        X, Y, Z = torch.stack(nx), torch.stack(ny), torch.stack(nz)
    loss.backward()

    def g(x):
        return np.zeros(0) if x is None or x.grad is None else x.grad.numpy().ravel().copy()

    out = dict(T1=g(T1), T2=g(T2), Rho=g(Rho), dB0=g(dB0), Mx0=g(Mx0), My0=g(My0), Mz0=g(Mz0),
               rf=(rfa.grad.numpy().copy() if rfa.grad is not None else np.zeros((0, TX, 2))) if TX > 1 else
               (rfa.grad.numpy()[:, 0].copy() if rfa.grad is not None else np.zeros((0, 2))),
               Sx=sig_x.numpy().ravel(), Sy=sig_y.numpy().ravel())
    if has_k:
        out["K"] = g(K)
    return out
