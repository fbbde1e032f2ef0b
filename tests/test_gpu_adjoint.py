"""The adjoint (mrl_adjoint) against central finite differences of the
all-FP64 oracle's forward scan, L = sum |S - target|^2.

Tissue parameters and the initial magnetisation: the whole gradient vector
against the FP64 finite-difference gradient taken one element at a time
(step h = 1e-3 relative to the element), norm-wise.  The rf waveform: the
directional derivatives along "scale every amplitude by 1 + h" and "shift
every phase by h"."""
import numpy as np
import pytest

import oracle
from mrilab_gb300 import engine, phantoms

pytestmark = pytest.mark.gpu

H = 1e-3
# relative error bound (FP32 adjoint vs FP64 central differences)
TOL = 1e-3
# dB0 is zero in many voxels: its finite-difference step is absolute, and
# small, because the loss is strongly curved in it (1e-9 T moves the phase
# by 0.27 rad/s: differences of 1e-9 and 4e-9 T already disagree by 0.7 %,
# of 1e-10 and 2e-10 T by 1.5e-5)
DB0_STEP = 1e-10  # T


def _loss(sc, target):
    out = oracle.run_port(sc, "f64")
    rx, ry = out["Sx"] - target[0], out["Sy"] - target[1]
    return float(np.sum(rx * rx + ry * ry)), 2 * rx, 2 * ry


def _with(sc, struct, key, flat):
    """A copy of sc with struct[key] replaced by `flat` (column-major)."""
    out = sc.copy()
    d = getattr(out, struct)
    d[key] = np.asfortranarray(np.asarray(flat, d[key].dtype).reshape(d[key].shape, order="F"))
    return out


def _fd_gradient(sc, target, struct, key, idx, steps):
    """Central differences of L, one element at a time.  The parameters are
    stored in single precision: the step actually taken is used."""
    arr = getattr(sc, struct)[key]
    base = np.asarray(arr, np.float64).ravel(order="F")
    g = np.zeros(len(idx))
    for j, (i, h) in enumerate(zip(idx, steps)):
        plus, minus = base.copy(), base.copy()
        plus[i] = np.float64(arr.dtype.type(base[i] + h))
        minus[i] = np.float64(arr.dtype.type(base[i] - h))
        lp, _, _ = _loss(_with(sc, struct, key, plus), target)
        lm, _, _ = _loss(_with(sc, struct, key, minus), target)
        g[j] = (lp - lm) / (plus[i] - minus[i])
    return g


def _check(label, adj, fd):
    err = float(np.linalg.norm(adj - fd) / np.linalg.norm(fd))
    print(f"{label}: |grad| {np.linalg.norm(fd):.4e}, relative error {err:.2e} over {fd.size} elements")
    assert err <= TOL


def _target(sc):
    # the signal of the same object with T1 and T2 5 % longer
    t = sc.copy()
    t.VObj["T1"] = np.asfortranarray(t.VObj["T1"] * np.float32(1.05))
    t.VObj["T2"] = np.asfortranarray(t.VObj["T2"] * np.float32(1.05))
    out = oracle.run_port(t, "f64")
    return out["Sx"], out["Sy"]


def _run(sc):
    target = _target(sc)
    _, gsx, gsy = _loss(sc, target)
    g = engine.adjoint(sc, gsx, gsy)
    o = sc.VObj
    P = int(o["TypeNum"])
    act = ((o["Rho"] != 0) & (o["T1"] != 0) & (o["T2"] != 0)).ravel(order="F")
    for key in ("T1", "T2", "Rho"):
        p = np.asarray(o[key], np.float64).ravel(order="F")
        idx = np.flatnonzero(act)
        _check(key, g[key][idx], _fd_gradient(sc, target, "VObj", key, idx, H * np.abs(p[idx])))
    vidx = np.flatnonzero(act.reshape(-1, P, order="F").any(axis=1))
    _check("dB0", g["dB0"][vidx], _fd_gradient(sc, target, "VMag", "dB0", vidx, np.full(vidx.size, DB0_STEP)))
    mz = np.asarray(o["Mz"], np.float64).ravel(order="F")
    idx = np.flatnonzero(mz)
    _check("Mz0", g["Mz0"][idx], _fd_gradient(sc, target, "VObj", "Mz", idx, H * np.abs(mz[idx])))
    if "K" in g:
        k = np.asarray(o["K"], np.float64).ravel(order="F")
        idx = np.flatnonzero(k)
        _check("K", g["K"][idx], _fd_gradient(sc, target, "VObj", "K", idx, H * np.abs(k[idx])))
    # rf: scale every amplitude by (1 + h): dA/dh = A; shift every phase by h: dA/dh = i A
    a, grf = g["rf_a"], g["rf"]
    amp = np.asarray(sc.VSeq["rfAmpLine"], np.float64).ravel()
    lp, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", amp * (1 + H)), target)
    lm, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", amp * (1 - H)), target)
    fd = (lp - lm) / (2 * H)
    adj = float(np.sum(grf[:, 0] * a[:, 0] + grf[:, 1] * a[:, 1]))
    print(f"rf amplitude: adjoint {adj:.6e}, finite difference {fd:.6e}")
    assert abs(adj - fd) <= TOL * abs(fd)
    ph = np.asarray(sc.VSeq["rfPhaseLine"], np.float64).ravel()
    lp, _, _ = _loss(_with(sc, "VSeq", "rfPhaseLine", ph + H), target)
    lm, _, _ = _loss(_with(sc, "VSeq", "rfPhaseLine", ph - H), target)
    fd = (lp - lm) / (2 * H)
    adj = float(np.sum(-grf[:, 0] * a[:, 1] + grf[:, 1] * a[:, 0]))
    print(f"rf phase: adjoint {adj:.6e}, finite difference {fd:.6e}")
    assert abs(adj - fd) <= TOL * abs(fd)
    return g


def test_adjoint_single_pool_gre(built):
    _run(phantoms.config1_gre(seed=31, n=8, n_tr=3))


def test_adjoint_two_pool_exchange(built):
    _run(phantoms.small_multipool("me", seed=32, n=6, pools=2, spins=2, coils=2, n_tr=2))


def test_adjoint_three_pool_exchange(built):
    _run(phantoms.small_multipool("me", seed=34, n=5, pools=3, spins=1, coils=3, n_tr=2))


def test_adjoint_rejects_bound_pools(built):
    sc = phantoms.small_multipool("mt", seed=33, n=4, pools=2, spins=1, coils=1, n_tr=1, seq="sat")
    with pytest.raises(engine.ScanError) as e:
        engine.adjoint(sc, np.zeros(1), np.zeros(1))
    assert e.value.status == -6
