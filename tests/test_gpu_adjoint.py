"""The adjoint (mrl_adjoint) against central finite differences of the
all-FP64 oracle's forward scan: for each parameter family a random
direction d, the adjoint's sum(grad . d) against (L(p + h d) - L(p - h d)) / 2h
with h = 1e-3 relative, L = sum |S - target|^2."""
import numpy as np
import pytest

import oracle
from mrilab_gb300 import engine, phantoms

pytestmark = pytest.mark.gpu

H = 1e-3
# relative error of the directional derivative (FP32 adjoint vs FP64 differences)
TOL = 1e-3


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


def _check(sc, target, struct, key, grad, direction, label):
    arr = getattr(sc, struct)[key]
    base = np.asarray(arr, np.float64).ravel(order="F")
    # the parameters are stored in single precision: the step actually taken
    plus = (base + H * direction).astype(arr.dtype).astype(np.float64)
    minus = (base - H * direction).astype(arr.dtype).astype(np.float64)
    lp, _, _ = _loss(_with(sc, struct, key, plus), target)
    lm, _, _ = _loss(_with(sc, struct, key, minus), target)
    fd = (lp - lm) / (2 * H)
    adj = float(np.dot(grad.astype(np.float64), (plus - minus) / (2 * H)))
    err = abs(adj - fd) / max(abs(fd), 1e-30)
    print(f"{label}: adjoint {adj:.6e}, finite difference {fd:.6e}, relative error {err:.2e}")
    assert err <= TOL


def _target(sc):
    # the signal of the same object with T1 and T2 5 % longer
    t = sc.copy()
    t.VObj["T1"] = np.asfortranarray(t.VObj["T1"] * np.float32(1.05))
    t.VObj["T2"] = np.asfortranarray(t.VObj["T2"] * np.float32(1.05))
    out = oracle.run_port(t, "f64")
    return out["Sx"], out["Sy"]


def _run(sc, check_k):
    rng = np.random.default_rng(7)
    target = _target(sc)
    _, gsx, gsy = _loss(sc, target)
    g = engine.adjoint(sc, gsx, gsy)
    o = sc.VObj
    act = ((o["Rho"] != 0) & (o["T1"] != 0) & (o["T2"] != 0)).ravel(order="F")
    r = lambda n: rng.uniform(-1, 1, n)
    for key in ("T1", "T2", "Rho"):
        p = np.asarray(o[key], np.float64).ravel(order="F")
        _check(sc, target, "VObj", key, g[key], p * r(p.size) * act, key)
    vact = act.reshape(-1, int(o["TypeNum"]), order="F").any(axis=1)
    _check(sc, target, "VMag", "dB0", g["dB0"], 5e-7 * r(vact.size) * vact, "dB0")
    mz = np.asarray(o["Mz"], np.float64).ravel(order="F")
    _check(sc, target, "VObj", "Mz", g["Mz0"], mz * r(mz.size), "Mz0")
    if check_k:
        k = np.asarray(o["K"], np.float64).ravel(order="F")
        _check(sc, target, "VObj", "K", g["K"], k * r(k.size), "K")
    # rf: scale every amplitude by (1 + h): dA/dh = A; shift every phase by h: dA/dh = i A
    a = g["rf_a"]
    amp = np.asarray(sc.VSeq["rfAmpLine"], np.float64).ravel()
    lp, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", amp * (1 + H)), target)
    lm, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", amp * (1 - H)), target)
    fd = (lp - lm) / (2 * H)
    adj = float(np.sum(g["rf"][:, 0] * a[:, 0] + g["rf"][:, 1] * a[:, 1]))
    print(f"rf amplitude: adjoint {adj:.6e}, finite difference {fd:.6e}")
    assert abs(adj - fd) <= TOL * abs(fd)
    ph = np.asarray(sc.VSeq["rfPhaseLine"], np.float64).ravel()
    lp, _, _ = _loss(_with(sc, "VSeq", "rfPhaseLine", ph + H), target)
    lm, _, _ = _loss(_with(sc, "VSeq", "rfPhaseLine", ph - H), target)
    fd = (lp - lm) / (2 * H)
    adj = float(np.sum(-g["rf"][:, 0] * a[:, 1] + g["rf"][:, 1] * a[:, 0]))
    print(f"rf phase: adjoint {adj:.6e}, finite difference {fd:.6e}")
    assert abs(adj - fd) <= TOL * abs(fd)
    return g


def test_adjoint_single_pool_gre(built):
    _run(phantoms.config1_gre(seed=31, n=8, n_tr=3), check_k=False)


def test_adjoint_two_pool_exchange(built):
    _run(phantoms.small_multipool("me", seed=32, n=6, pools=2, spins=2, coils=2, n_tr=2), check_k=True)


def test_adjoint_rejects_bound_pools(built):
    sc = phantoms.small_multipool("mt", seed=33, n=4, pools=2, spins=1, coils=1, n_tr=1, seq="sat")
    with pytest.raises(engine.ScanError) as e:
        engine.adjoint(sc, np.zeros(1), np.zeros(1))
    assert e.value.status == -6
