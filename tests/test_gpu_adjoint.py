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


def _phase_modulated(sc, seed):
    """sc with random rf phases on the rf-on entries: without ties between
    neighbouring |phase| values every entry's phase derivative is two-sided.
    The phases are all positive, so shifting every phase by +-h keeps the
    order of the magnitudes and with it the entries the steps hold."""
    out = sc.copy()
    amp = np.asarray(out.VSeq["rfAmpLine"], np.float64)
    ph = np.asarray(out.VSeq["rfPhaseLine"], np.float64).copy()
    on = amp != 0
    ph[on] = np.random.default_rng(seed).uniform(0.05, 0.45, int(on.sum()))
    out.VSeq["rfPhaseLine"] = ph
    return out


def _untied(v, tol):
    """Entries j of a line whose magnitude differs from both neighbours' by
    more than tol[j] (the held value cannot switch under a step of tol / 4)."""
    a = np.abs(v)
    j = np.arange(1, v.size - 1)
    return j[(np.abs(a[j] - a[j - 1]) > tol[j]) & (np.abs(a[j] - a[j + 1]) > tol[j])]


def _run(sc):
    sc = _phase_modulated(sc, 5)
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
    # single waveform entries (VSeq.rfAmpLine / rfPhaseLine)
    rng = np.random.default_rng(11)
    cand = _untied(amp, 4 * H * np.abs(amp))
    # not the sinc's zero crossings: a relative step there leaves L unchanged
    cand = cand[np.abs(amp[cand]) > 1e-3 * np.abs(amp).max()]
    pick = np.sort(rng.choice(cand, min(24, cand.size), replace=False))
    _check("rfAmpLine", g["rf_amp_line"][pick],
           _fd_gradient(sc, target, "VSeq", "rfAmpLine", pick, H * np.abs(amp[pick])))
    ph = np.asarray(sc.VSeq["rfPhaseLine"], np.float64).ravel()
    cand = _untied(ph, np.full(ph.size, 4 * H))
    cand = cand[(np.abs(ph[cand]) > 4 * H) & (g["rf_phase_line"][cand] != 0)]
    pick = np.sort(rng.choice(cand, min(24, cand.size), replace=False))
    _check("rfPhaseLine", g["rf_phase_line"][pick],
           _fd_gradient(sc, target, "VSeq", "rfPhaseLine", pick, np.full(pick.size, H)))
    return g


def test_adjoint_single_pool_gre(built):
    _run(phantoms.config1_gre(seed=31, n=8, n_tr=3))


def test_adjoint_two_pool_exchange(built):
    _run(phantoms.small_multipool("me", seed=32, n=6, pools=2, spins=2, coils=2, n_tr=2))


def test_adjoint_three_pool_exchange(built):
    _run(phantoms.small_multipool("me", seed=34, n=5, pools=3, spins=1, coils=3, n_tr=2))


def test_adjoint_gm_bound_pool(built):
    """The general model with a bound pool (TypeFlag 1, T2b 10 us) under
    off-resonance Gaussian saturation pulses: the saturation's share of the
    rf gradient, and dB0 and T2b through the lineshape."""
    _run(phantoms.small_multipool("gm", seed=38, n=5, pools=3, spins=1, coils=2, n_tr=3, seq="sat"))


def test_adjoint_mt_model(built):
    """The MT model (free pool + bound pool, K12 / K21 in channels 1 and 2)
    under off-resonance saturation pulses: relaxation, exchange, the bound
    pool's saturation through its lineshape, and the rf waveform, against
    FP64 central differences."""
    _run(phantoms.small_multipool("mt", seed=47, n=5, pools=2, spins=2, coils=2, n_tr=2, seq="sat"))


def test_adjoint_cest_model(built):
    """The CEST model with water, the MT pool and one CEST pool (its own
    chemical shift, exchanging with water only)."""
    _run(phantoms.small_multipool("cest", seed=48, n=5, pools=3, spins=1, coils=2, n_tr=2, seq="sat"))


def test_adjoint_mt_epi_many_coils(built):
    """The MT + exchange EPI (free, myelin and bound pools, 8 ms MT pulse)
    on a small phantom with 12 receive coils."""
    _run(phantoms.config5_mt_epi(seed=5, nx=4, ny=4, nz=1, spins=1, n_coils=12, n_read=8, n_pe=8))


def test_adjoint_two_level_checkpoints(built, monkeypatch):
    """Checkpoints stored every 4 windows (64 steps), the adjoint rebuilding
    each segment's window checkpoints: the gradients of the one-level plan,
    to the FP32 rounding of the rebuilt states."""
    sc = _phase_modulated(phantoms.small_multipool("gm", seed=39, n=5, pools=3, spins=2, coils=3, n_tr=3,
                                                   seq="sat"), 10)
    tx, ty = _target(sc)
    out = engine.scan(sc)
    gx, gy = 2 * (out["Sx"] - tx), 2 * (out["Sy"] - ty)
    one = engine.adjoint(sc, gx, gy)
    for seg in ("4", "3"):
        monkeypatch.setenv("MRL_ADJ_SEGMENT", seg)
        plan = engine.AdjointPlan(sc)
        try:
            ck = plan.checkpoints()
            assert ck["stored_every"] == 16 * int(seg) and ck["window"] == 16
            plan.forward()
            o2 = plan.signal()
            np.testing.assert_array_equal(o2["Sx"], out["Sx"])
            plan.backward(gx, gy)
            g = plan.gradients()
        finally:
            plan.close()
        for k in ("T1", "T2", "Rho", "dB0", "K", "Mz0", "rf"):
            a, b = np.asarray(g[k], np.float64), np.asarray(one[k], np.float64)
            err = float(np.linalg.norm(a - b) / np.linalg.norm(b))
            print(f"segment {seg}: {k} relative difference {err:.2e}")
            assert err <= 1e-4


@pytest.mark.parametrize("case", ["gre", "me3", "gm_bound", "bssfp", "mt", "cest3", "tx2", "tx3", "mt_epi_s4",
                                  "me3_s2_rx8", "me1_s4_rx8"])
def test_adjoint_vs_fp64_adjoint(built, case):
    """The FP32 adjoint kernel against the FP64 reference gradient
    (oracle.adjoint64: the oracle's map in float64, differentiated by
    autograd) for the same dL/dS, every element of every family, norm-wise
    per family."""
    pytest.importorskip("torch")
    from oracle import adjoint64

    sc = {"gre": lambda: phantoms.config1_gre(seed=41, n=6, n_tr=2),
          "me3": lambda: phantoms.small_multipool("me", seed=42, n=4, pools=3, spins=2, coils=3, n_tr=2),
          "gm_bound": lambda: phantoms.small_multipool("gm", seed=43, n=4, pools=3, spins=1, coils=2, n_tr=2,
                                                       seq="sat"),
          "bssfp": lambda: phantoms.config4_adjoint(seed=44, nx=4, ny=4, nz=2, n_tr=2),
          # MT and CEST: pool 1 bound (saturated through its lineshape), the
          # models' K channels, no transverse outflow to the bound pool, pool
          # 0 received
          "mt": lambda: phantoms.small_multipool("mt", seed=45, n=4, pools=2, spins=2, coils=2, n_tr=2, seq="sat"),
          "cest3": lambda: phantoms.small_multipool("cest", seed=46, n=4, pools=3, spins=1, coils=2, n_tr=2,
                                                    seq="sat"),
          # several transmit coils: B = sum of TxCoil_c A_c, the rf gradient per coil
          "tx2": lambda: phantoms.multi_tx_gre(seed=47, n=6, n_tr=2, tx_coils=2, rx_coils=2),
          "tx3": lambda: phantoms.multi_tx_gre(seed=48, n=6, n_tr=2, tx_coils=3, rx_coils=3),
          # 4 spins, 12 coils: the four lanes of a voxel split its receive term
          "mt_epi_s4": lambda: phantoms.config5_mt_epi(seed=49, nx=4, ny=4, nz=1, spins=4, n_coils=12, n_read=8,
                                                       n_pe=8),
          # the split in the free three-pool and one-pool instantiations
          "me3_s2_rx8": lambda: phantoms.small_multipool("me", seed=50, n=4, pools=3, spins=2, coils=8, n_tr=2),
          "me1_s4_rx8": lambda: phantoms.small_multipool("me", seed=51, n=4, pools=1, spins=4, coils=8, n_tr=2)}[case]()
    sc = _phase_modulated(sc, 12)
    tx, ty = _target(sc)
    _, gx, gy = _loss(sc, (tx, ty))
    g = engine.adjoint(sc, gx, gy)
    ref = adjoint64.gradients(sc, gx, gy)
    o = sc.VObj
    P, S = int(o["TypeNum"]), int(o["SpinNum"])
    act = ((o["Rho"] != 0) & (o["T1"] != 0) & (o["T2"] != 0)).ravel(order="F")
    vact = act.reshape(-1, P, order="F").any(axis=1)
    fams = [("T1", act), ("T2", act), ("Rho", act), ("dB0", vact),
            ("Mz0", np.tile(vact, P * S)), ("Mx0", np.tile(vact, P * S))]
    if "K" in ref:
        fams.append(("K", np.ones(ref["K"].size, bool)))
    for key, sel in fams:
        a, b = np.asarray(g[key], np.float64)[sel], ref[key][sel]
        err = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        print(f"{case} {key}: |grad| {np.linalg.norm(b):.4e}, relative error {err:.2e} over {b.size} elements")
        assert err <= TOL
    err = float(np.linalg.norm(g["rf"] - ref["rf"]) / np.linalg.norm(ref["rf"]))
    print(f"{case} rf: relative error {err:.2e} over {ref['rf'].shape[0]} steps")
    assert err <= TOL


@pytest.mark.parametrize("tx", [2, 3])
def test_adjoint_multi_tx(built, tx):
    """Several transmit coils (BlochKernel.h:57-122: the rf field is the sum
    of TxCoil_c A_c): the tissue gradients and, per coil, the rf gradient
    against central differences of the FP64 oracle's loss -- scaling one
    coil's amplitudes, shifting one coil's phases, and single entries of
    that coil's VSeq.rfAmpLine / rfPhaseLine."""
    sc = _phase_modulated(phantoms.multi_tx_gre(seed=50 + tx, n=6, n_tr=2, tx_coils=tx, rx_coils=2), 7)
    target = _target(sc)
    _, gsx, gsy = _loss(sc, target)
    g = engine.adjoint(sc, gsx, gsy)
    o = sc.VObj
    act = ((o["Rho"] != 0) & (o["T1"] != 0) & (o["T2"] != 0)).ravel(order="F")
    idx = np.flatnonzero(act)
    for key in ("T1", "T2"):
        p = np.asarray(o[key], np.float64).ravel(order="F")
        _check(key, g[key][idx], _fd_gradient(sc, target, "VObj", key, idx, H * np.abs(p[idx])))
    _check("dB0", g["dB0"][idx], _fd_gradient(sc, target, "VMag", "dB0", idx, np.full(idx.size, DB0_STEP)))
    a, grf = g["rf_a"], g["rf"]
    assert grf.shape[1:] == (tx, 2)
    coil = np.asarray(sc.VSeq["rfCoilLine"]).ravel()
    amp = np.asarray(sc.VSeq["rfAmpLine"], np.float64).ravel()
    ph = np.asarray(sc.VSeq["rfPhaseLine"], np.float64).ravel()
    rng = np.random.default_rng(13)
    for c in range(tx):
        mine = coil == c + 1
        lp, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", np.where(mine, amp * (1 + H), amp)), target)
        lm, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", np.where(mine, amp * (1 - H), amp)), target)
        fd = (lp - lm) / (2 * H)
        adj = float(np.sum(grf[:, c, 0] * a[:, c, 0] + grf[:, c, 1] * a[:, c, 1]))
        print(f"coil {c} rf amplitude: adjoint {adj:.6e}, finite difference {fd:.6e}")
        assert abs(adj - fd) <= TOL * abs(fd)
        lp, _, _ = _loss(_with(sc, "VSeq", "rfPhaseLine", np.where(mine, ph + H, ph)), target)
        lm, _, _ = _loss(_with(sc, "VSeq", "rfPhaseLine", np.where(mine, ph - H, ph)), target)
        fd = (lp - lm) / (2 * H)
        adj = float(np.sum(-grf[:, c, 0] * a[:, c, 1] + grf[:, c, 1] * a[:, c, 0]))
        print(f"coil {c} rf phase: adjoint {adj:.6e}, finite difference {fd:.6e}")
        assert abs(adj - fd) <= TOL * abs(fd)
        # single entries of this coil's lines
        cand = _untied(amp, 4 * H * np.abs(amp))
        cand = cand[mine[cand] & (np.abs(amp[cand]) > 1e-3 * np.abs(amp).max())]
        pick = np.sort(rng.choice(cand, min(8, cand.size), replace=False))
        _check(f"coil {c} rfAmpLine", g["rf_amp_line"][pick],
               _fd_gradient(sc, target, "VSeq", "rfAmpLine", pick, H * np.abs(amp[pick])))


def test_adjoint_rejects_four_cest_pools(built):
    sc = phantoms.small_multipool("cest", seed=33, n=4, pools=4, spins=1, coils=1, n_tr=1, seq="sat")
    with pytest.raises(engine.ScanError) as e:
        engine.adjoint(sc, np.zeros(1), np.zeros(1))
    assert e.value.status == -6


def test_autograd_bridge(built):
    """The torch.autograd bridge: loss.backward() gives mrl_adjoint's
    gradients, in the parameters' shapes, and they match FP64 differences."""
    torch = pytest.importorskip("torch")
    from mrilab_gb300 import autograd

    sc = _phase_modulated(phantoms.small_multipool("me", seed=35, n=6, pools=2, spins=2, coils=2, n_tr=2), 6)
    tx, ty = _target(sc)
    params = autograd.parameters(sc, names=("T1", "T2", "Rho", "dB0", "K", "rfAmp"))
    sx, sy = autograd.scan(sc, **params)
    loss = ((sx - torch.from_numpy(tx)) ** 2 + (sy - torch.from_numpy(ty)) ** 2).sum()
    loss.backward()
    out = engine.scan(sc)
    g = engine.adjoint(sc, 2 * (out["Sx"] - tx), 2 * (out["Sy"] - ty))
    for name, key in (("T1", "T1"), ("T2", "T2"), ("Rho", "Rho"), ("dB0", "dB0"), ("K", "K"),
                      ("rfAmp", "rf_amp_line")):
        t = params[name]
        assert t.grad is not None and t.grad.shape == t.shape
        flat = t.grad.numpy().ravel(order="F")
        np.testing.assert_allclose(flat, g[key][: flat.size], rtol=1e-6, atol=1e-12 * np.abs(g[key]).max())
    # one direction of T2 against differences of the FP64 oracle
    t2 = np.asarray(sc.VObj["T2"], np.float64)
    d = np.random.default_rng(3).uniform(-1, 1, t2.shape) * t2
    lp, _, _ = _loss(_with(sc, "VObj", "T2", (t2 + H * d).ravel(order="F")), (tx, ty))
    lm, _, _ = _loss(_with(sc, "VObj", "T2", (t2 - H * d).ravel(order="F")), (tx, ty))
    plus = (t2 + H * d).astype(np.float32).astype(np.float64)
    minus = (t2 - H * d).astype(np.float32).astype(np.float64)
    fd = (lp - lm) / (2 * H)
    adj = float(np.sum(params["T2"].grad.numpy() * (plus - minus) / (2 * H)))
    print(f"autograd T2 direction: {adj:.6e}, finite difference {fd:.6e}")
    assert abs(adj - fd) <= TOL * abs(fd)


def test_adjoint_plan_iterations(built):
    """An adjoint plan run twice gives the one-shot call's gradients, and its
    forward pass the signal of mrl_scan."""
    sc = _phase_modulated(phantoms.small_multipool("me", seed=36, n=6, pools=2, spins=2, coils=2, n_tr=2), 7)
    tx, ty = _target(sc)
    ref = engine.scan(sc)
    gx, gy = 2 * (ref["Sx"] - tx), 2 * (ref["Sy"] - ty)
    one = engine.adjoint(sc, gx, gy)
    plan = engine.AdjointPlan(sc)
    try:
        for _ in range(2):
            plan.forward()
            out = plan.signal()
            np.testing.assert_array_equal(out["Sx"], ref["Sx"])
            np.testing.assert_array_equal(out["Sy"], ref["Sy"])
            plan.backward(gx, gy)
            g = plan.gradients()
            for k in ("T1", "T2", "Rho", "dB0", "K", "Mz0", "rf", "rf_amp_line", "rf_phase_line"):
                np.testing.assert_array_equal(g[k], one[k])
        w = plan.work()
        assert w["n_rf"] == len(one["rf"]) and w["steps"] > 0
    finally:
        plan.close()


def test_adjoint_long_train(built):
    """200 TRs of balanced SSFP (123,800 steps) on a small phantom: the
    gradients keep their accuracy over a long train (the checkpoints come
    from the anchored forward integrator; the backward sweep runs the whole
    train in single precision)."""
    sc = _phase_modulated(phantoms.config4_adjoint(seed=3, nx=4, ny=4, nz=2, n_tr=200), 8)
    target = _target(sc)
    _, gsx, gsy = _loss(sc, target)
    g = engine.adjoint(sc, gsx, gsy)
    o = sc.VObj
    rng = np.random.default_rng(12)
    act = ((o["Rho"] != 0) & (o["T1"] != 0) & (o["T2"] != 0)).ravel(order="F")
    # 8 elements per family: one oracle run of the train takes about a second
    idx = np.sort(rng.choice(np.flatnonzero(act), 8, replace=False))
    for key in ("T1", "T2"):
        p = np.asarray(o[key], np.float64).ravel(order="F")
        _check(key + " (200 TRs)", g[key][idx], _fd_gradient(sc, target, "VObj", key, idx, H * np.abs(p[idx])))
    vidx = np.sort(rng.choice(np.flatnonzero(act.reshape(-1, 2, order="F").any(axis=1)), 8, replace=False))
    _check("dB0 (200 TRs)", g["dB0"][vidx],
           _fd_gradient(sc, target, "VMag", "dB0", vidx, np.full(vidx.size, DB0_STEP)))
    a, grf = g["rf_a"], g["rf"]
    amp = np.asarray(sc.VSeq["rfAmpLine"], np.float64).ravel()
    lp, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", amp * (1 + H)), target)
    lm, _, _ = _loss(_with(sc, "VSeq", "rfAmpLine", amp * (1 - H)), target)
    fd = (lp - lm) / (2 * H)
    adj = float(np.sum(grf[:, 0] * a[:, 0] + grf[:, 1] * a[:, 1]))
    print(f"rf amplitude (200 TRs): adjoint {adj:.6e}, finite difference {fd:.6e}")
    assert abs(adj - fd) <= TOL * abs(fd)


def test_adjoint_receiver_phase(built):
    """A nonzero receiver reference phase (VVar.rfRef) rotates the signal;
    the adjoint rotates dL/dS back."""
    sc = _phase_modulated(phantoms.config1_gre(seed=37, n=6, n_tr=2), 9)
    sc.VVar["rfRef"] = np.float64(0.7)
    target = _target(sc)
    _, gsx, gsy = _loss(sc, target)
    g = engine.adjoint(sc, gsx, gsy)
    o = sc.VObj
    act = ((o["Rho"] != 0) & (o["T1"] != 0) & (o["T2"] != 0)).ravel(order="F")
    idx = np.flatnonzero(act)
    p = np.asarray(o["T2"], np.float64).ravel(order="F")
    _check("T2 (rfRef 0.7)", g["T2"][idx], _fd_gradient(sc, target, "VObj", "T2", idx, H * np.abs(p[idx])))
    vidx = np.flatnonzero(act)
    _check("dB0 (rfRef 0.7)", g["dB0"][vidx],
           _fd_gradient(sc, target, "VMag", "dB0", vidx, np.full(vidx.size, DB0_STEP)))
