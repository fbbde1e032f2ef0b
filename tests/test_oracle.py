"""The CPU oracle, pinned against the reference engine (CPU only)."""
import numpy as np
import pytest

import oracle
from mrilab_gb300 import phantoms
from conftest import load_golden, rel_l2, signal

GOLDEN = ["gre2d_n16_tr4_seed1", "gre2d_n32_tr8_seed2", "gre2d_n64_full_seed0",
          # two and three transmit coils
          "gre_tx2_n8_seed1", "gre_tx3_n8_seed2"]


@pytest.mark.parametrize("name", GOLDEN)
def test_port_matches_reference_cpu_engine_golden(built, name):
    """The single-precision port reproduces the reference CPU engine's
    signal (golden vectors recorded from DoScanAtCPU on the stand-ins)."""
    sc, g = load_golden(name)
    out = oracle.run_port(sc, "f32", threads=2)
    ref = g["ref_Sx"] + 1j * g["ref_Sy"]
    assert rel_l2(signal(out), ref) <= 1e-6
    np.testing.assert_allclose(out["Kx"], g["ref_Kx"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(out["Ky"], g["ref_Ky"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(out["Mz"], g["ref_Mz"], rtol=0, atol=2e-6)


@pytest.mark.parametrize("name", GOLDEN)
def test_fp64_oracle_is_stable_against_golden(built, name):
    """The all-FP64 oracle reproduces its recorded output on this machine,
    and the reference's own FP32 error against it is at its known level."""
    sc, g = load_golden(name)
    out = oracle.run_port(sc, "f64", threads=2)
    f64 = g["f64_Sx"] + 1j * g["f64_Sy"]
    assert rel_l2(signal(out), f64) <= 1e-12
    ref = g["ref_Sx"] + 1j * g["ref_Sy"]
    assert rel_l2(ref, f64) < 1e-3


def test_port_threads_do_not_change_result(built):
    sc = phantoms.config1_gre(seed=5, n=16, n_tr=3)
    a = oracle.run_port(sc, "f32", threads=1)
    b = oracle.run_port(sc, "f32", threads=4)
    assert rel_l2(signal(a), signal(b)) < 1e-12
    np.testing.assert_array_equal(a["Mz"], b["Mz"])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not mounted")
@pytest.mark.parametrize("seed,n,n_tr", [(7, 8, 2), (8, 12, 3)])
def test_port_matches_live_reference_cpu_engine(built, seed, n, n_tr):
    sc = phantoms.config1_gre(seed=seed, n=n, n_tr=n_tr)
    ref = oracle.run_ref_cpu(sc)
    out = oracle.run_port(sc, "f32")
    assert rel_l2(signal(out), signal(ref)) <= 1e-6


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not mounted")
@pytest.mark.parametrize("case", ["two_voxels", "rf_ref", "empty_object"])
def test_port_edge_cases_match_live_reference_cpu_engine(built, case):
    """Edge cases against the reference CPU engine: a 2x2 phantom, a
    nonzero receiver phase (VVar.rfRef), and an empty object (Rho and the
    initial Mz zero: a zero signal, k-space still accumulated)."""
    if case == "two_voxels":
        sc = phantoms.config1_gre(seed=9, n=2, n_tr=2)
    else:
        sc = phantoms.config1_gre(seed=10, n=8, n_tr=2)
    if case == "rf_ref":
        sc.VVar["rfRef"] = np.float64(0.4)
    if case == "empty_object":
        for k in ("Rho", "Mz"):
            sc.VObj[k] = np.asfortranarray(sc.VObj[k] * 0)
    ref = oracle.run_ref_cpu(sc)
    out = oracle.run_port(sc, "f32")
    if case == "empty_object":
        assert not np.any(signal(ref)) and not np.any(signal(out))
    else:
        assert rel_l2(signal(out), signal(ref)) <= 1e-6
    np.testing.assert_array_equal(out["Kx"], ref["Kx"])
    np.testing.assert_allclose(out["Mz"], ref["Mz"], atol=1e-6)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not mounted")
@pytest.mark.parametrize("model,pools,seq", [("me", 2, "gre"), ("me", 3, "gre"), ("gm", 3, "sat"),
                                             ("mt", 2, "sat"), ("cest", 3, "sat"), ("cest", 4, "sat")])
@pytest.mark.parametrize("spins,coils", [(1, 1), (2, 2)])
def test_port_matches_reference_kernels(built, model, pools, seq, spins, coils):
    """Multi-pool models: the port agrees with the reference's own kernels
    (BlochKernel{ME,MT,CEST,GM}.cuh compiled as host C) at float-rounding
    level; a wrong exchange index or update order shows up as >1e-3."""
    sc = phantoms.small_multipool(model, seed=3, pools=pools, spins=spins, coils=coils, seq=seq)
    ref = oracle.run_ref_kernel(sc)
    out = oracle.run_port(sc, "f32")
    assert rel_l2(signal(out), signal(ref)) <= 2e-5
    np.testing.assert_allclose(out["Mz"], ref["Mz"], atol=1e-4)


MULTI_GOLDEN = ["mp_me_p2_s2_c2", "mp_me_p3_s1_c1", "mp_gm_p3_s2_c2", "mp_mt_p2_s2_c2", "mp_cest_p4_s2_c2",
                "mp_cest_p5_s1_c2", "mt_epi_gm_p3_s2_c4"]


@pytest.mark.parametrize("name", MULTI_GOLDEN)
def test_port_matches_reference_kernel_golden(built, name):
    """The single-precision port against the committed outputs of the
    reference's own multi-pool kernels (ME, GM, MT, CEST up to 5 pools, and
    the MT + exchange EPI: make_golden.py), without the reference tree: the
    signal at float-rounding distance, the final Mz within 1e-4."""
    sc, g = load_golden(name)
    out = oracle.run_port(sc, "f32")
    err = rel_l2(signal(out), g["ref_Sx"] + 1j * g["ref_Sy"])
    assert err <= 2e-5, err
    np.testing.assert_allclose(out["Mz"], g["ref_Mz"], atol=1e-4)
    # and the FP64 oracle is where it was when the fixture was made
    f64 = oracle.run_port(sc, "f64")
    assert rel_l2(signal(f64), g["f64_Sx"] + 1j * g["f64_Sy"]) <= 1e-12


def test_port_ext_callback_zeroes_transverse(built):
    """Ext events reach the callback with the state written back; an ideal
    spoiler plugin (DoExtPlugin case 6) zeroes Mxy."""
    sc = phantoms.config1_gre(seed=4, n=8, n_tr=3)
    lines, ntr = phantoms.gre_lines(n_read=8, n_pe=3, fov=(0.24,) * 3, tr_ms=20.0, te_ms=(5.0,), flip=30.0,
                                    rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0, ext_every=1)
    sc.VSeq = lines
    calls = []

    def cb(val, out):
        calls.append(val)
        out["Mx"][:] = 0
        out["My"][:] = 0
        return 0

    out = oracle.run_port(sc, "f64", ext_cb=cb)
    assert len(calls) == 3
    base = oracle.run_port(sc, "f64")
    assert rel_l2(signal(out), signal(base)) > 1e-3  # the spoiler changed later echoes


def test_port_history_matches_reference_cpu_engine_golden(built):
    """RunMode 1: the port's per-time-point state history and step times
    equal the reference CPU engine's (recorded from DoScanAtCPU)."""
    sc, g = load_golden("history_gre2d_n4_tr2_seed4")
    out = oracle.run_port(sc, "f32")
    for k in ("Mxs", "Mys", "Mzs"):
        np.testing.assert_allclose(out[k], g["ref_" + k], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(out["Muts"].ravel(), g["ref_Muts"].ravel())
    f64 = oracle.run_port(sc, "f64")
    for k in ("Mxs", "Mys", "Mzs"):
        np.testing.assert_allclose(f64[k], g["f64_" + k], rtol=0, atol=1e-12)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not mounted")
def test_port_history_matches_live_reference_cpu_engine(built):
    sc = phantoms.with_history(phantoms.config1_gre(seed=9, n=4, n_tr=3))
    ref = oracle.run_ref_cpu(sc)
    out = oracle.run_port(sc, "f32")
    for k in ("Mxs", "Mys", "Mzs"):
        np.testing.assert_allclose(out[k], ref[k], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(out["Muts"], ref["Muts"])


@pytest.mark.parametrize("model", ["me", "gm", "gm_bound", "mt", "cest"])
def test_exact_oracle_matches_bloch_mcconnell_expm(built, model):
    """The oracle's exact propagator (rotate every pool, then exp of the
    relaxation-exchange generator) equals the exponential of the whole
    Bloch-McConnell generator when every pool precesses at the same
    frequency (rotation about z then commutes with relaxation and exchange):
    one voxel, three pools with stiff exchange, free precession at dB0, the
    state read after the last of several uneven steps.  ``gm_bound``: pool 2
    is a bound pool (no transverse generator: its transverse state held, no
    transverse inflow from it; in the longitudinal one like the others).
    ``mt`` / ``cest``: pool 1 is the bound MT pool, rates only between pool 0
    and each other pool (the models' K layouts), and a free pool's
    transverse state does not flow out to the bound pool (the models'
    transverse map)."""
    bound = model == "gm_bound"
    mtc = model in ("mt", "cest")
    model = "gm" if bound else model
    scipy_linalg = pytest.importorskip("scipy.linalg")
    from mrilab_gb300 import seq as S

    P = 2 if model == "mt" else 3
    rho = np.array([[[[0.7, 0.2, 0.1][:P]]]], np.float32)
    t1 = np.array([[[[1.1, 0.45, 0.8][:P]]]], np.float32)
    t2 = np.array([[[[0.07, 0.015, 0.03][:P]]]], np.float32)
    rates = np.zeros((1, 1, 1, P, P), np.float32)
    rates[..., 1, 0] = 300.0
    rates[..., 0, 1] = rates[..., 1, 0] * rho[..., 1] / rho[..., 0]
    if P == 3:
        rates[..., 2, 0] = 120.0
        rates[..., 0, 2] = rates[..., 2, 0] * rho[..., 2] / rho[..., 0]
        if not mtc:
            rates[..., 1, 2] = 40.0
            rates[..., 2, 1] = rates[..., 1, 2] * rho[..., 1] / rho[..., 2]
    if mtc:
        t2[..., 1] = 12e-6
    tr = S.TR(30_000_000)
    times = [0, 1_500_000, 1_700_000, 6_000_000, 6_010_000, 18_000_000, 30_000_000]
    tr.adc(times[1:-1])
    lines = S.concat([tr])
    tf = (np.array([0.0, 0.0, 1.0]) if bound else np.zeros(P)) if model == "gm" else None
    if bound:
        t2[..., 2] = 12e-6
    sc = phantoms.assemble(rho, t1, t2, db0_hz=np.full((1, 1, 1), 37.0), model=model, rates=rates,
                           type_flag=tf, seqlines=lines)
    m0 = np.array([[0.3, -0.2, 0.4], [0.05, 0.1, 0.02], [-0.03, 0.04, 0.05]])[:P]  # [pool][x, y, z]
    if mtc:
        m0[1, :2] = 0.0  # the MT pool carries no transverse magnetisation
    for k, comp in (("Mx", 0), ("My", 1), ("Mz", 2)):
        sc.VObj[k] = np.asfortranarray(m0[:, comp].reshape(1, 1, 1, 1, P).astype(np.float32))
    out = oracle.run_port(sc, "f64", exact=True)
    # the generator on (x_0..x_P-1, y.., z.., 1)
    w = float(sc.VObj["Gyro"]) * float(sc.VMag["dB0"].ravel()[0])
    n = 3 * P + 1
    G = np.zeros((n, n))
    bnd = [(bound and t == 2) or (mtc and t == 1) for t in range(P)]
    for t in range(P):
        for c, r in ((0, 1 / t2[0, 0, 0, t]), (1, 1 / t2[0, 0, 0, t]), (2, 1 / t1[0, 0, 0, t])):
            if c < 2 and bnd[t]:
                continue  # a bound pool's transverse state is held
            kout = sum(rates[0, 0, 0, t, p] for p in range(P) if p != t and not (mtc and c < 2 and bnd[p]))
            G[c * P + t, c * P + t] = -r - kout
            for p in range(P):
                if p != t and not (c < 2 and bnd[p]):
                    G[c * P + t, c * P + p] = rates[0, 0, 0, p, t]
        if not bnd[t]:
            G[0 * P + t, 1 * P + t] += w   # dx/dt = w y
            G[1 * P + t, 0 * P + t] -= w   # dy/dt = -w x
        G[2 * P + t, n - 1] = rho[0, 0, 0, t] / t1[0, 0, 0, t]
    state = np.concatenate([m0[:, 0], m0[:, 1], m0[:, 2], [1.0]])
    # the integrated time: every dt > 0 step of the decoded sequence
    uts = sc.VSeq["utsLine"]
    total = float(np.sum(np.diff(uts)[np.diff(uts) > 0]))
    ref = scipy_linalg.expm(G * total) @ state
    got = np.concatenate([out["Mx"], out["My"], out["Mz"]])
    # the oracle's FP64 state is returned in the single-precision state arrays
    assert np.abs(got - ref[:-1]).max() <= 2e-7 * np.abs(ref[:-1]).max()


def _fp64_adjoint_case(name):
    return {
        "me2": lambda: phantoms.small_multipool("me", seed=32, n=5, pools=2, spins=2, coils=2, n_tr=2),
        "gm_bound": lambda: phantoms.small_multipool("gm", seed=38, n=4, pools=3, spins=1, coils=2, n_tr=2,
                                                     seq="sat"),
        "mt": lambda: phantoms.small_multipool("mt", seed=61, n=4, pools=2, spins=2, coils=2, n_tr=2, seq="sat"),
        "cest4": lambda: phantoms.small_multipool("cest", seed=62, n=4, pools=4, spins=1, coils=2, n_tr=2,
                                                  seq="sat"),
        # several transmit coils: the field is the sum of TxCoil_c A_c
        "tx2": lambda: phantoms.multi_tx_gre(seed=63, n=5, n_tr=2, tx_coils=2, rx_coils=2),
        "tx3": lambda: phantoms.multi_tx_gre(seed=64, n=5, n_tr=2, tx_coils=3, rx_coils=2),
    }[name]()


@pytest.mark.parametrize("name", ["me2", "gm_bound", "mt", "cest4", "tx2", "tx3"])
def test_fp64_adjoint_pinned(name):
    """The FP64 reference gradient (oracle.adjoint64: the oracle's map
    restated in float64 PyTorch, differentiated by autograd) is pinned to
    the C oracle: its signal is the FP64 port's, and its gradient of
    L = gx.Sx + gy.Sy matches central differences of the FP64 port (step
    1e-3 relative, dB0 1e-10 T) element by element."""
    pytest.importorskip("torch")
    from oracle import adjoint64

    sc = _fp64_adjoint_case(name)
    P, RX, A = int(sc.VObj["TypeNum"]), int(sc.VCoi["RxCoilNum"]), int(sc.VSig["SignalNum"])
    gx = np.random.default_rng(0).normal(size=P * RX * A)
    gy = np.random.default_rng(1).normal(size=P * RX * A)
    g = adjoint64.gradients(sc, gx, gy)
    ref = oracle.run_port(sc, "f64")
    assert rel_l2(g["Sx"] + 1j * g["Sy"], ref["Sx"] + 1j * ref["Sy"]) <= 1e-12

    def loss(s):
        o = oracle.run_port(s, "f64")
        return float(np.dot(gx, o["Sx"]) + np.dot(gy, o["Sy"]))

    for struct, key in (("VObj", "T1"), ("VObj", "T2"), ("VObj", "Rho"), ("VMag", "dB0"), ("VObj", "K")):
        if key not in getattr(sc, struct):
            continue
        arr = getattr(sc, struct)[key]
        base = np.asarray(arr, np.float64).ravel(order="F")
        nz = np.flatnonzero(base)
        for i in nz[:: max(1, nz.size // 3)][:3]:
            h = 1e-10 if key == "dB0" else 1e-3 * abs(base[i])
            out = []
            for sgn in (1, -1):
                b = base.copy()
                b[i] = np.float32(base[i] + sgn * h)
                s = sc.copy()
                d = getattr(s, struct)
                d[key] = np.asfortranarray(b.astype(arr.dtype).reshape(arr.shape, order="F"))
                out.append((loss(s), b[i]))
            fd = (out[0][0] - out[1][0]) / (out[0][1] - out[1][1])
            # (the differences' own truncation reaches 1e-5 for a bound pool's T2)
            assert abs(g[key][i] - fd) <= 5e-5 * abs(fd) + 1e-12, (key, i, g[key][i], fd)
    tx = int(sc.VCoi["TxCoilNum"])
    if tx > 1:
        # per coil: scale that coil's rf amplitudes by (1 + h), dA_c/dh = A_c at
        # the steps it is on (the rf steps' A from the port's step records)
        rec = oracle.run_port(sc, "f64", step_records=oracle.run_port(sc, "f64")["steps"])["records"]
        rec = rec[rec[:, 7] != 0]
        coil = np.asarray(sc.VSeq["rfCoilLine"]).ravel()
        amp = np.asarray(sc.VSeq["rfAmpLine"], np.float64).ravel()
        assert g["rf"].shape == (rec.shape[0], tx, 2)
        for c in range(tx):
            ca, cp = (4, 5) if c == 0 else (10 + 3 * (c - 1), 11 + 3 * (c - 1))
            a_re, a_im = rec[:, ca] * np.cos(rec[:, cp]), rec[:, ca] * np.sin(rec[:, cp])
            adj = float(np.sum(g["rf"][:, c, 0] * a_re + g["rf"][:, c, 1] * a_im))
            out = []
            for sgn in (1, -1):
                s2 = sc.copy()
                s2.VSeq["rfAmpLine"] = np.where(coil == c + 1, amp * (1 + sgn * 1e-4), amp)
                out.append(loss(s2))
            fd = (out[0] - out[1]) / 2e-4
            assert abs(adj - fd) <= 1e-5 * abs(fd), (c, adj, fd)
