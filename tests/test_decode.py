"""The engine's sequence decoder (mrl_decode, host only) against the
oracle's decoder (DoScanAtCPU.cpp:246-420 as the C oracle restates it) on
the same VSeq lines: every dt > 0 step, bit for bit -- dt, gradients, ADC
sample index, rf frequency -- and the complex rf amplitude (the oracle folds
a negative amplitude into the phase) to rounding."""
import numpy as np
import pytest

import oracle
from mrilab_gb300 import engine, phantoms


def _compare(sc):
    d = engine.decode(sc)
    o = oracle.run_port(sc, "f64", step_records=max(1, d.shape[0]) + 16)
    r = o["records"]
    tx = int(sc.VCoi["TxCoilNum"])
    assert d.shape[0] == r.shape[0] == o["steps"]
    np.testing.assert_array_equal(d[:, 0], r[:, 0])            # dt
    np.testing.assert_array_equal(d[:, 1:4], r[:, 1:4])        # Gz, Gy, Gx
    np.testing.assert_array_equal(d[:, 4], np.where(r[:, 8] != 0, r[:, 9], -1))  # ADC sample
    np.testing.assert_array_equal(d[:, 7], r[:, 6])            # rf frequency
    for c in range(tx):  # every Tx coil: complex amplitude and frequency
        a_eng = d[:, 5 + 3 * c] * np.exp(1j * d[:, 6 + 3 * c])
        j = 4 if c == 0 else 10 + 3 * (c - 1)
        a_ora = r[:, j] * np.exp(1j * r[:, j + 1])
        scale = max(1e-30, float(np.abs(a_ora).max()))
        assert np.abs(a_eng - a_ora).max() <= 1e-12 * scale
        np.testing.assert_array_equal(d[:, 7 + 3 * c], r[:, j + 2])
    return d


def _gre_with_ext():
    sc = phantoms.config1_gre(seed=4, n=8, n_tr=3)
    lines, _ = phantoms.gre_lines(n_read=8, n_pe=3, fov=(0.24,) * 3, tr_ms=20.0, te_ms=(5.0,), flip=30.0,
                                  rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0, ext_every=1)
    sc.VSeq = lines
    return sc


SEQUENCES = {
    "gre": lambda: phantoms.config1_gre(seed=1, n=16, n_tr=4),
    # one Ext event per TR: decoded through (no plugin) the step list is the
    # one without stops
    "gre_ext": _gre_with_ext,
    "sat_gre": lambda: phantoms.small_multipool("mt", seed=2, n=4, pools=2, n_tr=3, seq="sat"),
    "bssfp": lambda: phantoms.config4_adjoint(seed=3, nx=4, ny=4, nz=2, n_tr=6),
    "mt_epi": lambda: phantoms.config5_mt_epi(seed=4, nx=4, ny=4, nz=2, spins=1, n_coils=2, n_read=16, n_pe=8),
    "cest_train": lambda: phantoms.cest_instance(5, 64, 4, 3.5, 2.0, 2.0),
    "gre_tx2": lambda: phantoms.multi_tx_gre(seed=6, n=6, n_tr=2, tx_coils=2),
    "gre_tx3": lambda: phantoms.multi_tx_gre(seed=7, n=6, n_tr=2, tx_coils=3),
}


@pytest.mark.parametrize("name", sorted(SEQUENCES))
def test_decoder_matches_oracle(built, name):
    d = _compare(SEQUENCES[name]())
    assert d.shape[0] > 0 and (d[:, 4] >= 0).any()


def test_decoder_matches_oracle_random_gre(built):
    """Seeded random GRE sizes (TR count, matrix) and receiver settings."""
    hypothesis = pytest.importorskip("hypothesis")
    st = hypothesis.strategies

    @hypothesis.settings(max_examples=12, deadline=None)
    @hypothesis.given(seed=st.integers(0, 1000), n=st.sampled_from([2, 4, 6, 8]), n_tr=st.integers(1, 5))
    def run(seed, n, n_tr):
        _compare(phantoms.config1_gre(seed=seed, n=n, n_tr=n_tr))

    run()


def test_decoder_matches_oracle_random_epi(built):
    """Seeded random EPI readouts (odd and even lengths, line counts)."""
    hypothesis = pytest.importorskip("hypothesis")
    st = hypothesis.strategies

    @hypothesis.settings(max_examples=8, deadline=None)
    @hypothesis.given(seed=st.integers(0, 1000), n_read=st.integers(3, 24), n_pe=st.integers(1, 9))
    def run(seed, n_read, n_pe):
        _compare(phantoms.config5_mt_epi(seed=seed, nx=2, ny=2, nz=1, spins=1, n_coils=1, n_read=n_read,
                                         n_pe=n_pe))

    run()


def test_decode_reports_the_count_when_short(built):
    import ctypes

    sc = phantoms.config1_gre(seed=1, n=4, n_tr=1)
    lib = engine.library()
    hs = engine.HostScan(sc)
    n = ctypes.c_longlong(0)
    buf = (ctypes.c_double * 8)()
    lib.mrl_decode.argtypes = [ctypes.POINTER(engine.ScanArgs), ctypes.POINTER(ctypes.c_double), ctypes.c_longlong,
                               ctypes.POINTER(ctypes.c_longlong)]
    assert lib.mrl_decode(ctypes.byref(hs.args), buf, 1, ctypes.byref(n)) == -1
    assert n.value == engine.decode(sc).shape[0] > 1


def _pack(sc, ckpt_every=0):
    import ctypes

    lib = engine.library()
    fn = lib.mrl_selftest_pack
    fn.argtypes = [ctypes.POINTER(engine.ScanArgs), ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_longlong,
                   ctypes.POINTER(ctypes.c_longlong)]
    hs = engine.HostScan(sc)
    n = ctypes.c_longlong(0)
    fn(ctypes.byref(hs.args), ckpt_every, None, 0, ctypes.byref(n))
    out = np.zeros((n.value, 16), np.float32)
    assert fn(ctypes.byref(hs.args), ckpt_every, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), n.value,
              ctypes.byref(n)) == 0
    return out


@pytest.mark.parametrize("name", ["gre", "bssfp", "mt_epi"])
def test_step_records_carry_fp64_phase_moments(built, name):
    """The accurate integrator's step records: the frame's phase moments
    (elapsed free-precession time and gradient areas, summed over the steps
    without rf before each step) travel as float (hi, lo) pairs whose sum is
    the FP64 sum to ~2^-48 relative; the step flags mark ADC, rf, a change
    of the float dt or gradients, and every ckpt_every-th step."""
    sc = SEQUENCES[name]()
    d = engine.decode(sc)
    rec = _pack(sc, ckpt_every=16)
    assert rec.shape[0] == d.shape[0]
    rf = d[:, 5].astype(np.float32) != 0
    free = ~rf
    dt, gz, gy, gx = d[:, 0], d[:, 1], d[:, 2], d[:, 3]
    for col, w in ((8, np.ones_like(dt)), (10, gx), (12, gy), (14, gz)):
        before = np.concatenate([[0.0], np.cumsum(np.where(free, w * dt, 0.0))[:-1]])
        got = rec[:, col].astype(np.float64) + rec[:, col + 1].astype(np.float64)
        scale = max(1e-300, float(np.abs(before).max()))
        assert np.abs(got - before).max() <= 2.0 ** -46 * scale
    flags = rec[:, 7].view(np.int32)
    np.testing.assert_array_equal((flags & 1) != 0, d[:, 4] >= 0)       # ADC
    np.testing.assert_array_equal((flags & 2) != 0, rf)                 # rf
    f32 = d[:, :4].astype(np.float32)
    prev = np.vstack([np.full((1, 4), np.nan, np.float32), f32[:-1]])
    prev[0, 0] = -1.0
    prev[0, 1:] = 0.0
    new_dt = f32[:, 0] != prev[:, 0]
    np.testing.assert_array_equal((flags & 16) != 0, new_dt)            # dt changed
    np.testing.assert_array_equal((flags & 8) != 0, new_dt | (f32[:, 1:] != prev[:, 1:]).any(axis=1))
    np.testing.assert_array_equal((flags & 32) != 0, np.arange(len(d)) % 16 == 0)
