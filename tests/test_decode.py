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
    assert d.shape[0] == r.shape[0] == o["steps"]
    np.testing.assert_array_equal(d[:, 0], r[:, 0])            # dt
    np.testing.assert_array_equal(d[:, 1:4], r[:, 1:4])        # Gz, Gy, Gx
    np.testing.assert_array_equal(d[:, 4], np.where(r[:, 8] != 0, r[:, 9], -1))  # ADC sample
    np.testing.assert_array_equal(d[:, 7], r[:, 6])            # rf frequency
    a_eng = d[:, 5] * np.exp(1j * d[:, 6])
    a_ora = r[:, 4] * np.exp(1j * r[:, 5])
    scale = max(1e-30, float(np.abs(a_ora).max()))
    assert np.abs(a_eng - a_ora).max() <= 1e-12 * scale
    return d


SEQUENCES = {
    "gre": lambda: phantoms.config1_gre(seed=1, n=16, n_tr=4),
    "sat_gre": lambda: phantoms.small_multipool("mt", seed=2, n=4, pools=2, n_tr=3, seq="sat"),
    "bssfp": lambda: phantoms.config4_adjoint(seed=3, nx=4, ny=4, nz=2, n_tr=6),
    "mt_epi": lambda: phantoms.config5_mt_epi(seed=4, nx=4, ny=4, nz=2, spins=1, n_coils=2, n_read=16, n_pe=8),
    "cest_train": lambda: phantoms.cest_instance(5, 64, 4, 3.5, 2.0, 2.0),
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
