"""Native sequence compiler (mrl_seq_compile, include/mrl_seq.h): MRiLab's
per-TR PSD merge, TR concatenation with dummy TRs and the sequence checks,
host only.  Pinned to the oracle's restatement of the MATLAB rules
(oracle/seqmerge.py, integer-nanosecond arithmetic) on every sequence the
workloads use, bit for bit."""
import numpy as np
import pytest

from mrilab_gb300 import phantoms, seq, seqc
from oracle import seqmerge

GAMMA = seq.GAMMA_H


def _gre(n_tr=3, tx=1, ext_every=0):
    trs = []
    for i in range(n_tr):
        tr = seq.TR(20_000_000)
        t, a = seq.sinc_rf(0, 2_000_000, 10_000, 30.0, 4.0)
        tr.rf(t, a)
        for c in range(2, tx + 1):
            tr.rf(t, np.asarray(a) / c, 0.7 * (c - 1), 0.0, coil=c)
        tr.trap("z", 0, 2_000_000, 1e-3, ramp_ns=10_000)
        tr.trap("y", 2_100_000, 3_000_000, (i - n_tr // 2) * 1e-3, ramp_ns=100_000)
        tr.trap("x", 3_000_000, 6_000_000, 4e-3, ramp_ns=100_000)
        tr.adc_t += [0]
        tr.adc_v += [0.0]
        tr.adc(3_100_000 + 31_250 * np.arange(64))
        tr.adc_t += [20_000_000]
        tr.adc_v += [0.0]
        if ext_every and i % ext_every == 0:
            tr.ext(7_000_000, 1.0)
        trs.append(tr)
    return trs


def _same(a, b):
    assert set(a) == set(b)
    for k in a:
        np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]), err_msg=k)


@pytest.mark.parametrize("kw", [dict(), dict(tx=3), dict(ext_every=2), dict(n_tr=1)])
def test_compiler_matches_oracle(kw):
    trs = _gre(**kw)
    multi = kw.get("tx", 1) > 1
    _same(seq.concat(trs, multi_transmit=multi, tx_coil_num=3, master_tx_coil=1),
          seqmerge.concat(_gre(**kw), multi_transmit=multi))


@pytest.mark.parametrize("builder", ["config1", "config2", "multi_tx", "bssfp", "epi", "sat", "zspec"])
def test_workload_sequences_match_oracle(builder):
    """The sequence builders of every workload, through the compiler and
    through the oracle: the same lines."""
    import inspect

    calls = {
        "config1": lambda: phantoms.gre_lines(n_read=16, n_pe=16, fov=(0.24,) * 3, tr_ms=20.0, te_ms=(5.0,),
                                              flip=30.0, rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0,
                                              n_tr=4),
        "config2": lambda: phantoms.gre_lines(n_read=32, n_pe=4, n_par=2, fov=(0.24, 0.24, 0.06), tr_ms=25.0,
                                              te_ms=(2.0, 6.0, 10.0, 14.0, 18.0, 22.0), flip=20.0, rf_ms=0.5,
                                              rf_raster_us=10.0, tbw=2.0, bw_hz=64000.0, n_tr=3),
        "multi_tx": lambda: phantoms.gre_lines(n_read=8, n_pe=8, fov=(0.24,) * 3, tr_ms=20.0, te_ms=(5.0,),
                                               flip=30.0, rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0,
                                               n_tr=2, tx_coils=3),
        "bssfp": lambda: phantoms.bssfp_lines(n_read=16, n_pe=4, n_par=1, n_tr=3),
        "epi": lambda: phantoms.epi_lines(n_read=8, n_pe=8),
        "sat": lambda: phantoms.sat_gre_lines(n_read=8, n_pe=2),
        "zspec": lambda: phantoms.zspec_lines(offset_hz=400.0, sat_ms=5.0, b1_ut=1.0),
    }
    # run each builder twice: once as is (native compiler), once with seq.concat
    # replaced by the oracle's concatenation
    native = calls[builder]()[0]
    real = seq.concat
    try:
        seq.concat = lambda trs, multi_transmit=False, **k: seqmerge.concat(trs, multi_transmit=multi_transmit)
        ref = calls[builder]()[0]
    finally:
        seq.concat = real
    assert inspect.isfunction(real)
    _same(native, ref)


def test_dummy_trs_zero_gradients_and_adc():
    """DP_Flag 'on' with DP_Num 2: the first two TRs keep their rf and lose
    their gradients and ADC (DoPulseGen.m:71-87)."""
    out = seq.concat(_gre(n_tr=4), dummy_trs=2)
    _same(out, seqmerge.concat(_gre(n_tr=4), dummy_trs=2))
    per = seqmerge.concat(_gre(n_tr=1))
    n_gx, n_adc = per["GxAmpLine"].size, per["ADCLine"].size
    assert np.all(out["GxAmpLine"][:2 * n_gx] == 0) and np.any(out["GxAmpLine"][2 * n_gx:] != 0)
    assert np.all(out["ADCLine"][:2 * n_adc] == 0) and np.count_nonzero(out["ADCLine"]) == 2 * 64
    np.testing.assert_array_equal(out["rfAmpLine"][:per["rfAmpLine"].size], per["rfAmpLine"])


def test_checks_reject_what_the_reference_rejects():
    trs = _gre(n_tr=2)
    # gradient amplitude (4 mT/m readout against 3 mT/m, beyond the 0.5 % tolerance)
    with pytest.raises(seqc.SeqError, match="GxR exceeds maximum allowed gradient amplitude"):
        seq.concat(trs, max_grad=3e-3)
    seq.concat(_gre(n_tr=2), max_grad=3.99e-3)  # within 0.5 %
    # slew rate: the 0.1 ms ramps to 4 mT/m are 40 T/m/s
    with pytest.raises(seqc.SeqError, match="slew rate"):
        seq.concat(_gre(n_tr=2), max_slew=30.0)
    seq.concat(_gre(n_tr=2), max_slew=200.0, max_grad=0.05)
    # update rate: rf sampled every 10 us against a 20 us minimum
    with pytest.raises(seqc.SeqError, match="rf1 sequence line exceeds minimum update rate"):
        seq.concat(_gre(n_tr=2), min_upd_rate=20e-6)
    seq.concat(_gre(n_tr=2), min_upd_rate=1e-6)
    # multi-transmit: coil 3 on a 2-coil system, and the master coil unused
    with pytest.raises(seqc.SeqError, match="more coil elements"):
        seq.concat(_gre(n_tr=1, tx=3), multi_transmit=True, tx_coil_num=2)
    with pytest.raises(seqc.SeqError, match="Master Tx coil"):
        seq.concat(_gre(n_tr=1, tx=3), multi_transmit=True, tx_coil_num=3, master_tx_coil=4)


def test_empty_channel_is_an_error():
    ch = _gre(n_tr=1)[0].channels()
    ch["gy"] = (np.zeros(0), np.zeros(0))
    with pytest.raises(seqc.SeqError, match="GyPE sequence line can not be empty"):
        seqc.compile_lines([ch])


def test_samples_outside_the_span_are_dropped():
    tr = _gre(n_tr=1)[0]
    ch = tr.channels()
    t, v = ch["gx"]
    ch["gx"] = (np.append(t, 0.5), np.append(v, 9.0))  # beyond the 20 ms TR
    out = seqc.compile_lines([ch])
    ref = seqc.compile_lines([tr.channels()])
    _same(out, ref)
