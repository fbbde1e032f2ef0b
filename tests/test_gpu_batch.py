"""Batched scans (mrl_batch_*, mrl_scan_batched): many independent scans of
different tissue models, sizes and sequences run together.  Each instance's
result must equal the same scan run alone through mrl_scan."""
import numpy as np
import pytest

from conftest import rel_l2, signal
from mrilab_gb300 import engine, phantoms

pytestmark = pytest.mark.gpu


def _instances():
    return [
        phantoms.config1_gre(seed=21, n=24, n_tr=3),
        phantoms.small_multipool("me", seed=22, n=10, pools=2, spins=4, coils=3, n_tr=2),
        phantoms.small_multipool("cest", seed=23, n=6, pools=4, spins=1, coils=1, n_tr=2, seq="sat"),
        phantoms.config1_gre(seed=24, n=8, n_tr=2),
        phantoms.small_multipool("mt", seed=25, n=12, pools=2, spins=2, coils=2, n_tr=2, seq="sat"),
        phantoms.small_multipool("gm", seed=26, n=7, pools=3, spins=2, coils=2, n_tr=2, seq="sat"),
        phantoms.small_multipool("cest", seed=27, n=9, pools=3, spins=1, coils=2, n_tr=1, seq="sat"),
        # five pools: water, MT and three CEST pools (config 3's largest instances)
        phantoms.small_multipool("cest", seed=28, n=5, pools=5, spins=1, coils=2, n_tr=1, seq="sat"),
    ]


def _same(a, b):
    for k in ("Sx", "Sy", "Mx", "My", "Mz", "Kx", "Ky", "Kz"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_batch_equals_individual_scans(built):
    scans = _instances()
    alone = [engine.scan(sc, numerics="accurate") for sc in scans]
    b = engine.Batch(scans)
    try:
        w = b.work()
        assert w["units"] > 0 and w["launches"] >= 2
        b.execute("persistent")
        first = [dict((k, np.copy(v)) for k, v in o.items() if isinstance(v, np.ndarray)) for o in b.download()]
        for o, a in zip(first, alone):  # same kernel, same tiles, same reduction order: identical
            _same(o, a)
        b.execute("persistent")  # the captured graph, replayed
        for o, a in zip(b.download(), alone):
            _same(o, a)
        b.execute("plain")
        for o, a in zip(b.download(), alone):
            _same(o, a)
    finally:
        b.close()


def test_batch_tuned_matches_within_rounding(built):
    scans = _instances()
    alone = [engine.scan(sc, numerics="accurate") for sc in scans]
    b = engine.Batch(scans)
    try:
        b.tune()
        b.execute("persistent")
        for o, a in zip(b.download(), alone):
            # another spins-per-thread choice sums the spins in another order
            # (and pairs of spins take the packed f32x2 path, which adds the
            # increments in another order)
            assert rel_l2(signal(o), signal(a)) <= 3e-6
            np.testing.assert_allclose(o["Mz"], a["Mz"], rtol=0, atol=1e-6)
    finally:
        b.close()


def test_scan_batched_one_shot(built):
    scans = _instances()[:3]
    outs = engine.scan_batched(scans)
    for o, sc in zip(outs, scans):
        _same(o, engine.scan(sc, numerics="accurate"))
