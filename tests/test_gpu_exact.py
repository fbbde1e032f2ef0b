"""MRL_NUMERICS_EXACT (exact relaxation-exchange propagator) through the C
ABI against the oracle's exact scheme in FP64."""
import numpy as np
import pytest

import oracle
from conftest import rel_l2, signal
from mrilab_gb300 import engine, phantoms

pytestmark = pytest.mark.gpu


def _gm_free(sc):
    sc.VObj["TypeFlag"] = np.zeros(int(sc.VObj["TypeNum"]))
    return sc


CASES = {
    "me2": lambda: phantoms.small_multipool("me", seed=51, n=8, pools=2, spins=2, coils=2, n_tr=3),
    "me3": lambda: phantoms.small_multipool("me", seed=52, n=6, pools=3, spins=1, coils=3, n_tr=2),
    "gm3_free": lambda: _gm_free(phantoms.small_multipool("gm", seed=53, n=6, pools=3, spins=2, coils=2, n_tr=2)),
    # a bound pool (TypeFlag 1, last) under off-resonance saturation pulses
    "gm2_bound": lambda: phantoms.small_multipool("gm", seed=57, n=6, pools=2, spins=2, coils=2, n_tr=2, seq="sat"),
    "gm3_bound": lambda: phantoms.small_multipool("gm", seed=58, n=6, pools=3, spins=2, coils=2, n_tr=2, seq="sat"),
    # the MT + exchange EPI's tissue and sequence (8 ms MT pulse), small
    "mt_epi": lambda: phantoms.config5_mt_epi(seed=6, nx=6, ny=6, nz=2, spins=2, n_coils=4, n_read=8, n_pe=8),
    # the MT and CEST models (pool 1 bound, the models' K layouts and
    # transverse maps) under saturation pulses, up to five pools
    "mt": lambda: phantoms.small_multipool("mt", seed=59, n=6, pools=2, spins=2, coils=2, n_tr=2, seq="sat"),
    "cest3": lambda: phantoms.small_multipool("cest", seed=60, n=6, pools=3, spins=2, coils=2, n_tr=2, seq="sat"),
    "cest4": lambda: phantoms.small_multipool("cest", seed=61, n=5, pools=4, spins=1, coils=2, n_tr=2, seq="sat"),
    "cest5": lambda: phantoms.small_multipool("cest", seed=62, n=5, pools=5, spins=1, coils=2, n_tr=1, seq="sat"),
}
# the MT EPI's FP32 bounds (signal, final Mz): as for its accurate mode
# against the FP64 oracle, the 8 ms MT pulse's single-precision state
# (measured 1.4e-5 and 2.0e-5)
TOL = {"mt_epi": (2e-5, 3e-5)}


@pytest.mark.parametrize("case", sorted(CASES))
def test_exact_matches_fp64_exact_oracle(built, case):
    sc = CASES[case]()
    ref = oracle.run_port(sc, "f64", exact=True)
    out = engine.scan(sc, numerics="exact")
    err = rel_l2(signal(out), signal(ref))
    err_mz = rel_l2(out["Mz"], ref["Mz"])
    split = rel_l2(signal(oracle.run_port(sc, "f64")), signal(ref))
    print(f"{case}: exact GPU vs exact FP64 {err:.2e} (Mz {err_mz:.2e}); split scheme vs exact {split:.2e}")
    tol, tol_mz = TOL.get(case, (1e-5, 1e-5))
    assert err <= tol and err_mz <= tol_mz


def test_exact_with_stiff_exchange(built):
    """Exchange 100x faster than the phantom's (k dt up to ~10 in the long
    steps): the exact mode still follows the exact solution, while the
    reference's split exchange departs from it."""
    sc = phantoms.small_multipool("me", seed=54, n=6, pools=2, spins=1, coils=1, n_tr=2)
    sc.VObj["K"] = np.asfortranarray(sc.VObj["K"] * np.float32(100))
    ref = oracle.run_port(sc, "f64", exact=True)
    out = engine.scan(sc, numerics="exact")
    err = rel_l2(signal(out), signal(ref))
    split = rel_l2(signal(engine.scan(sc)), signal(ref))
    print(f"stiff exchange: exact GPU vs exact FP64 {err:.2e}, split scheme (accurate mode) vs exact {split:.2e}")
    assert err <= 1e-5
    assert split > 1e-2


def test_exact_plan_repeats_scan(built):
    sc = CASES["me2"]()
    one = engine.scan(sc, numerics="exact")
    plan = engine.Plan(sc, numerics="exact")
    try:
        for _ in range(2):
            plan.execute()
            out = plan.download()
            np.testing.assert_array_equal(out["Sx"], one["Sx"])
            np.testing.assert_array_equal(out["Mz"], one["Mz"])
    finally:
        plan.close()


def test_exact_cest_with_config3_exchange(built):
    """Config 3's fastest exchange (k up to 5000 1/s: k dt reaches 0.05 per
    10 us step and far more over the sequence's long gaps) with five pools:
    the exact mode follows the exact solution; the reference's split scheme
    departs from it."""
    sc = phantoms.small_multipool("cest", seed=63, n=5, pools=5, spins=1, coils=1, n_tr=1, seq="sat")
    k = np.asarray(sc.VObj["K"], np.float32)
    sc.VObj["K"] = np.asfortranarray(np.where(k > 0, np.float32(5000.0), k).astype(np.float32))
    ref = oracle.run_port(sc, "f64", exact=True)
    out = engine.scan(sc, numerics="exact")
    err = rel_l2(signal(out), signal(ref))
    split = rel_l2(signal(oracle.run_port(sc, "f64")), signal(ref))
    print(f"CEST k = 5000: exact GPU vs exact FP64 {err:.2e}, split scheme vs exact {split:.2e}")
    assert err <= 1e-5 and split > 1.0


def test_exact_normal_model_is_the_accurate_mode(built):
    """A single pool's relaxation is already exact: the exact mode runs the
    accurate integrator."""
    sc = phantoms.config1_gre(seed=56, n=8, n_tr=2)
    np.testing.assert_array_equal(engine.scan(sc, numerics="exact")["Sx"], engine.scan(sc)["Sx"])
