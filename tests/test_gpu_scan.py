"""GPU parity of the scan engine, called through the C ABI (libmrl_scan.so)
and through the mex wrappers, against the reference's recorded outputs and
the CPU oracle."""
import os

import numpy as np
import pytest

import oracle
from conftest import ROOT, load_golden, rel_l2, signal
from mrilab_gb300 import engine, mexsim, phantoms

pytestmark = pytest.mark.gpu

SINGLE = ["gre2d_n16_tr4_seed1", "gre2d_n32_tr8_seed2", "gre2d_n64_full_seed0"]
MULTI = ["mp_me_p2_s2_c2", "mp_me_p3_s1_c1", "mp_gm_p3_s2_c2", "mp_mt_p2_s2_c2", "mp_cest_p4_s2_c2",
         "mp_cest_p5_s1_c2"]
# several transmit coils: B1 is the complex sum over the coils
# (BlochKernel.h:57-122), golden vectors from the reference CPU engine
MULTI_TX = ["gre_tx2_n8_seed1", "gre_tx3_n8_seed2"]

# Reference-order numerics: relative L2 of the complex signal against the
# reference CPU engine's own output (its float rounding reproduced op by op;
# transcendentals differ by < 1 ulp between libm and the device).
TOL_REF_CPU = 1e-5
# Multi-pool models against the reference's kernels run on the CPU in
# double-per-operation arithmetic: both sit at float-rounding distance
# (~1e-5) from the FP64 oracle.
TOL_REF_KERN = 3e-5
# Against the single-precision oracle port on the same inputs.
TOL_PORT = 1e-5


@pytest.mark.parametrize("name", SINGLE)
def test_reference_numerics_match_reference_cpu_engine(built, name):
    sc, g = load_golden(name)
    out = engine.scan(sc, numerics="reference")
    ref = g["ref_Sx"] + 1j * g["ref_Sy"]
    err = rel_l2(signal(out), ref)
    print(f"{name}: GPU vs reference CPU engine {err:.3e}")
    assert err <= TOL_REF_CPU
    np.testing.assert_allclose(out["Kx"], g["ref_Kx"], atol=1e-9)
    np.testing.assert_allclose(out["Ky"], g["ref_Ky"], atol=1e-9)
    # the final magnetisation of individual isochromats carries their own
    # rounding history (18k steps for the full scan) without the averaging
    # of the receive sum, hence a looser bound than the signal's
    assert rel_l2(out["Mz"], g["ref_Mz"]) <= 5e-5


@pytest.mark.parametrize("name", MULTI_TX)
def test_reference_numerics_multi_tx(built, name):
    """Two and three transmit coils in the reference's operation order
    against the reference CPU engine's own multi-Tx output."""
    sc, g = load_golden(name)
    assert int(sc.VCoi["TxCoilNum"]) >= 2
    out = engine.scan(sc, numerics="reference")
    err = rel_l2(signal(out), g["ref_Sx"] + 1j * g["ref_Sy"])
    print(f"{name}: GPU vs reference CPU engine {err:.3e}")
    assert err <= TOL_REF_CPU
    np.testing.assert_allclose(out["Kx"], g["ref_Kx"], atol=1e-9)
    assert rel_l2(out["Mz"], g["ref_Mz"]) <= 5e-5


@pytest.mark.parametrize("name", MULTI)
def test_reference_numerics_multipool_models(built, name):
    sc, g = load_golden(name)
    out = engine.scan(sc, numerics="reference")
    ref = g["ref_Sx"] + 1j * g["ref_Sy"]
    err_ref = rel_l2(signal(out), ref)
    port = oracle.run_port(sc, "f32")
    err_port = rel_l2(signal(out), signal(port))
    print(f"{name}: GPU vs reference kernels {err_ref:.3e}, vs port {err_port:.3e}")
    assert err_ref <= TOL_REF_KERN
    assert err_port <= TOL_PORT
    np.testing.assert_allclose(out["Mz"], port["Mz"], atol=1e-4)


def test_mex_wrapper_path(built):
    """DoScanAtGPU through the mex stand-in: globals in, globals out."""
    sc, g = load_golden("gre2d_n16_tr4_seed1")
    ms = mexsim.MexSession()
    for k, v in sc.structs().items():
        ms.set_global(k, v)
    ms.set_field("VCtl", "Numerics", np.float64(1.0))
    ms.call(os.path.join(ROOT, "mrilab_gb300", "mex", "DoScanAtGPU.so"))
    sx = ms.get("VSig", "Sx").ravel(order="F")
    sy = ms.get("VSig", "Sy").ravel(order="F")
    assert rel_l2(sx + 1j * sy, g["ref_Sx"] + 1j * g["ref_Sy"]) <= TOL_REF_CPU
    assert int(ms.get("VVar", "TRCount").ravel()[0]) == 4


@pytest.mark.parametrize("wrapper,name", [("DoMEScanAtGPU", "mp_me_p2_s2_c2"), ("DoMTScanAtGPU", "mp_mt_p2_s2_c2"),
                                          ("DoCESTScanAtGPU", "mp_cest_p4_s2_c2"), ("DoGMScanAtGPU", "mp_gm_p3_s2_c2")])
def test_multipool_mex_wrappers(built, wrapper, name):
    sc, g = load_golden(name)
    ms = mexsim.MexSession()
    for k, v in sc.structs().items():
        ms.set_global(k, v)
    ms.set_field("VCtl", "Numerics", np.float64(1.0))
    ms.call(os.path.join(ROOT, "mrilab_gb300", "mex", wrapper + ".so"))
    sx = ms.get("VSig", "Sx").ravel(order="F")
    sy = ms.get("VSig", "Sy").ravel(order="F")
    assert rel_l2(sx + 1j * sy, g["ref_Sx"] + 1j * g["ref_Sy"]) <= TOL_REF_KERN


def test_plan_matches_scan_and_reruns(built):
    sc, g = load_golden("gre2d_n32_tr8_seed2")
    direct = engine.scan(sc, numerics="reference")
    plan = engine.Plan(sc, numerics="reference")
    w = plan.work()
    assert w["samples"] == sc.signal_num and w["units"] > 0
    for _ in range(2):  # re-execution restarts from the initial state
        plan.execute()
        out = plan.download()
        assert rel_l2(signal(out), signal(direct)) <= 1e-12
    plan.close()


def test_inplace_scan_writes_the_callers_arrays(built):
    """scan(..., inplace=True) writes the final state and the signal into the
    caller's own arrays (as the mex entry points write the MATLAB globals)
    and gives the same outputs as the copying call."""
    sc, g = load_golden("mp_me_p2_s2_c2")
    ref = engine.scan(sc)
    assert not np.shares_memory(ref["Mx"], sc.VObj["Mx"])
    run = sc.copy()
    out = engine.scan(run, inplace=True)
    assert np.shares_memory(out["Sx"], run.VSig["Sx"]) and np.shares_memory(out["Mz"], run.VObj["Mz"])
    for k in ("Sx", "Sy", "Mx", "My", "Mz"):
        np.testing.assert_array_equal(out[k], ref[k])
    np.testing.assert_array_equal(np.asarray(run.VSig["Sx"]).reshape(-1, order="F"), ref["Sx"])
    np.testing.assert_array_equal(np.asarray(run.VObj["Mz"]).reshape(-1, order="F"), ref["Mz"])


def test_pinned_staging_matches_direct_copies(built, monkeypatch):
    """Objects and results above MRL_STAGE_MIN_MB (8 MB by default) travel
    through the calling thread's pinned buffer; staged and direct copies give
    the same outputs, also when that buffer grows between calls."""
    small = phantoms.small_multipool("me", seed=7, n=8, pools=2, spins=2, coils=3, n_tr=2)
    large = phantoms.small_multipool("me", seed=8, n=16, nz=2, pools=2, spins=2, coils=3, n_tr=2)
    monkeypatch.setenv("MRL_STAGE_MIN_MB", "100000")  # every copy direct
    ref = [engine.scan(sc) for sc in (small, large)]
    monkeypatch.setenv("MRL_STAGE_MIN_MB", "0")  # every copy staged
    for _ in range(2):
        for sc, r in zip((small, large), ref):
            out = engine.scan(sc)
            for k in ("Sx", "Sy", "Kx", "Mx", "My", "Mz"):
                np.testing.assert_array_equal(out[k], r[k])


def test_ext_plugin_callback(built):
    """An Ext plugin that spoils the transverse magnetisation (DoExtPlugin
    case 6) sees the state after the step that starts at the Ext sample."""
    sc = phantoms.config1_gre(seed=4, n=8, n_tr=3)
    lines, _ = phantoms.gre_lines(n_read=8, n_pe=3, fov=(0.24,) * 3, tr_ms=20.0, te_ms=(5.0,), flip=30.0,
                                  rf_ms=2.0, rf_raster_us=10.0, tbw=4.0, bw_hz=32000.0, ext_every=1)
    sc.VSeq = lines
    hs = engine.HostScan(sc, numerics="reference")
    calls = []

    def cb(args, what):
        calls.append(what)
        if what == engine.EXT_FETCH:
            return 1
        hs.keep["mx"][:] = 0
        hs.keep["my"][:] = 0
        return 0

    out = engine.run(hs, cb)
    assert calls == [engine.EXT_FETCH, engine.EXT_PLUGIN] * 3
    base = engine.scan(sc, numerics="reference")
    assert rel_l2(signal(out), signal(base)) > 1e-3
    # the same plugin in the CPU oracle (which runs it before the step that
    # starts at the Ext sample; that step is a 10 us free precession here)
    port = oracle.run_port(sc, "f32", ext_cb=lambda v, o: (o["Mx"].fill(0), o["My"].fill(0), 0)[-1])
    assert rel_l2(signal(out), signal(port)) <= 1e-3
    # a plugin error propagates as a status code
    hs2 = engine.HostScan(sc, numerics="reference")
    with pytest.raises(engine.ScanError) as e:
        engine.run(hs2, lambda args, what: 0 if what == engine.EXT_FETCH else 1)
    assert e.value.status == -4


def test_empty_object_gives_zero_signal(built):
    sc = phantoms.config1_gre(seed=0, n=8, n_tr=2)
    sc.VObj["Rho"][:] = 0
    sc.VObj["Mz"][:] = 0
    out = engine.scan(sc, numerics="reference")
    assert np.all(out["Sx"] == 0) and np.all(out["Sy"] == 0)
    assert np.count_nonzero(out["Kx"]) > 0


def test_multiple_partial_launches(built, monkeypatch):
    """A tiny partial budget splits the scan into many launches; the signal
    is unchanged."""
    sc, g = load_golden("gre2d_n16_tr4_seed1")
    monkeypatch.setenv("MRL_PARTIAL_MB", "0.0001")
    out = engine.scan(sc, numerics="reference")
    t = engine.last_timing()
    assert t["launches"] > 8
    assert rel_l2(signal(out), g["ref_Sx"] + 1j * g["ref_Sy"]) <= TOL_REF_CPU


# Accurate numerics: relative L2 of the complex signal against the all-FP64
# oracle (the reference algorithm in double precision).
TOL_FP64 = 1e-5


@pytest.mark.parametrize("name", SINGLE)
def test_accurate_numerics_vs_fp64_oracle(built, name):
    sc, g = load_golden(name)
    out = engine.scan(sc, numerics="accurate")
    f64 = g["f64_Sx"] + 1j * g["f64_Sy"]
    ref = g["ref_Sx"] + 1j * g["ref_Sy"]
    err64 = rel_l2(signal(out), f64)
    print(f"{name}: accurate GPU vs FP64 oracle {err64:.3e}; reference CPU engine vs FP64 {rel_l2(ref, f64):.3e}; "
          f"GPU vs reference CPU engine {rel_l2(signal(out), ref):.3e}")
    assert err64 <= TOL_FP64


@pytest.mark.parametrize("name", MULTI)
def test_accurate_multipool_vs_fp64_oracle(built, name):
    sc, g = load_golden(name)
    out = engine.scan(sc, numerics="accurate")
    f64 = g["f64_Sx"] + 1j * g["f64_Sy"]
    err64 = rel_l2(signal(out), f64)
    print(f"{name}: accurate GPU vs FP64 oracle {err64:.3e}, reference kernels vs FP64 "
          f"{rel_l2(g['ref_Sx'] + 1j * g['ref_Sy'], f64):.3e}")
    assert err64 <= TOL_FP64


@pytest.mark.parametrize("name", MULTI_TX)
def test_accurate_multi_tx_vs_fp64_oracle(built, name):
    sc, g = load_golden(name)
    out = engine.scan(sc, numerics="accurate")
    f64 = g["f64_Sx"] + 1j * g["f64_Sy"]
    err64 = rel_l2(signal(out), f64)
    print(f"{name}: accurate GPU vs FP64 oracle {err64:.3e}; reference CPU engine vs FP64 "
          f"{rel_l2(g['ref_Sx'] + 1j * g['ref_Sy'], f64):.3e}")
    assert err64 <= TOL_FP64


@pytest.mark.parametrize("spt", ["1", "2", "4"])
def test_accurate_spins_per_thread_agree(built, monkeypatch, spt):
    """The spins-per-thread tiling (an autotuned knob) does not change results."""
    sc, g = load_golden("mp_me_p2_s2_c2")
    sc = phantoms.small_multipool("me", seed=5, pools=2, spins=4, coils=3, n_tr=2)
    monkeypatch.setenv("MRL_SPINS_PER_THREAD", spt)
    out = engine.scan(sc, numerics="accurate")
    f64 = oracle.run_port(sc, "f64")
    assert rel_l2(signal(out), signal(f64)) <= TOL_FP64


def test_config2_full_length_subset(built):
    """The benchmark scan itself at its full length -- the two-pool
    multi-echo GRE's 256 TRs (220,416 steps), 4 spins, 8 Rx coils -- on a
    16 x 16 x 32 subset of its voxels spread over the field of view, against
    the all-FP64 oracle and the reference's own ME kernel (compiled from its
    source as host C) on the same voxels (committed at every 127th sample of
    each pool and coil signal).

    Over 220,416 steps the single-precision state's rounding walks: the
    reference kernel ends 2.5e-4 from FP64 (its FP32 restatement 2.2e-4)
    and two FP32 evaluations of the reference algorithm that differ only in
    their transcendental functions' rounding (the reference-order integrator
    on the GPU and the kernel on the host) end 1.5e-4 apart.  The accurate
    integrator rounds each isochromat's longitudinal state once per step
    (increment form) and ends 8.8e-6 from FP64, inside the 1e-5 bar (three
    roundings per step had walked to 2.4e-5)."""
    sc, g = load_golden("config2_full_length_subset")
    keep = g["sample_index"]
    P, C, A = int(sc.VObj["TypeNum"]), int(sc.VCoi["RxCoilNum"]), sc.signal_num
    out = engine.scan(sc, numerics="accurate")
    s_acc = signal(out).reshape(P, C, A)[..., keep]
    ref = engine.scan(sc, numerics="reference")
    s_ref = signal(ref).reshape(P, C, A)[..., keep]
    e64 = rel_l2(s_acc, g["f64_S"])
    e_acc_ref = rel_l2(s_acc, g["ref_S"])
    e_ro = rel_l2(s_ref, g["ref_S"])
    print(f"config 2 full length: accurate vs FP64 {e64:.3e}, accurate vs reference kernel {e_acc_ref:.3e}, "
          f"reference order vs reference kernel {e_ro:.3e}, reference order vs FP64 {rel_l2(s_ref, g['f64_S']):.3e}; "
          f"reference kernel vs FP64 {float(g['full_ref_vs_f64']):.3e}")
    ref_err = float(g["full_ref_vs_f64"])
    assert e64 <= 1e-5 and e64 <= 0.1 * ref_err
    # the reference-order integrator stays within the FP32 algorithm's own
    # spread around the reference kernel
    assert e_ro <= ref_err


def test_accurate_two_pool_3d_multiecho(built):
    """The benchmark workload's structure (two exchanging pools, 4 spins with
    intravoxel dephasing, 8 Rx coils, 6 echoes) on a shrunken object."""
    sc = phantoms.config2_me_gre(seed=0, nx=16, ny=16, nz=4, n_pe=4, n_par=2, n_read=32, n_tr=3)
    out = engine.scan(sc, numerics="accurate")
    f64 = oracle.run_port(sc, "f64")
    f32 = oracle.run_port(sc, "f32")
    err = rel_l2(signal(out), signal(f64))
    print(f"config2 shrunk: accurate GPU vs FP64 {err:.3e}; FP32 reference algorithm vs FP64 "
          f"{rel_l2(signal(f32), signal(f64)):.3e}")
    assert err <= TOL_FP64


def test_device_sincos_error_bounds(built):
    """The accurate kernel's own sine/cosine (Cody-Waite reduction + Taylor
    polynomials) against FP64 sin/cos of the same float arguments: absolute
    error within 2.5e-7 (about 2 ulp at 1) up to |x| = 1000, and relative
    error of the sine within 3e-7 for the small per-step rotation angles."""
    import ctypes

    lib = engine.library()
    fp = ctypes.POINTER(ctypes.c_float)
    lib.mrl_selftest_sincos.argtypes = [fp, fp, fp, ctypes.c_int]
    lib.mrl_selftest_sincos.restype = ctypes.c_int
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-np.pi, np.pi, 200000), rng.uniform(-1000, 1000, 200000),
                        np.geomspace(1e-9, 0.8, 20000), -np.geomspace(1e-9, 0.8, 20000),
                        np.arange(-64, 65) * (np.pi / 4), [0.0]]).astype(np.float32)
    sn = np.empty_like(x)
    cs = np.empty_like(x)
    rc = lib.mrl_selftest_sincos(x.ctypes.data_as(fp), sn.ctypes.data_as(fp), cs.ctypes.data_as(fp), x.size)
    assert rc == 0
    xd = x.astype(np.float64)
    err_s = np.abs(sn - np.sin(xd))
    err_c = np.abs(cs - np.cos(xd))
    print(f"max abs error: sin {err_s.max():.2e}, cos {err_c.max():.2e}")
    assert err_s.max() <= 2.5e-7 and err_c.max() <= 2.5e-7
    small = np.abs(xd) <= 0.8
    rel = err_s[small] / np.maximum(np.abs(np.sin(xd[small])), 1e-30)
    print(f"max relative sine error for |x| <= 0.8: {rel.max():.2e}")
    assert rel.max() <= 3e-7


def test_device_one_minus_exp_error_bounds(built):
    """The accurate kernel's 1 - exp(-x) (Taylor series below |x| = 1/16,
    expm1f above) against FP64 and against CUDA's expm1f on the same float
    arguments: relative error within 2e-7 (about 3 ulp) everywhere."""
    import ctypes

    lib = engine.library()
    fp = ctypes.POINTER(ctypes.c_float)
    lib.mrl_selftest_one_minus_exp.argtypes = [fp, fp, fp, ctypes.c_int]
    lib.mrl_selftest_one_minus_exp.restype = ctypes.c_int
    rng = np.random.default_rng(4)
    x = np.concatenate([np.geomspace(1e-12, 0.0625, 100000), -np.geomspace(1e-12, 0.0625, 20000),
                        rng.uniform(-0.0625, 0.0625, 100000), rng.uniform(0.0, 20.0, 50000),
                        [0.0, 0.0625, np.nextafter(np.float32(0.0625), np.float32(0))]]).astype(np.float32)
    ours = np.empty_like(x)
    lib_v = np.empty_like(x)
    rc = lib.mrl_selftest_one_minus_exp(x.ctypes.data_as(fp), ours.ctypes.data_as(fp), lib_v.ctypes.data_as(fp),
                                        x.size)
    assert rc == 0
    ref = -np.expm1(-x.astype(np.float64))
    nz = ref != 0
    rel = np.abs(ours[nz] - ref[nz]) / np.abs(ref[nz])
    rel_lib = np.abs(lib_v[nz] - ref[nz]) / np.abs(ref[nz])
    print(f"max relative error: ours {rel.max():.2e}, expm1f {rel_lib.max():.2e}")
    assert rel.max() <= 2e-7
    assert ours[x == 0].max() == 0.0


def test_tf32_rounding_matches_hardware_conversion(built):
    """The receive contraction rounds its TF32 operands with integer
    arithmetic; it must give the bits of cvt.rna.tf32.f32 for finite inputs."""
    import ctypes

    lib = engine.library()
    fp = ctypes.POINTER(ctypes.c_float)
    up = ctypes.POINTER(ctypes.c_uint32)
    lib.mrl_selftest_tf32.argtypes = [fp, up, up, ctypes.c_int]
    lib.mrl_selftest_tf32.restype = ctypes.c_int
    rng = np.random.default_rng(5)
    bits = rng.integers(0, 2**32, 400000, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    x = x[np.isfinite(x) & (np.abs(x) < 1e38)]
    x = np.concatenate([x, rng.standard_normal(100000).astype(np.float32), np.float32([0.0, -0.0, 1.0, 1e-40])])
    x = np.ascontiguousarray(x)
    rn = np.empty(x.size, np.uint32)
    cvt = np.empty(x.size, np.uint32)
    assert lib.mrl_selftest_tf32(x.ctypes.data_as(fp), rn.ctypes.data_as(up), cvt.ctypes.data_as(up), x.size) == 0
    assert np.array_equal(rn, cvt), f"{np.count_nonzero(rn != cvt)} of {x.size} differ"


# RunMode 1 history (relative L2 over every time point of every isochromat)
TOL_HIST = 1e-5


def _history(out):
    return np.stack([out["Mxs"], out["Mys"], out["Mzs"]])


def test_runmode1_history_single_pool(built):
    """VSig.Mx/My/Mz[slot] = state at uts[slot] and VSig.Muts, against the
    FP64 oracle's history and the reference CPU engine's step times; the
    history changes nothing else."""
    sc, g = load_golden("history_gre2d_n4_tr2_seed4")
    out = engine.scan(sc, numerics="accurate")
    ref64 = np.stack([g["f64_Mxs"], g["f64_Mys"], g["f64_Mzs"]])
    err = rel_l2(_history(out), ref64)
    print(f"RunMode 1 history vs FP64 oracle: {err:.2e}")
    assert err <= TOL_HIST
    np.testing.assert_array_equal(out["Muts"].ravel(), g["ref_Muts"].ravel())
    plain = sc.copy()
    plain.VCtl["RunMode"] = np.int32(0)
    out0 = engine.scan(plain, numerics="accurate")
    np.testing.assert_array_equal(out["Mx"], out0["Mx"])
    np.testing.assert_array_equal(signal(out), signal(out0))
    np.testing.assert_array_equal(out["Mzs"][-1], out["Mz"])


def test_runmode1_history_exchange_model(built):
    sc = phantoms.with_history(phantoms.small_multipool("me", seed=11, n=3, pools=2, spins=2, coils=1, n_tr=1))
    out = engine.scan(sc, numerics="accurate")
    ref = oracle.run_port(sc, "f64")
    err = rel_l2(_history(out), _history(ref))
    print(f"ME RunMode 1 history vs FP64 oracle: {err:.2e}")
    assert err <= TOL_HIST
    np.testing.assert_array_equal(out["Muts"], ref["Muts"])


def test_runmode1_needs_accurate_numerics(built):
    sc, _ = load_golden("history_gre2d_n4_tr2_seed4")
    with pytest.raises(engine.ScanError) as e:
        engine.scan(sc, numerics="reference")
    assert e.value.status == -6


@pytest.mark.gpu
@pytest.mark.parametrize("rf_ref", [0.0, 0.6])
def test_direct_receive_matches_partials(built, monkeypatch, rf_ref):
    """The direct receive (blocks add into the FP64 signal with atomics, used
    when the per-block partials would exceed the launch budget) gives the
    signal of the partial-sum path up to the order of FP64 additions."""
    from mrilab_gb300 import engine, phantoms

    sc = phantoms.config5_mt_epi(seed=5, nx=16, ny=16, nz=4, spins=2, n_coils=6, n_read=16, n_pe=16)
    sc.VVar["rfRef"] = np.float64(rf_ref)
    monkeypatch.setenv("MRL_RECEIVE", "partials")
    a = engine.scan(sc)
    monkeypatch.setenv("MRL_RECEIVE", "direct")
    b = engine.scan(sc)
    sa, sb = a["Sx"] + 1j * a["Sy"], b["Sx"] + 1j * b["Sy"]
    assert np.linalg.norm(sa) > 0
    assert np.linalg.norm(sa - sb) <= 1e-12 * np.linalg.norm(sa)
    np.testing.assert_array_equal(a["Mz"], b["Mz"])
    # and a prepared plan re-run twice in direct mode gives the same signal
    plan = engine.Plan(sc)
    try:
        for _ in range(2):
            plan.execute(None)
            out = plan.download()
            so = out["Sx"] + 1j * out["Sy"]
            assert np.linalg.norm(so - sb) <= 1e-12 * np.linalg.norm(sb)
    finally:
        plan.close()


@pytest.mark.gpu
def test_mt_epi_matches_fp64_oracle(built):
    """The 3-pool MT + exchange EPI (general model, bound pool, 32-coil
    class receive on a shrunken phantom) against the all-FP64 oracle.  The
    EPI's k-space encoding cancels most of each sample's sum, so FP32
    arithmetic shows more here: the reference algorithm in single precision
    is 2.7e-5 from FP64 on this case, the accurate kernel 1.4e-5 (the same
    with anchors at every step, without the MT pulse 1.0e-5); bound 2e-5."""
    from mrilab_gb300 import engine, phantoms
    import oracle

    sc = phantoms.config5_mt_epi(seed=6, nx=12, ny=12, nz=3, spins=2, n_coils=8, n_read=16, n_pe=16)
    ref = oracle.run_port(sc, "f64")
    out = engine.scan(sc)
    err = rel_l2(signal(out), signal(ref))
    port32 = rel_l2(signal(oracle.run_port(sc, "f32")), signal(ref))
    print(f"MT EPI shrunk: relative L2 {err:.2e} (reference algorithm in FP32: {port32:.2e})")
    assert err <= 2e-5 and err < port32


@pytest.mark.gpu
def test_many_coil_receive_matches_fp64_oracle(built):
    """More than 16 Rx coils: the coil maps stay float2 in shared memory and
    are split into TF32 parts in the receive flush (up to 16 they are split
    once per launch).  Against the all-FP64 oracle."""
    from mrilab_gb300 import engine, phantoms
    import oracle

    sc = phantoms.small_multipool("me", seed=61, n=8, pools=2, spins=2, coils=20, n_tr=2)
    assert int(sc.VCoi["RxCoilNum"]) == 20
    ref = oracle.run_port(sc, "f64")
    out = engine.scan(sc)
    err = rel_l2(signal(out), signal(ref))
    print(f"20 coils: relative L2 {err:.2e}")
    assert err <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("spins_per_thread", ["2", "1", "4"])
def test_tcgen05_receive_mt_epi_32_coils(built, monkeypatch, spins_per_thread):
    """The receive contraction on tcgen05 (17 to 32 coils): the MT + exchange
    EPI's model (general model, bound pool, 4 spins) with 32 Rx coils, two,
    four and one thread(s) per voxel (the voxels' spin sums are the
    contraction's K: 64, 32 and 128 voxels per block; the last taken on
    tcgen05 only when asked, MRL_RECEIVE_TC=1).  Against the all-FP64 oracle
    (the MT EPI bound, 2e-5) and against the warp-level TF32 contraction
    (MRL_RECEIVE_TC=0); the two results are not bit-identical, so both
    contractions ran."""
    from mrilab_gb300 import engine, phantoms
    import oracle

    sc = phantoms.config5_mt_epi(seed=7, nx=12, ny=12, nz=3, spins=4, n_coils=32, n_read=16, n_pe=16)
    assert int(sc.VCoi["RxCoilNum"]) == 32
    monkeypatch.setenv("MRL_SPINS_PER_THREAD", spins_per_thread)
    if spins_per_thread == "4":
        monkeypatch.setenv("MRL_RECEIVE_TC", "1")
    ref = oracle.run_port(sc, "f64")
    out_tc = engine.scan(sc)
    monkeypatch.setenv("MRL_RECEIVE_TC", "0")
    out_mma = engine.scan(sc)
    e_tc = rel_l2(signal(out_tc), signal(ref))
    e_mma = rel_l2(signal(out_mma), signal(ref))
    e_between = rel_l2(signal(out_tc), signal(out_mma))
    port32 = rel_l2(signal(oracle.run_port(sc, "f32")), signal(ref))
    print(f"32 coils, {spins_per_thread} spin(s) per thread: tcgen05 {e_tc:.2e}, warp-level {e_mma:.2e}, "
          f"between {e_between:.2e} (reference algorithm in FP32: {port32:.2e})")
    assert e_tc <= 2e-5 and e_tc < port32
    assert e_between <= 5e-6
    assert not np.array_equal(signal(out_tc), signal(out_mma))
    for k in ("Mx", "My", "Mz"):  # the final state does not depend on the receive
        np.testing.assert_array_equal(out_tc[k], out_mma[k])
