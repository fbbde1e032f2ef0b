"""mrl_scan_noalloc: the scan entry point for callers that cannot allocate
device memory (a host application that owns the whole device heap and hands
out only its own buffers, such as a MATLAB session passing gpuArray storage
or a server with a fixed memory pool).  The caller owns every input and
output buffer --
here torch tensors stand in for them -- and the call must reproduce the
allocating entry point, mrl_scan, on the same inputs, call after call.

Kept in a file of its own that pytest collects last, so a failure here does
not stop the rest of the GPU suite."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2, signal
from mrilab_gb300 import engine, phantoms

pytestmark = pytest.mark.gpu

# same bar as the other accurate-numerics tests: relative L2 of the complex
# signal and of the final magnetisation
TOL = 1e-5


def _device_args(sc, torch):
    """ScanArgs whose arrays live in caller-owned device memory (torch)."""
    hs = engine.HostScan(sc, numerics="accurate")
    a = hs.args
    dev = {}

    def put(name, host, ctype):
        t = torch.from_numpy(np.ascontiguousarray(host)).cuda()
        dev[name] = t
        return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctype))

    K = hs.keep
    f = ctypes.c_float
    a.obj.rho, a.obj.t1, a.obj.t2 = put("rho", K["rho"], f), put("t1", K["t1"], f), put("t2", K["t2"], f)
    if "k" in K:
        a.obj.k = put("k", K["k"], f)
    a.obj.mx, a.obj.my, a.obj.mz = put("mx", K["mx"], f), put("my", K["my"], f), put("mz", K["mz"], f)
    a.mag.db0, a.mag.dwrnd = put("db0", K["db0"], f), put("dwrnd", K["dwrnd"], f)
    a.mag.gzgrid, a.mag.gygrid, a.mag.gxgrid = put("gzg", K["gzg"], f), put("gyg", K["gyg"], f), put("gxg", K["gxg"], f)
    a.coil.tx_mg, a.coil.tx_pe = put("txmg", K["txmg"], f), put("txpe", K["txpe"], f)
    a.coil.rx_x, a.coil.rx_y = put("rxx", K["rxx"], f), put("rxy", K["rxy"], f)
    a.sig.sx = put("sx", K["sx"], ctypes.c_double)
    a.sig.sy = put("sy", K["sy"], ctypes.c_double)
    n_uts = sc.VSeq["utsLine"].size
    steps = torch.empty(n_uts * 16, dtype=torch.float32, device="cuda")
    dev["steps"] = steps
    return hs, dev, steps


def _call(lib, hs, dev, steps):
    rc = lib.mrl_scan_noalloc(ctypes.byref(hs.args), ctypes.c_void_p(steps.data_ptr()),
                              ctypes.c_size_t(steps.numel() * 4), None)
    if rc != 0:
        raise engine.ScanError(rc, lib.mrl_last_error().decode())
    sx, sy = dev["sx"].cpu().numpy(), dev["sy"].cpu().numpy()
    return dict(Sx=sx, Sy=sy, Mx=dev["mx"].cpu().numpy(), My=dev["my"].cpu().numpy(), Mz=dev["mz"].cpu().numpy())


def _lib():
    lib = engine.library()
    lib.mrl_scan_noalloc.argtypes = [ctypes.POINTER(engine.ScanArgs), ctypes.c_void_p, ctypes.c_size_t,
                                     ctypes.c_void_p]
    lib.mrl_scan_noalloc.restype = ctypes.c_int
    return lib


@pytest.mark.parametrize("case", ["gre2d", "two_pool_coils", "split_launches"])
def test_noalloc_matches_mrl_scan_twice(built, case):
    torch = pytest.importorskip("torch")
    lib = _lib()
    if case == "gre2d":
        sc = phantoms.config1_gre(seed=2, n=32, n_tr=6)
    elif case == "two_pool_coils":
        sc = phantoms.small_multipool("me", seed=6, n=12, pools=2, spins=2, coils=3, n_tr=3)
    else:
        # 8192 voxels (at least 64 blocks of 128 threads), 2 pools x 8 Rx
        # coils: one sample's partial sums take at least 8 KiB, so the 32 MiB
        # scratch holds at most about 4090 samples and the scan's 6144 samples
        # take more than one launch
        sc = phantoms.config2_me_gre(seed=3, nx=32, ny=32, nz=8, n_pe=4, n_par=2, n_read=128, n_tr=8)
        assert sc.signal_num > 4096
    expect = engine.scan(sc, numerics="accurate")
    hs, dev, steps = _device_args(sc, torch)
    m0 = {k: dev[k].clone() for k in ("mx", "my", "mz")}
    # the engine resumes from the caller's pulse-packet cursor (VVar), as the
    # reference engines do; restart it for each scan as DoPreScan would
    var0 = {k: v.copy() for k, v in hs.keep.items() if k.startswith("var_")}
    for call in range(2):  # the shared static scratch is reused by the second call
        for k in ("mx", "my", "mz"):
            dev[k].copy_(m0[k])
        for k, v in var0.items():
            hs.keep[k][:] = v
        dev["sx"].zero_()
        dev["sy"].zero_()
        out = _call(lib, hs, dev, steps)
        launches = engine.last_timing()["launches"]
        err = rel_l2(signal(out), signal(expect))
        print(f"{case} call {call}: no-alloc vs mrl_scan signal {err:.2e} ({launches:.0f} launches)")
        assert err <= TOL
        for k in ("Mx", "My", "Mz"):
            assert rel_l2(out[k], expect[k]) <= TOL
        if case == "split_launches":
            assert launches > 1
            # and against the all-FP64 oracle
            if call == 0:
                import oracle

                f64 = oracle.run_port(sc, "f64")
                err64 = rel_l2(signal(out), signal(f64))
                print(f"split launches: no-alloc vs FP64 oracle {err64:.2e}")
                assert err64 <= TOL
        else:
            assert launches == 1


def test_noalloc_rejects_small_step_buffer(built):
    torch = pytest.importorskip("torch")
    lib = _lib()
    sc = phantoms.config1_gre(seed=2, n=8, n_tr=1)
    hs, dev, steps = _device_args(sc, torch)
    rc = lib.mrl_scan_noalloc(ctypes.byref(hs.args), ctypes.c_void_p(steps.data_ptr()), ctypes.c_size_t(64), None)
    assert rc == -1
    assert b"needed" in lib.mrl_last_error()


def test_noalloc_rejects_misaligned_step_buffer(built):
    """The step records are staged by bulk copies that need a 16-byte aligned
    source: a buffer at an odd offset is refused on the host, before any
    launch."""
    torch = pytest.importorskip("torch")
    lib = _lib()
    sc = phantoms.config1_gre(seed=2, n=8, n_tr=1)
    hs, dev, steps = _device_args(sc, torch)
    rc = lib.mrl_scan_noalloc(ctypes.byref(hs.args), ctypes.c_void_p(steps.data_ptr() + 4),
                              ctypes.c_size_t(steps.numel() * 4 - 16), None)
    assert rc == -1
    assert b"aligned" in lib.mrl_last_error()
