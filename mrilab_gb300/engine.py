"""Python binding of the scan engine's C ABI (``include/mrl_scan.h``).

``scan(sc, ...)`` runs one MRiLab scan on the GPU through ``mrl_scan`` --
the same call the mex wrappers make -- with the seven MATLAB structs of a
``phantoms.Scan`` passed as host arrays, exactly as the reference engines
receive them (``Lib/src/engine/GPUEngine/DoScanAtGPU.cu:117-214``).  There
is no CPU fallback: if ``libmrl_scan.so`` is missing or no GPU is usable the
call raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Callable, Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmrl_scan.so")

MODEL = {"normal": 0, "me": 1, "mt": 2, "cest": 3, "gm": 4}
NUMERICS = {"accurate": 0, "reference": 1, "exact": 2}
EXT_FETCH, EXT_PLUGIN = 1, 2
ABI_VERSION = 1

_d = ctypes.POINTER(ctypes.c_double)
_f = ctypes.POINTER(ctypes.c_float)
_i = ctypes.POINTER(ctypes.c_int)


class Object(ctypes.Structure):
    _fields_ = [("ny", ctypes.c_int), ("nx", ctypes.c_int), ("nz", ctypes.c_int), ("spin_num", ctypes.c_int),
                ("type_num", ctypes.c_int), ("gyro", ctypes.c_double), ("rho", _f), ("t1", _f), ("t2", _f),
                ("k", _f), ("k_channels", ctypes.c_int), ("type_flag", _d), ("mx", _f), ("my", _f), ("mz", _f)]


class Field(ctypes.Structure):
    _fields_ = [("db0", _f), ("dwrnd", _f), ("gzgrid", _f), ("gygrid", _f), ("gxgrid", _f)]


class Coils(ctypes.Structure):
    _fields_ = [("tx_num", ctypes.c_int), ("rx_num", ctypes.c_int), ("tx_default", ctypes.c_double),
                ("rx_default", ctypes.c_double), ("tx_mg", _f), ("tx_pe", _f), ("rx_x", _f), ("rx_y", _f)]


class Control(ctypes.Structure):
    _fields_ = [("cs", _d), ("tr_num", ctypes.c_int), ("run_mode", ctypes.c_int), ("gpu_index", ctypes.c_int),
                ("numerics", ctypes.c_int)]


class Sequence(ctypes.Structure):
    _fields_ = [(n, _d) for n in ("uts", "ts", "rf_amp", "rf_phase", "rf_freq", "rf_coil", "gz", "gy", "gx",
                                  "adc", "ext", "flags")] + \
               [(n, ctypes.c_int) for n in ("n_uts", "n_ts", "n_rf", "n_gz", "n_gy", "n_gx", "n_adc", "n_ext")]


class State(ctypes.Structure):
    _fields_ = [(n, _d) for n in ("t", "dt", "rf_amp", "rf_phase", "rf_freq", "rf_coil", "rf_ref", "gz", "gy",
                                  "gx", "adc", "ext", "kz", "ky", "kx", "gpu_fetch")] + \
               [(n, _i) for n in ("utsi", "rfi", "gzi", "gyi", "gxi", "adci", "exti", "tr_count")]


class Signal(ctypes.Structure):
    _fields_ = [("sx", _d), ("sy", _d), ("kz", _d), ("ky", _d), ("kx", _d), ("signal_num", ctypes.c_int),
                ("mxs", _f), ("mys", _f), ("mzs", _f), ("muts", _d)]


class ScanArgs(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_int), ("model", ctypes.c_int), ("obj", Object), ("mag", Field),
                ("coil", Coils), ("ctl", Control), ("seq", Sequence), ("var", State), ("sig", Signal)]


EXT_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ScanArgs), ctypes.c_int)

_lib: Optional[ctypes.CDLL] = None


def library() -> ctypes.CDLL:
    """Load libmrl_scan.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        lib = ctypes.CDLL(LIB_PATH)
        lib.mrl_scan.argtypes = [ctypes.POINTER(ScanArgs), EXT_FN, ctypes.c_void_p]
        lib.mrl_scan.restype = ctypes.c_int
        lib.mrl_status_string.argtypes = [ctypes.c_int]
        lib.mrl_status_string.restype = ctypes.c_char_p
        lib.mrl_last_error.restype = ctypes.c_char_p
        lib.mrl_last_timing.argtypes = [ctypes.POINTER(ctypes.c_double)]
        lib.mrl_last_timing.restype = ctypes.c_int
        _lib = lib
    return _lib


class ScanError(RuntimeError):
    def __init__(self, status: int, detail: str):
        super().__init__(f"mrl_scan failed ({status}): {detail}")
        self.status = status


def _flat(a, dtype, copy=True):
    """Column-major flat array of ``a``.  Arrays the engine writes (magnetisation,
    signal, pulse-packet cursor) are always copies, so a scan leaves the
    caller's structs unchanged; read-only inputs that already have MATLAB's
    layout and the right type are passed through without a copy."""
    a = np.asarray(a, dtype)
    if not copy and a.flags.f_contiguous:
        return a.reshape(-1, order="F")
    return a.flatten(order="F")


# host arrays mrl_scan writes into
_WRITTEN = frozenset({"mx", "my", "mz", "sx", "sy", "skz", "sky", "skx", "hmx", "hmy", "hmz", "muts"})


class HostScan:
    """Column-major host copies of a Scan's arrays, bound into ScanArgs.

    ``inplace``: the engine writes the final magnetisation and the signal
    into the caller's arrays themselves, as the reference engines write the
    MATLAB globals (``DoScanAtGPU.cu:124-214`` binds them with
    ``mxGetPr``); arrays without the engine's type and column-major layout
    are still copied.  By default every written array is a copy, so a scan
    leaves the caller's structs unchanged."""

    def __init__(self, sc, model: Optional[str] = None, numerics: str = "accurate", gpu_index: int = 0,
                 inplace: bool = False):
        self.sc = sc
        o, m, c, ctl, q, v, sig = sc.VObj, sc.VMag, sc.VCoi, sc.VCtl, sc.VSeq, sc.VVar, sc.VSig
        self.keep = {}
        K = self.keep
        # inputs the engine only reads may alias the caller's arrays
        wr = lambda k: k in _WRITTEN and not inplace
        f32 = lambda k, a: K.setdefault(k, _flat(a, np.float32, copy=wr(k)))
        f64 = lambda k, a: K.setdefault(k, _flat(a, np.float64, copy=wr(k) or k.startswith("var_")))
        i32 = lambda k, a: K.setdefault(k, _flat(a, np.int32, copy=True))
        p = lambda a, t: a.ctypes.data_as(t)
        a = ScanArgs()
        a.abi_version = ABI_VERSION
        a.model = MODEL[model or sc.model]
        Y, X, Z = o["Rho"].shape[:3]
        V = Y * X * Z
        ob = a.obj
        ob.ny, ob.nx, ob.nz = Y, X, Z
        ob.spin_num, ob.type_num = int(o["SpinNum"]), int(o["TypeNum"])
        ob.gyro = float(o["Gyro"])
        ob.rho, ob.t1, ob.t2 = p(f32("rho", o["Rho"]), _f), p(f32("t1", o["T1"]), _f), p(f32("t2", o["T2"]), _f)
        if "K" in o:
            ob.k = p(f32("k", o["K"]), _f)
            ob.k_channels = K["k"].size // V
        if "TypeFlag" in o:
            ob.type_flag = p(f64("tf", o["TypeFlag"]), _d)
        ob.mx, ob.my, ob.mz = (p(f32("mx", o["Mx"]), _f), p(f32("my", o["My"]), _f), p(f32("mz", o["Mz"]), _f))
        fm = a.mag
        fm.db0, fm.dwrnd = p(f32("db0", m["dB0"]), _f), p(f32("dwrnd", m["dWRnd"]), _f)
        fm.gzgrid, fm.gygrid, fm.gxgrid = (p(f32("gzg", m["Gzgrid"]), _f), p(f32("gyg", m["Gygrid"]), _f),
                                           p(f32("gxg", m["Gxgrid"]), _f))
        co = a.coil
        co.tx_num, co.rx_num = int(c["TxCoilNum"]), int(c["RxCoilNum"])
        co.tx_default, co.rx_default = float(c["TxCoilDefault"]), float(c["RxCoilDefault"])
        co.tx_mg, co.tx_pe = p(f32("txmg", c["TxCoilmg"]), _f), p(f32("txpe", c["TxCoilpe"]), _f)
        co.rx_x, co.rx_y = p(f32("rxx", c["RxCoilx"]), _f), p(f32("rxy", c["RxCoily"]), _f)
        ct = a.ctl
        ct.cs = p(f64("cs", ctl["CS"]), _d)
        ct.tr_num, ct.run_mode = int(ctl["TRNum"]), int(ctl["RunMode"])
        ct.gpu_index = gpu_index
        ct.numerics = NUMERICS[numerics]
        sq = a.seq
        for fld, key in [("uts", "utsLine"), ("ts", "tsLine"), ("rf_amp", "rfAmpLine"), ("rf_phase", "rfPhaseLine"),
                         ("rf_freq", "rfFreqLine"), ("rf_coil", "rfCoilLine"), ("gz", "GzAmpLine"),
                         ("gy", "GyAmpLine"), ("gx", "GxAmpLine"), ("adc", "ADCLine"), ("ext", "ExtLine"),
                         ("flags", "flagsLine")]:
            setattr(sq, fld, p(f64("seq_" + fld, q[key]), _d))
        sq.n_uts, sq.n_ts = q["utsLine"].size, q["tsLine"].size
        sq.n_rf, sq.n_gz, sq.n_gy, sq.n_gx = (q["rfAmpLine"].size, q["GzAmpLine"].size, q["GyAmpLine"].size,
                                              q["GxAmpLine"].size)
        sq.n_adc, sq.n_ext = q["ADCLine"].size, q["ExtLine"].size
        st = a.var
        for fld, key in [("t", "t"), ("dt", "dt"), ("rf_amp", "rfAmp"), ("rf_phase", "rfPhase"),
                         ("rf_freq", "rfFreq"), ("rf_coil", "rfCoil"), ("rf_ref", "rfRef"), ("gz", "GzAmp"),
                         ("gy", "GyAmp"), ("gx", "GxAmp"), ("adc", "ADC"), ("ext", "Ext"), ("kz", "Kz"),
                         ("ky", "Ky"), ("kx", "Kx"), ("gpu_fetch", "gpuFetch")]:
            setattr(st, fld, p(f64("var_" + fld, v[key]), _d))
        for fld, key in [("utsi", "utsi"), ("rfi", "rfi"), ("gzi", "Gzi"), ("gyi", "Gyi"), ("gxi", "Gxi"),
                         ("adci", "ADCi"), ("exti", "Exti"), ("tr_count", "TRCount")]:
            setattr(st, fld, p(i32("var_" + fld, v[key]), _i))
        sg = a.sig
        sg.sx, sg.sy = p(f64("sx", sig["Sx"]), _d), p(f64("sy", sig["Sy"]), _d)
        sg.kz, sg.ky, sg.kx = p(f64("skz", sig["Kz"]), _d), p(f64("sky", sig["Ky"]), _d), p(f64("skx", sig["Kx"]), _d)
        sg.signal_num = int(sig["SignalNum"])
        if ct.run_mode == 1:  # RunMode 1 history, written by the engine
            sg.mxs, sg.mys, sg.mzs = (p(f32("hmx", sig["Mx"]), _f), p(f32("hmy", sig["My"]), _f),
                                      p(f32("hmz", sig["Mz"]), _f))
            sg.muts = p(f64("muts", sig["Muts"]), _d)
        self.args = a

    def outputs(self) -> Dict[str, np.ndarray]:
        K = self.keep
        out = dict(Sx=K["sx"], Sy=K["sy"], Kx=K["skx"], Ky=K["sky"], Kz=K["skz"], Mx=K["mx"], My=K["my"],
                   Mz=K["mz"], TRCount=int(K["var_tr_count"][0]), utsi=int(K["var_utsi"][0]))
        if "hmx" in K:  # RunMode 1 history [len(uts)][P*S*V]
            n = K["muts"].size
            out.update(Mxs=K["hmx"].reshape(n, -1), Mys=K["hmy"].reshape(n, -1), Mzs=K["hmz"].reshape(n, -1),
                       Muts=K["muts"])
        return out


def last_timing() -> Dict[str, float]:
    buf = (ctypes.c_double * 8)()
    library().mrl_last_timing(buf)
    return dict(total_ms=buf[0], scan_ms=buf[1], reduce_ms=buf[2], h2d_ms=buf[3], d2h_ms=buf[4],
                launches=int(buf[5]), h2d_bytes=int(buf[6]), d2h_bytes=int(buf[7]))


def run(hs: HostScan, ext: Optional[Callable[[ScanArgs, int], int]] = None) -> Dict[str, np.ndarray]:
    lib = library()
    cb = EXT_FN(lambda user, args, what: int(ext(args.contents, what)) if ext else 0)
    rc = lib.mrl_scan(ctypes.byref(hs.args), cb, None)
    if rc != 0:
        raise ScanError(rc, lib.mrl_last_error().decode())
    return hs.outputs()


def scan(sc, model: Optional[str] = None, numerics: str = "accurate", gpu_index: int = 0,
         ext: Optional[Callable[[ScanArgs, int], int]] = None, inplace: bool = False) -> Dict[str, np.ndarray]:
    """Run ``sc`` (a phantoms.Scan) on the GPU; returns Sx, Sy, Kx, Ky, Kz and
    the final Mx, My, Mz (flattened column-major), leaving ``sc`` unchanged
    unless ``inplace`` (then the final state and the signal are written into
    ``sc``'s own arrays, as the mex entry points write the MATLAB globals)."""
    return run(HostScan(sc, model=model, numerics=numerics, gpu_index=gpu_index, inplace=inplace), ext)


def decode(sc) -> np.ndarray:
    """``mrl_decode``: the dt > 0 steps of ``sc``'s sequence as the engine
    decodes them (host only, no device), one row each: dt, Gz, Gy, Gx, ADC
    sample index (-1: none), then amplitude, phase and frequency of every Tx
    coil."""
    lib = library()
    lib.mrl_decode.argtypes = [ctypes.POINTER(ScanArgs), ctypes.POINTER(ctypes.c_double), ctypes.c_longlong,
                               ctypes.POINTER(ctypes.c_longlong)]
    hs = HostScan(sc)
    stride = 5 + 3 * int(sc.VCoi["TxCoilNum"])
    n = ctypes.c_longlong(0)
    rc = lib.mrl_decode(ctypes.byref(hs.args), None, 0, ctypes.byref(n))
    if rc != 0 and n.value == 0:
        raise ScanError(rc, lib.mrl_last_error().decode())
    out = np.zeros((max(n.value, 1), stride))
    rc = lib.mrl_decode(ctypes.byref(hs.args), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n.value,
                        ctypes.byref(n))
    if rc != 0:
        raise ScanError(rc, lib.mrl_last_error().decode())
    return out[: n.value]


class Plan:
    """A prepared scan (``mrl_plan``): inputs resident on the device, the
    sequence decoded once; ``execute(stream)`` re-runs the whole scan from
    the initial magnetisation without host work."""

    def __init__(self, sc, model: Optional[str] = None, numerics: str = "accurate", gpu_index: int = 0):
        lib = library()
        lib.mrl_plan_create.argtypes = [ctypes.POINTER(ScanArgs), ctypes.POINTER(ctypes.c_void_p)]
        lib.mrl_plan_execute.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.mrl_plan_download.argtypes = [ctypes.c_void_p, ctypes.POINTER(ScanArgs)]
        lib.mrl_plan_work.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]
        lib.mrl_plan_destroy.argtypes = [ctypes.c_void_p]
        self.lib = lib
        self.host = HostScan(sc, model=model, numerics=numerics, gpu_index=gpu_index)
        self.ptr = ctypes.c_void_p()
        rc = lib.mrl_plan_create(ctypes.byref(self.host.args), ctypes.byref(self.ptr))
        if rc != 0:
            raise ScanError(rc, lib.mrl_last_error().decode())

    def work(self) -> Dict[str, int]:
        buf = (ctypes.c_longlong * 5)()
        self.lib.mrl_plan_work(self.ptr, buf)
        return dict(units=buf[0], steps=buf[1], rf_steps=buf[2], samples=buf[3], launches=buf[4])

    def execute(self, stream: int = 0) -> None:
        rc = self.lib.mrl_plan_execute(self.ptr, ctypes.c_void_p(stream))
        if rc != 0:
            raise ScanError(rc, self.lib.mrl_last_error().decode())

    def download(self) -> Dict[str, np.ndarray]:
        rc = self.lib.mrl_plan_download(self.ptr, ctypes.byref(self.host.args))
        if rc != 0:
            raise ScanError(rc, self.lib.mrl_last_error().decode())
        return self.host.outputs()

    def close(self) -> None:
        if self.ptr:
            self.lib.mrl_plan_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


BATCH_MODES = {"persistent": 0, "plain": 1}


class Batch:
    """Many independent scans prepared together (``mrl_batch``): one
    persistent launch per kernel instantiation runs them all
    (``execute("persistent")``, captured into a CUDA graph on first use), or
    one launch per instance in turn (``execute("plain")``)."""

    def __init__(self, scans, numerics: str = "accurate", gpu_index: int = 0):
        lib = library()
        vp = ctypes.c_void_p
        lib.mrl_batch_create.argtypes = [ctypes.POINTER(ctypes.POINTER(ScanArgs)), ctypes.c_int, ctypes.POINTER(vp)]
        lib.mrl_batch_tune.argtypes = [vp, vp]
        lib.mrl_batch_execute.argtypes = [vp, ctypes.c_int, vp]
        lib.mrl_batch_download.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(ScanArgs)), ctypes.c_int]
        lib.mrl_batch_work.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        lib.mrl_batch_destroy.argtypes = [vp]
        self.lib = lib
        self.hosts = [HostScan(sc, numerics=numerics, gpu_index=gpu_index) for sc in scans]
        n = len(self.hosts)
        self._arr = (ctypes.POINTER(ScanArgs) * n)(*[ctypes.pointer(h.args) for h in self.hosts])
        self.ptr = vp()
        self._check(lib.mrl_batch_create(self._arr, n, ctypes.byref(self.ptr)))

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise ScanError(rc, self.lib.mrl_last_error().decode())

    def tune(self) -> None:
        self._check(self.lib.mrl_batch_tune(self.ptr, None))

    def execute(self, mode: str = "persistent", stream: int = 0) -> None:
        self._check(self.lib.mrl_batch_execute(self.ptr, BATCH_MODES[mode], ctypes.c_void_p(stream)))

    def download(self):
        self._check(self.lib.mrl_batch_download(self.ptr, self._arr, len(self.hosts)))
        return [h.outputs() for h in self.hosts]

    def work(self) -> Dict[str, int]:
        buf = (ctypes.c_longlong * 5)()
        self.lib.mrl_batch_work(self.ptr, buf)
        return dict(units=buf[0], steps=buf[1], samples=buf[2], launches=buf[3], plain_launches=buf[4])

    def close(self) -> None:
        if self.ptr:
            self.lib.mrl_batch_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def scan_batched(scans, numerics: str = "accurate", gpu_index: int = 0, inplace: bool = False):
    """``mrl_scan_batched``: every scan of ``scans`` in one batched pass;
    returns their outputs like ``scan`` (``inplace`` as there)."""
    lib = library()
    lib.mrl_scan_batched.argtypes = [ctypes.POINTER(ctypes.POINTER(ScanArgs)), ctypes.c_int]
    hosts = [HostScan(sc, numerics=numerics, gpu_index=gpu_index, inplace=inplace) for sc in scans]
    arr = (ctypes.POINTER(ScanArgs) * len(hosts))(*[ctypes.pointer(h.args) for h in hosts])
    rc = lib.mrl_scan_batched(arr, len(hosts))
    if rc != 0:
        raise ScanError(rc, lib.mrl_last_error().decode())
    return [h.outputs() for h in hosts]


class AdjointArgs(ctypes.Structure):
    _fields_ = [("grad_sx", _d), ("grad_sy", _d), ("g_t1", _f), ("g_t2", _f), ("g_rho", _f), ("g_db0", _f),
                ("g_k", _f), ("g_mx0", _f), ("g_my0", _f), ("g_mz0", _f), ("g_rf", _d), ("rf_a", _d),
                ("rf_step_uts", ctypes.POINTER(ctypes.c_int)), ("rf_capacity", ctypes.c_int),
                ("n_rf_steps", ctypes.c_int), ("g_rf_amp_line", _d), ("g_rf_phase_line", _d)]


def _adjoint_outputs(sc, rf_capacity: Optional[int]):
    """Host arrays for the gradients of ``sc`` and the AdjointArgs pointing at them."""
    o = sc.VObj
    V = o["Rho"].size // int(o["TypeNum"])
    P, S = int(o["TypeNum"]), int(o["SpinNum"])
    if rf_capacity is None:
        rf_capacity = int(np.count_nonzero(np.diff(sc.VSeq["utsLine"]) > 0))
    n_line = max(int(np.size(sc.VSeq["rfAmpLine"])), 1)
    tx = int(sc.VCoi["TxCoilNum"])
    rf_shape = (max(rf_capacity, 1), 2) if tx == 1 else (max(rf_capacity, 1), tx, 2)  # [step][coil][re, im]
    out = dict(T1=np.zeros(P * V, np.float32), T2=np.zeros(P * V, np.float32), Rho=np.zeros(P * V, np.float32),
               dB0=np.zeros(V, np.float32), Mx0=np.zeros(P * S * V, np.float32),
               My0=np.zeros(P * S * V, np.float32), Mz0=np.zeros(P * S * V, np.float32),
               rf=np.zeros(rf_shape), rf_a=np.zeros(rf_shape),
               rf_uts=np.zeros(max(rf_capacity, 1), np.int32),
               rf_amp_line=np.zeros(n_line), rf_phase_line=np.zeros(n_line))
    if "K" in o:
        out["K"] = np.zeros(o["K"].size, np.float32)
    a = AdjointArgs()
    f = lambda k: out[k].ctypes.data_as(_f) if k in out else ctypes.cast(None, _f)
    a.g_t1, a.g_t2, a.g_rho, a.g_db0, a.g_k = f("T1"), f("T2"), f("Rho"), f("dB0"), f("K")
    a.g_mx0, a.g_my0, a.g_mz0 = f("Mx0"), f("My0"), f("Mz0")
    a.g_rf = out["rf"].ctypes.data_as(_d)
    a.rf_a = out["rf_a"].ctypes.data_as(_d)
    a.rf_step_uts = out["rf_uts"].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    a.rf_capacity = rf_capacity
    a.g_rf_amp_line = out["rf_amp_line"].ctypes.data_as(_d)
    a.g_rf_phase_line = out["rf_phase_line"].ctypes.data_as(_d)
    return out, a


def _trim_rf(out, n):
    out["rf"], out["rf_a"], out["rf_uts"] = out["rf"][:n], out["rf_a"][:n], out["rf_uts"][:n]
    return out


def adjoint(sc, grad_sx, grad_sy, gpu_index: int = 0, rf_capacity: Optional[int] = None) -> Dict[str, np.ndarray]:
    """``mrl_adjoint``: gradients of a loss L of the signal of ``sc`` given
    dL/dSx, dL/dSy (flat [P][Rx][A]).  Returns T1, T2, Rho ([P*V]), dB0
    ([V]), K ([nK*V], exchange models), Mx0/My0/Mz0 ([P*S*V]), rf ([n_rf, 2]:
    dL/dRe A, dL/dIm A per rf-on step; [n_rf, Tx, 2] per Tx coil with
    several, zero for a coil that is off at that step), rf_a (their A),
    rf_uts (their uts indices) and rf_amp_line, rf_phase_line (dL/d
    VSeq.rfAmpLine and dL/d VSeq.rfPhaseLine, each coil's entries)."""
    lib = library()
    lib.mrl_adjoint.argtypes = [ctypes.POINTER(ScanArgs), ctypes.POINTER(AdjointArgs)]
    lib.mrl_adjoint.restype = ctypes.c_int
    hs = HostScan(sc, numerics="accurate", gpu_index=gpu_index)
    gsx = np.ascontiguousarray(np.asarray(grad_sx, np.float64).ravel())
    gsy = np.ascontiguousarray(np.asarray(grad_sy, np.float64).ravel())
    out, a = _adjoint_outputs(sc, rf_capacity)
    a.grad_sx, a.grad_sy = gsx.ctypes.data_as(_d), gsy.ctypes.data_as(_d)
    rc = lib.mrl_adjoint(ctypes.byref(hs.args), ctypes.byref(a))
    if rc != 0:
        raise ScanError(rc, lib.mrl_last_error().decode())
    return _trim_rf(out, a.n_rf_steps)


class AdjointPlan:
    """``mrl_adjoint_plan``: the forward scan (writing checkpoints) and the
    adjoint of one scan, resident on the device for repeated iterations:
    ``forward(stream)``, ``signal()``, ``backward(gx, gy, stream)``,
    ``gradients()``."""

    def __init__(self, sc, gpu_index: int = 0):
        lib = library()
        lib.mrl_adjoint_plan_create.argtypes = [ctypes.POINTER(ScanArgs), ctypes.POINTER(ctypes.c_void_p)]
        lib.mrl_adjoint_plan_forward.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        lib.mrl_adjoint_plan_download.argtypes = [ctypes.c_void_p, ctypes.POINTER(ScanArgs)]
        lib.mrl_adjoint_plan_backward.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_void_p]
        lib.mrl_adjoint_plan_gradients.argtypes = [ctypes.c_void_p, ctypes.POINTER(AdjointArgs)]
        lib.mrl_adjoint_plan_work.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]
        lib.mrl_adjoint_plan_checkpoints.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]
        lib.mrl_adjoint_plan_destroy.argtypes = [ctypes.c_void_p]
        self.lib = lib
        self.sc = sc
        self.host = HostScan(sc, numerics="accurate", gpu_index=gpu_index)
        self.ptr = ctypes.c_void_p()
        rc = lib.mrl_adjoint_plan_create(ctypes.byref(self.host.args), ctypes.byref(self.ptr))
        if rc != 0:
            raise ScanError(rc, lib.mrl_last_error().decode())
        self._out, self._args = _adjoint_outputs(sc, None)

    def _check(self, rc):
        if rc != 0:
            raise ScanError(rc, self.lib.mrl_last_error().decode())

    def work(self) -> Dict[str, int]:
        buf = (ctypes.c_longlong * 6)()
        self.lib.mrl_adjoint_plan_work(self.ptr, buf)
        return dict(units=buf[0], steps=buf[1], rf_steps=buf[2], samples=buf[3], launches=buf[4], n_rf=buf[5])

    def checkpoints(self) -> Dict[str, int]:
        """Steps between stored checkpoints, between the checkpoints the
        backward walk starts from, and their device bytes."""
        buf = (ctypes.c_longlong * 3)()
        self._check(self.lib.mrl_adjoint_plan_checkpoints(self.ptr, buf))
        return dict(stored_every=buf[0], window=buf[1], bytes=buf[2])

    def forward(self, stream: Optional[int] = None) -> None:
        self._check(self.lib.mrl_adjoint_plan_forward(self.ptr, ctypes.c_void_p(stream or 0)))

    def signal(self) -> Dict[str, np.ndarray]:
        """Signal and final magnetisation of the last forward pass."""
        self._check(self.lib.mrl_adjoint_plan_download(self.ptr, ctypes.byref(self.host.args)))
        return self.host.outputs()

    def backward(self, grad_sx, grad_sy, stream: Optional[int] = None) -> None:
        self._gx = np.ascontiguousarray(np.asarray(grad_sx, np.float64).ravel())
        self._gy = np.ascontiguousarray(np.asarray(grad_sy, np.float64).ravel())
        self._check(self.lib.mrl_adjoint_plan_backward(self.ptr, self._gx.ctypes.data_as(_d),
                                                       self._gy.ctypes.data_as(_d), ctypes.c_void_p(stream or 0)))

    def gradients(self) -> Dict[str, np.ndarray]:
        self._check(self.lib.mrl_adjoint_plan_gradients(self.ptr, ctypes.byref(self._args)))
        return _trim_rf({k: v.copy() for k, v in self._out.items()}, self._args.n_rf_steps)

    def close(self) -> None:
        if self.ptr:
            self.lib.mrl_adjoint_plan_destroy(self.ptr)
            self.ptr = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
