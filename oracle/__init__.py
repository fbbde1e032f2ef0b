"""CPU oracle for the MRiLab scan engine -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline / reference arm may use this package, and only as the reference
results the product is compared with or as the timed CPU baseline; the product (``mrilab_gb300``) never imports it.

Three oracles live here:

* ``run_port``: ``port/mrl_port.c``, a plain-C restatement of the reference
  scan algorithm (sequence decode ``DoScanAtCPU.cpp:246-420``; single-pool
  kernel ``BlochKernel.h``; ME/MT/CEST/GM kernels ``BlochKernel*.cuh``) in
  single precision (``"f32"``) and all-double (``"f64"``).  It travels with
  the repository and is built where it runs by ``build()``.
* ``run_ref_cpu``: the reference CPU engine itself
  (``Lib/src/engine/CPUEngine/DoScanAtCPU.cpp``), compiled unmodified from
  the reference tree against project-written mex/IPP shims into ``_ref/``
  by ``Makefile`` -- only where the reference tree exists (this container).
* ``run_ref_kernel``: the reference CUDA kernel headers compiled as host C
  (``_ref/libmrl_refkern.so``, driver ``ref_driver.c``), for the multi-pool
  models -- same availability as ``run_ref_cpu``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "port", "libmrl_port.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_CPU_SO = os.path.join(REF_DIR, "DoScanAtCPU.so")
REF_KERN_SO = os.path.join(REF_DIR, "libmrl_refkern.so")
# The MRiLab reference tree to build the reference objects from: taken from
# the environment only (no default); unset, only the port is built and the
# tests that need the reference objects skip.
REFERENCE_ROOT = os.environ.get("MRILAB_REFERENCE_ROOT", "")

MODEL_ID = {"normal": 0, "me": 1, "mt": 2, "cest": 3, "gm": 4}

_d = ctypes.POINTER(ctypes.c_double)
_f = ctypes.POINTER(ctypes.c_float)
_EXT_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_double)


class PortArgs(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("nz", ctypes.c_int),
        ("spin_num", ctypes.c_int), ("type_num", ctypes.c_int),
        ("tx_num", ctypes.c_int), ("rx_num", ctypes.c_int),
        ("gyro", ctypes.c_double),
        ("rho", _f), ("t1", _f), ("t2", _f), ("k", _f), ("type_flag", _d),
        ("mx", _f), ("my", _f), ("mz", _f),
        ("db0", _f), ("gzgrid", _f), ("gygrid", _f), ("gxgrid", _f), ("dwrnd", _f),
        ("tx_mg", _f), ("tx_pe", _f), ("rx_x", _f), ("rx_y", _f),
        ("tx_default", ctypes.c_double), ("rx_default", ctypes.c_double),
        ("cs", _d), ("rf_ref", ctypes.c_double),
        ("uts", _d), ("ts", _d), ("rf_amp", _d), ("rf_phase", _d), ("rf_freq", _d),
        ("rf_coil", _d), ("gz", _d), ("gy", _d), ("gx", _d), ("adc", _d), ("ext", _d),
        ("flags", _d),
        ("n_uts", ctypes.c_int), ("n_ts", ctypes.c_int), ("n_rf", ctypes.c_int),
        ("n_gz", ctypes.c_int), ("n_gy", ctypes.c_int), ("n_gx", ctypes.c_int),
        ("n_adc", ctypes.c_int), ("n_ext", ctypes.c_int),
        ("sx", _d), ("sy", _d), ("kx", _d), ("ky", _d), ("kz", _d),
        ("signal_num", ctypes.c_int), ("threads", ctypes.c_int),
        ("max_steps", ctypes.c_longlong),
        ("ext_cb", _EXT_CB), ("ext_user", ctypes.c_void_p),
        ("run_mode", ctypes.c_int), ("mxs", _f), ("mys", _f), ("mzs", _f), ("muts", _d),
        ("exact", ctypes.c_int),
        ("steps_out", _d), ("steps_cap", ctypes.c_longlong),
    ]


def build(force: bool = False) -> None:
    """Compile the port (always) and the reference objects (where the
    reference tree exists).  Building the oracle is not using it."""
    src = os.path.join(HERE, "port", "mrl_port.c")
    hdr = os.path.join(HERE, "port", "mrl_port_impl.h")
    if force or not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < max(
            os.path.getmtime(src), os.path.getmtime(hdr)):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", src, "-o", PORT_SO, "-lm"])
    if REFERENCE_ROOT:
        if not os.path.isdir(os.path.join(REFERENCE_ROOT, "Lib", "src", "engine")):
            raise RuntimeError(f"MRILAB_REFERENCE_ROOT={REFERENCE_ROOT!r} is not an MRiLab tree "
                               "(no Lib/src/engine)")
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REFROOT={REFERENCE_ROOT}"])
    elif os.path.isdir(os.path.join(REF_DIR, "stage")):
        # the reference kernel headers staged by `make stage` (a copy of the
        # working tree on a machine without the reference tree)
        subprocess.check_call(["make", "-s", "-C", HERE, "refkern"])


def ref_available() -> bool:
    return os.path.exists(REF_CPU_SO) and os.path.exists(REF_KERN_SO)


def ref_kernel_available() -> bool:
    """The reference's CUDA kernels compiled as host C (from the reference
    tree, or from its staged kernel headers)."""
    return os.path.exists(REF_KERN_SO)


def _ptr(a, typ):
    return a.ctypes.data_as(typ) if a is not None else ctypes.cast(None, typ)


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).ravel(order="F"))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, np.float64).ravel(order="F"))


def run_port(scan, precision: str = "f32", threads: int = 0, max_steps: int = -1,
             ext_cb=None, exact: bool = False, step_records: int = 0) -> Dict[str, np.ndarray]:
    """Run the C oracle on a ``phantoms.Scan``; returns Sx, Sy, Kx, Ky, Kz,
    final Mx, My, Mz (flattened column-major) and ``steps``.  ``exact``: the
    exact relaxation-exchange propagator instead of the reference's split
    exchange (ME, and GM with free and bound pools).  ``step_records`` > 0: also
    ``records``, the decoded dt > 0 steps ([steps][10 + 3 (Tx - 1)]: dt, Gz,
    Gy, Gx, Tx-0 amplitude, phase, frequency, rf_sum, ADC flag, signal
    index, then amplitude, phase, frequency of each further Tx coil), at
    most that many."""
    lib = ctypes.CDLL(PORT_SO)
    fn = lib.mrl_port_scan_f32 if precision == "f32" else lib.mrl_port_scan_f64
    fn.argtypes = [ctypes.POINTER(PortArgs), ctypes.POINTER(ctypes.c_longlong)]
    fn.restype = ctypes.c_int
    steps = ctypes.c_longlong(0)
    rec = np.zeros((max(step_records, 1), 10 + 3 * (int(scan.VCoi["TxCoilNum"]) - 1)))

    def call(args):
        if step_records > 0:
            args.steps_out = _ptr(rec, _d)
            args.steps_cap = step_records
        return fn(ctypes.byref(args), ctypes.byref(steps))

    out = _call_with_args(scan, call, threads, max_steps, ext_cb, exact)
    out["steps"] = int(steps.value)
    if step_records > 0:
        out["records"] = rec[: min(out["steps"], step_records)].copy()
    return out


def _call_with_args(scan, call, threads: int = 0, max_steps: int = -1, ext_cb=None,
                    exact: bool = False) -> Dict[str, np.ndarray]:
    o, m, c, ctl, q, sig = scan.VObj, scan.VMag, scan.VCoi, scan.VCtl, scan.VSeq, scan.VSig
    Y, X, Z = o["Rho"].shape[:3]
    keep = {}

    def F(name, arr):
        keep[name] = _f32(arr)
        return _ptr(keep[name], _f)

    def D(name, arr):
        keep[name] = _f64(arr)
        return _ptr(keep[name], _d)

    A = int(sig["SignalNum"])
    P = int(o["TypeNum"])
    RX = int(c["RxCoilNum"])
    out = dict(Sx=np.zeros(A * P * RX), Sy=np.zeros(A * P * RX), Kx=np.zeros(A), Ky=np.zeros(A), Kz=np.zeros(A),
               Mx=_f32(o["Mx"]).copy(), My=_f32(o["My"]).copy(), Mz=_f32(o["Mz"]).copy())
    args = PortArgs()
    args.model = MODEL_ID[scan.model]
    args.ny, args.nx, args.nz = Y, X, Z
    args.spin_num, args.type_num = int(o["SpinNum"]), P
    args.tx_num, args.rx_num = int(c["TxCoilNum"]), RX
    args.gyro = float(o["Gyro"])
    args.rho, args.t1, args.t2 = F("rho", o["Rho"]), F("t1", o["T1"]), F("t2", o["T2"])
    args.k = F("k", o["K"]) if "K" in o else ctypes.cast(None, _f)
    args.type_flag = D("tf", o["TypeFlag"]) if "TypeFlag" in o else ctypes.cast(None, _d)
    args.mx, args.my, args.mz = _ptr(out["Mx"], _f), _ptr(out["My"], _f), _ptr(out["Mz"], _f)
    args.db0, args.gzgrid, args.gygrid, args.gxgrid = (F("db0", m["dB0"]), F("gzgrid", m["Gzgrid"]),
                                                      F("gygrid", m["Gygrid"]), F("gxgrid", m["Gxgrid"]))
    args.dwrnd = F("dwrnd", m["dWRnd"])
    args.tx_mg, args.tx_pe = F("txmg", c["TxCoilmg"]), F("txpe", c["TxCoilpe"])
    args.rx_x, args.rx_y = F("rxx", c["RxCoilx"]), F("rxy", c["RxCoily"])
    args.tx_default, args.rx_default = float(c["TxCoilDefault"]), float(c["RxCoilDefault"])
    args.cs = D("cs", ctl["CS"])
    args.rf_ref = float(scan.VVar["rfRef"])
    for fld, key in [("uts", "utsLine"), ("ts", "tsLine"), ("rf_amp", "rfAmpLine"), ("rf_phase", "rfPhaseLine"),
                     ("rf_freq", "rfFreqLine"), ("rf_coil", "rfCoilLine"), ("gz", "GzAmpLine"),
                     ("gy", "GyAmpLine"), ("gx", "GxAmpLine"), ("adc", "ADCLine"), ("ext", "ExtLine"),
                     ("flags", "flagsLine")]:
        setattr(args, fld, D(fld, q[key]))
    args.n_uts, args.n_ts = q["utsLine"].size, q["tsLine"].size
    args.n_rf, args.n_gz, args.n_gy, args.n_gx = (q["rfAmpLine"].size, q["GzAmpLine"].size,
                                                  q["GyAmpLine"].size, q["GxAmpLine"].size)
    args.n_adc, args.n_ext = q["ADCLine"].size, q["ExtLine"].size
    args.sx, args.sy = _ptr(out["Sx"], _d), _ptr(out["Sy"], _d)
    args.kx, args.ky, args.kz = _ptr(out["Kx"], _d), _ptr(out["Ky"], _d), _ptr(out["Kz"], _d)
    args.signal_num = A
    args.threads = threads
    args.max_steps = max_steps
    if ext_cb is not None:
        cb = _EXT_CB(lambda user, val: int(ext_cb(val, out)))
        keep["cb"] = cb
        args.ext_cb = cb
    args.exact = int(bool(exact))
    args.run_mode = int(ctl["RunMode"])
    if args.run_mode == 1:  # history [len(uts)][P][S][V], slot 0 = the initial state (DoSpinWatchExec.m:152-161)
        for k in ("Mx", "My", "Mz"):
            h = np.zeros((q["utsLine"].size, out[k].size), np.float32)
            h[0] = out[k]
            out[k + "s"] = h
        out["Muts"] = np.zeros(q["utsLine"].size)
        args.mxs, args.mys, args.mzs = _ptr(out["Mxs"], _f), _ptr(out["Mys"], _f), _ptr(out["Mzs"], _f)
        args.muts = _ptr(out["Muts"], _d)
    rc = call(args)
    if rc != 0:
        raise RuntimeError(f"oracle returned {rc}")
    return out


def run_ref_cpu(scan, threads: int = 1) -> Dict[str, np.ndarray]:
    """Run the reference CPU engine (DoScanAtCPU, single-pool only) on the
    scan through the mex stand-in; returns its VSig/VObj outputs."""
    from mrilab_gb300 import mexsim

    if scan.model != "normal":
        raise ValueError("the reference CPU engine runs single-pool scans only (SimuPanel.m:876-889)")
    ms = mexsim.MexSession()
    structs = scan.structs()
    structs["VCtl"] = dict(structs["VCtl"], MaxThreadNum=np.int32(threads))
    for name, fields in structs.items():
        ms.set_global(name, fields)
    ms.call(REF_CPU_SO)
    out = {k: ms.get("VSig", k).ravel(order="F").copy() for k in ("Sx", "Sy", "Kx", "Ky", "Kz")}
    for k in ("Mx", "My", "Mz"):
        out[k] = ms.get("VObj", k).ravel(order="F").copy()
    if int(scan.VCtl["RunMode"]) == 1:  # history [len(uts)][P*S*V]
        n = scan.VSeq["utsLine"].size
        for k in ("Mx", "My", "Mz"):
            out[k + "s"] = ms.get("VSig", k).ravel(order="F").reshape(n, -1).copy()
        out["Muts"] = ms.get("VSig", "Muts").ravel(order="F").copy()
    return out


def run_ref_kernel(scan, threads: int = 0) -> Dict[str, np.ndarray]:
    """Run the reference's own CUDA kernel for the scan's model, compiled as
    host C (``_ref/libmrl_refkern.so``), through a restatement of the
    reference GPU host loop (``ref_driver.c``).  Same outputs as run_port."""
    lib = ctypes.CDLL(REF_KERN_SO)
    fn = getattr(lib, "mrl_refkern_run_" + scan.model)
    fn.argtypes = [ctypes.POINTER(PortArgs)]
    fn.restype = ctypes.c_int
    return _call_with_args(scan, lambda args: fn(ctypes.byref(args)), threads)
