"""Python binding of the reconstruction's C ABI (``include/mrl_recon.h``):
``cart_recon`` (mrl_recon_cart: DoCartRecon.m / DoEPIRecon.m's transform on
the GPU) and ``grid2d`` (mrl_grid2d: the DoGridding mex).  No CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import engine

_d = ctypes.POINTER(ctypes.c_double)


class ReconArgs(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_int), ("sx", _d), ("sy", _d), ("res_freq", ctypes.c_int),
                ("lines", ctypes.c_int), ("slices", ctypes.c_int), ("rx", ctypes.c_int), ("pools", ctypes.c_int),
                ("echoes", ctypes.c_int), ("epi_etl", ctypes.c_int), ("zf_kx", ctypes.c_int),
                ("zf_ky", ctypes.c_int), ("zf_kz", ctypes.c_int), ("readout_first", ctypes.c_int),
                ("gpu_index", ctypes.c_int), ("img_real", _d), ("img_imag", _d), ("img_mag", _d),
                ("img_phase", _d), ("out_dims", ctypes.c_int * 3)]


def _lib():
    lib = engine.library()
    lib.mrl_recon_cart.argtypes = [ctypes.POINTER(ReconArgs)]
    lib.mrl_recon_cart.restype = ctypes.c_int
    lib.mrl_grid2d.argtypes = [_d, _d, _d, _d, _d, ctypes.c_int, _d, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               _d, _d, ctypes.c_int]
    lib.mrl_grid2d.restype = ctypes.c_int
    return lib


def out_dims(res_freq, lines, slices, epi_etl=0, zf=None, readout_first=False):
    """Image dims (N0, N1, N2) of a reconstruction."""
    F = res_freq - 1
    L = epi_etl * lines if epi_etl else lines
    fx, fy, fz = (zf[0], zf[1], zf[2] * slices) if zf is not None else (F, L, slices)
    return (fx, fy, fz) if readout_first else (fy, fx, fz)


def cart_recon(sx, sy, res_freq, lines, slices, rx, pools, echoes=1, epi_etl=0, zf=None, readout_first=False,
               gpu_index=0):
    """Images of a scan signal (VSig.Sx/Sy, column-major): Real, Imag, Mag
    and Phase as [N0][N1][N2][Rx][E] arrays (MATLAB layout)."""
    sx = np.ascontiguousarray(np.asarray(sx, np.float64).ravel(order="F"))
    sy = np.ascontiguousarray(np.asarray(sy, np.float64).ravel(order="F"))
    n = out_dims(res_freq, lines, slices, epi_etl, zf, readout_first)
    E = 1 if epi_etl else echoes
    shape = n + (rx, E)
    outs = {k: np.zeros(int(np.prod(shape))) for k in ("Real", "Imag", "Mag", "Phase")}
    a = ReconArgs()
    a.abi_version = engine.ABI_VERSION
    a.sx, a.sy = sx.ctypes.data_as(_d), sy.ctypes.data_as(_d)
    a.res_freq, a.lines, a.slices, a.rx, a.pools, a.echoes, a.epi_etl = (res_freq, lines, slices, rx, pools, E,
                                                                         epi_etl)
    if zf is not None:
        a.zf_kx, a.zf_ky, a.zf_kz = zf
    a.readout_first = int(bool(readout_first))
    a.gpu_index = gpu_index
    a.img_real, a.img_imag = outs["Real"].ctypes.data_as(_d), outs["Imag"].ctypes.data_as(_d)
    a.img_mag, a.img_phase = outs["Mag"].ctypes.data_as(_d), outs["Phase"].ctypes.data_as(_d)
    rc = _lib().mrl_recon_cart(ctypes.byref(a))
    if rc != 0:
        raise engine.ScanError(rc, engine.library().mrl_last_error().decode())
    assert tuple(a.out_dims) == n
    return {k: v.reshape(shape, order="F") for k, v in outs.items()}


def grid2d(kx, ky, sx, sy, dcf, kernel, grid_size, half_width, gpu_index=0):
    """Gridded (Sx2, Sy2), each [G * G] column-major (index ix * G + iy)."""
    arrs = [np.ascontiguousarray(np.asarray(v, np.float64).ravel()) for v in (kx, ky, sx, sy, dcf, kernel)]
    G = int(grid_size)
    gx, gy = np.zeros(G * G), np.zeros(G * G)
    p = [v.ctypes.data_as(_d) for v in arrs]
    rc = _lib().mrl_grid2d(p[0], p[1], p[2], p[3], p[4], arrs[0].size, p[5], arrs[5].size, G, float(half_width),
                           gx.ctypes.data_as(_d), gy.ctypes.data_as(_d), gpu_index)
    if rc != 0:
        raise engine.ScanError(rc, engine.library().mrl_last_error().decode())
    return gx, gy
