"""CPU oracle of the reconstruction -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` may use this module, as the reference results; the product
never imports it.

* ``cart_recon``: numpy restatement of the default Cartesian and EPI
  reconstructions, ``Src/Recon/Default/DoCartRecon.m:10-88`` and
  ``DoEPIRecon.m:10-95`` (pool sum, echo split / EPI line sorting with every
  second echo of the train reversed, last readout point dropped, zero
  filling, orientation, fftshift(ifftn(fftshift(.))) per coil) in FP64;
* ``grid2d_port``: restatement of the gridding mex
  ``Lib/src/recon/DoGridding/DoGridding.cpp:54-124`` in FP64;
* ``run_ref_grid``: that mex itself, compiled unmodified from the reference
  tree into ``_ref/DoGridding.so`` (where the reference tree is mounted).
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_GRID_SO = os.path.join(HERE, "_ref", "DoGridding.so")


def ref_grid_available() -> bool:
    return os.path.exists(REF_GRID_SO)


def cart_recon(sx, sy, res_freq, lines, slices, rx, pools, echoes=1, epi_etl=0, zf=None, readout_first=False):
    """Complex images [N0][N1][N2][Rx][E] (E = echoes; 1 for EPI)."""
    rows = res_freq * (epi_etl if epi_etl else echoes)
    shape = (rows, lines, slices, rx, pools)
    S5 = (np.asarray(sx, np.float64).reshape(shape, order="F") +
          1j * np.asarray(sy, np.float64).reshape(shape, order="F"))
    SX = S5[..., 0].copy()
    for p in range(1, pools):  # sum(SX, 5)
        SX += S5[..., p]
    if epi_etl:
        S = np.zeros((res_freq, epi_etl * lines, slices, rx), complex)
        for e in range(epi_etl):
            blk = SX[e * res_freq:(e + 1) * res_freq]
            if e % 2 == 1:  # the train's even (1-based) echoes are read backwards: row flipping
                blk = blk[::-1]
            S[:, e * lines:(e + 1) * lines] = blk
        vols = [S]
        L = epi_etl * lines
    else:
        vols = [SX[e * res_freq:(e + 1) * res_freq] for e in range(echoes)]
        L = lines
    F = res_freq - 1
    out = []
    for S in vols:
        S = S[:-1]  # drop the most positive kx point
        if zf is not None:
            zx, zy, zz = zf
            S2 = np.zeros((zx, zy, zz * slices, rx), complex)
            ox, oy, oz = zx // 2 - F // 2, zy // 2 - L // 2, zz * (slices // 2) - slices // 2
            S2[ox:ox + F, oy:oy + L, oz:oz + slices] = S
            S = S2
        S = S.transpose(1, 0, 2, 3)
        if readout_first:
            S = S.transpose(1, 0, 2, 3)
        img = np.stack([np.fft.fftshift(np.fft.ifftn(np.fft.fftshift(S[..., i]))) for i in range(rx)], -1)
        out.append(img)
    return np.stack(out, -1)


def grid2d_port(kx, ky, sx, sy, dcf, kernel, grid_size, half_width):
    """The reference gridding loop (sample order, FP64); [G][G] column-major
    flattened like the mex output (index ix * G + iy)."""
    G = int(grid_size)
    width = half_width / (G - 1)
    center = (G - 1) / 2
    kernel = np.asarray(kernel, np.float64).ravel()
    nk = kernel.size
    gx = np.zeros(G * G)
    gy = np.zeros(G * G)
    for x, y, a, b, d in zip(np.ravel(kx), np.ravel(ky), np.ravel(sx), np.ravel(sy), np.ravel(dcf)):
        kxmin, kxmax = max(x - width, -0.5), min(x + width, 0.5)
        kymin, kymax = max(y - width, -0.5), min(y + width, 0.5)
        for ix in range(int((kxmin + 0.5) * (G - 1)), int((kxmax + 0.5) * (G - 1)) + 1):
            dkx = (ix - center) / (G - 1) - x
            for iy in range(int((kymin + 0.5) * (G - 1)), int((kymax + 0.5) * (G - 1)) + 1):
                dky = (iy - center) / (G - 1) - y
                dk = np.sqrt(dkx * dkx + dky * dky)
                if dk <= width:
                    fi = (dk / width) * (nk - 1)
                    ki = int(fi)
                    fr = fi - ki
                    k1 = kernel[ki + 1] if ki + 1 < nk else kernel[nk - 1]
                    kv = kernel[ki] * (1 - fr) + k1 * fr
                    gx[ix * G + iy] += kv * a * d
                    gy[ix * G + iy] += kv * b * d
    return gx, gy


def run_ref_grid(kx, ky, sx, sy, dcf, kernel, grid_size, half_width):
    """The reference DoGridding mex through the mex stand-in."""
    from mrilab_gb300 import mexsim

    ms = mexsim.MexSession()
    a, b = ms.call_args(REF_GRID_SO, [np.asarray(v, np.float64) for v in (kx, ky, sx, sy, dcf, kernel)] +
                        [np.float64(grid_size), np.float64(half_width)], 2)
    return a.ravel(order="F"), b.ravel(order="F")
