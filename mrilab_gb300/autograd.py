"""``torch.autograd`` bridge over the scan engine, for test harnesses and
parameter fitting, through an adjoint plan (``mrl_adjoint_plan``): the
forward pass runs the accurate integrator, which leaves a checkpoint of
every isochromat every 16 steps on the device, and the backward pass runs
the adjoint kernel from those checkpoints; both through the C ABI on the
GPU.  There is no CPU path: without the CUDA library both raise.

    sx, sy = autograd.scan(sc, T1=t1, T2=t2, Rho=rho, dB0=db0)
    loss = ((sx - tx) ** 2 + (sy - ty) ** 2).sum()
    loss.backward()          # t1.grad, t2.grad, ... (same shapes)

Any of the differentiable inputs may be left out (the scan's own values are
used and get no gradient):

* ``T1``, ``T2``, ``Rho``: ``VObj`` pool maps ``[Y, X, Z(, P)]``;
* ``dB0``: ``VMag.dB0`` ``[Y, X, Z]`` (T);
* ``K``: ``VObj.K`` (the model's exchange channels);
* ``Mz0``: ``VObj.Mz`` (the initial longitudinal magnetisation);
* ``rfAmp``, ``rfPhase``: ``VSeq.rfAmpLine`` / ``VSeq.rfPhaseLine``.

The adjoint's scope applies (free-pool models, one Tx coil, RunMode 0, no
Ext events, TypeNum <= 3).  Sx and Sy come back as float64 tensors laid out
as ``VSig.Sx`` / ``VSig.Sy``.
"""
from __future__ import annotations

from typing import Dict, Optional, Tuple

import numpy as np
import torch

from . import engine

# name -> (struct, key, adjoint output)
_PARAMS = (
    ("T1", "VObj", "T1", "T1"),
    ("T2", "VObj", "T2", "T2"),
    ("Rho", "VObj", "Rho", "Rho"),
    ("dB0", "VMag", "dB0", "dB0"),
    ("K", "VObj", "K", "K"),
    ("Mz0", "VObj", "Mz", "Mz0"),
    ("rfAmp", "VSeq", "rfAmpLine", "rf_amp_line"),
    ("rfPhase", "VSeq", "rfPhaseLine", "rf_phase_line"),
)


def _with_values(sc, values: Dict[str, torch.Tensor]):
    out = sc.copy()
    for name, struct, key, _ in _PARAMS:
        if name not in values:
            continue
        d = getattr(out, struct)
        ref = np.asarray(d[key])
        v = values[name].detach().cpu().numpy()
        if v.size != ref.size:
            raise ValueError(f"{name}: {v.size} values for {struct}.{key} of {ref.size}")
        d[key] = np.asfortranarray(v.astype(ref.dtype).reshape(ref.shape, order="F"))
    return out


class _Scan(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sc, gpu_index, names, *tensors):
        s = _with_values(sc, dict(zip(names, tensors)))
        plan = engine.AdjointPlan(s, gpu_index=gpu_index)
        plan.forward()
        out = plan.signal()
        ctx.plan, ctx.sc, ctx.names = plan, s, names
        ctx.shapes = [t.shape for t in tensors]
        ctx.dtypes = [t.dtype for t in tensors]
        return torch.from_numpy(out["Sx"].copy()), torch.from_numpy(out["Sy"].copy())

    @staticmethod
    def backward(ctx, gsx, gsy):
        zero = lambda: np.zeros(ctx.sc.signal_num * int(ctx.sc.VObj["TypeNum"]) *
                                int(ctx.sc.VCoi["RxCoilNum"]))
        gx = gsx.detach().cpu().numpy() if gsx is not None else zero()
        gy = gsy.detach().cpu().numpy() if gsy is not None else zero()
        plan = ctx.plan
        plan.backward(gx, gy)
        g = plan.gradients()
        plan.close()  # the checkpoints are released with the graph's one backward pass
        outs = []
        key_of = {name: out for name, _, _, out in _PARAMS}
        for name, shape, dtype in zip(ctx.names, ctx.shapes, ctx.dtypes):
            flat = np.asarray(g[key_of[name]], np.float64)
            # column-major engine layout -> the tensor's (row-major) shape
            arr = flat[: int(np.prod(shape))].reshape(tuple(shape), order="F")
            outs.append(torch.from_numpy(np.ascontiguousarray(arr)).to(dtype))
        return (None, None, None, *outs)


def scan(sc, gpu_index: int = 0, **params: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
    """Differentiable scan of ``sc`` (a ``phantoms.Scan``) with the given
    parameter tensors; returns (Sx, Sy)."""
    known = {p[0] for p in _PARAMS}
    for name in params:
        if name not in known:
            raise KeyError(f"{name} is not a differentiable scan input ({sorted(known)})")
    names = tuple(params)
    return _Scan.apply(sc, gpu_index, names, *[params[n] for n in names])


def parameters(sc, names=("T1", "T2", "Rho", "dB0"), dtype=torch.float64) -> Dict[str, torch.Tensor]:
    """The scan's current values of ``names`` as leaf tensors that require
    gradients (shapes as in the scan's structs)."""
    out: Dict[str, torch.Tensor] = {}
    for name, struct, key, _ in _PARAMS:
        if name in names:
            a = np.asarray(getattr(sc, struct)[key], np.float64)
            out[name] = torch.tensor(np.ascontiguousarray(a), dtype=dtype, requires_grad=True)
    return out
