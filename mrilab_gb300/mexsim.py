"""A MATLAB global-workspace stand-in for calling MRiLab-style mex engines.

MRiLab's scan engines take no arguments: they read and mutate the MATLAB
globals ``VObj, VMag, VCoi, VCtl, VSeq, VVar, VSig`` in place
(``Lib/src/engine/CPUEngine/DoScanAtCPU.cpp:118-210``,
``Lib/src/engine/GPUEngine/DoScanAtGPU.cu:124-214``) and call back into
MATLAB with ``mexEvalString("DoExtPlugin")`` / ``"DoGPUFetch"``.

``MexSession`` drives the C stand-in ``libfakemex.so`` (``mex/fakemex.c``):
it turns dicts of numpy arrays into MATLAB structs (column-major, with the
dtypes fixed by ``Src/Main/DoDataTypeConv.m:19-138``), runs an engine's
``mexFunction`` and hands back numpy views of the mutated fields.
"""
from __future__ import annotations

import ctypes
import os
from typing import Callable, Dict, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
FAKEMEX_SO = os.path.join(_HERE, "mex", "libfakemex.so")

_CLASS = {np.dtype(np.float64): 6, np.dtype(np.float32): 7, np.dtype(np.int32): 12}
_DTYPE = {6: np.float64, 7: np.float32, 12: np.int32}

_EVAL_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_char_p)
_MEX_FN = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p)


def _lib() -> ctypes.CDLL:
    if not os.path.exists(FAKEMEX_SO):
        raise RuntimeError(f"{FAKEMEX_SO} is missing: run __graft_entry__.build() first")
    lib = ctypes.CDLL(FAKEMEX_SO, mode=ctypes.RTLD_GLOBAL)
    lib.fm_new_numeric.restype = ctypes.c_void_p
    lib.fm_new_numeric.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.fm_new_struct.restype = ctypes.c_void_p
    lib.fm_set_field.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
    lib.fm_set_global.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    lib.fm_data.restype = ctypes.c_void_p
    lib.fm_data.argtypes = [ctypes.c_void_p]
    lib.mexGetVariablePtr.restype = ctypes.c_void_p
    lib.mexGetVariablePtr.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    lib.mxGetField.restype = ctypes.c_void_p
    lib.mxGetField.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p]
    lib.mxGetNumberOfDimensions.restype = ctypes.c_int
    lib.mxGetNumberOfDimensions.argtypes = [ctypes.c_void_p]
    lib.mxGetDimensions.restype = ctypes.POINTER(ctypes.c_int)
    lib.mxGetDimensions.argtypes = [ctypes.c_void_p]
    lib.fm_set_eval_handler.argtypes = [_EVAL_FN]
    lib.fm_call.argtypes = [ctypes.c_void_p]
    lib.fm_call.restype = ctypes.c_int
    lib.fm_last_error.restype = ctypes.c_char_p
    lib.fm_set_verbose.argtypes = [ctypes.c_int]
    lib.fm_call_args.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_void_p)]
    lib.fm_call_args.restype = ctypes.c_int
    lib.fm_free_array.argtypes = [ctypes.c_void_p]
    return lib


class MexError(RuntimeError):
    """Raised when an engine called mexErrMsgTxt."""


class MexSession:
    """One MATLAB-like global workspace shared by every engine loaded."""

    _shared_lib: Optional[ctypes.CDLL] = None

    def __init__(self, verbose: bool = False):
        if MexSession._shared_lib is None:
            MexSession._shared_lib = _lib()
        self.lib = MexSession._shared_lib
        self.lib.fm_clear_globals()
        self.lib.fm_set_verbose(1 if verbose else 0)
        self._engines: Dict[str, ctypes.CDLL] = {}
        self._eval_cb = None
        self.eval_handler: Optional[Callable[[str], int]] = None
        self._install_eval()

    # -- globals -----------------------------------------------------------
    def _numeric(self, arr: np.ndarray) -> int:
        arr = np.asarray(arr)
        if arr.dtype not in _CLASS:
            raise TypeError(f"unsupported dtype {arr.dtype}")
        shape = arr.shape if arr.ndim >= 1 else (1,)
        if len(shape) == 1:
            shape = (1, shape[0])  # MATLAB row vector
        dims = (ctypes.c_int * len(shape))(*shape)
        ptr = self.lib.fm_new_numeric(_CLASS[arr.dtype], len(shape), dims)
        data = self.lib.fm_data(ptr)
        flat = np.asfortranarray(arr.reshape(shape)).ravel(order="F")
        ctypes.memmove(data, flat.ctypes.data, flat.nbytes)
        return ptr

    def set_global(self, name: str, fields: Dict[str, np.ndarray]) -> None:
        st = self.lib.fm_new_struct()
        for key, val in fields.items():
            self.lib.fm_set_field(st, key.encode(), self._numeric(val))
        self.lib.fm_set_global(name.encode(), st)

    def set_field(self, name: str, field: str, value: np.ndarray) -> None:
        st = self.lib.mexGetVariablePtr(b"global", name.encode())
        if not st:
            raise KeyError(name)
        self.lib.fm_set_field(st, field.encode(), self._numeric(value))

    def get(self, name: str, field: str) -> np.ndarray:
        """Numpy view (column-major, writable) of a global struct field."""
        st = self.lib.mexGetVariablePtr(b"global", name.encode())
        if not st:
            raise KeyError(name)
        arr = self.lib.mxGetField(st, 0, field.encode())
        if not arr:
            raise KeyError(f"{name}.{field}")
        nd = self.lib.mxGetNumberOfDimensions(arr)
        dp = self.lib.mxGetDimensions(arr)
        dims = tuple(dp[i] for i in range(nd))
        # class id lives in the first int of the C struct
        cls = ctypes.cast(arr, ctypes.POINTER(ctypes.c_int))[0]
        dt = np.dtype(_DTYPE[cls])
        n = int(np.prod(dims))
        buf = (ctypes.c_char * (n * dt.itemsize)).from_address(self.lib.fm_data(arr))
        return np.frombuffer(buf, dtype=dt, count=n).reshape(dims, order="F")

    # -- callbacks ---------------------------------------------------------
    def _install_eval(self) -> None:
        def _handler(cmd: bytes) -> int:
            if self.eval_handler is None:
                return 0
            try:
                return int(self.eval_handler(cmd.decode()))
            except Exception:  # an exception in a plugin is an Ext error
                return 1

        self._eval_cb = _EVAL_FN(_handler)
        self.lib.fm_set_eval_handler(self._eval_cb)

    # -- engines -----------------------------------------------------------
    def load(self, so_path: str) -> ctypes.CDLL:
        if so_path not in self._engines:
            if not os.path.exists(so_path):
                raise RuntimeError(f"engine library {so_path} is missing")
            self._engines[so_path] = ctypes.CDLL(so_path, mode=ctypes.RTLD_LOCAL)
        return self._engines[so_path]

    def _array(self, arr) -> np.ndarray:
        nd = self.lib.mxGetNumberOfDimensions(arr)
        dp = self.lib.mxGetDimensions(arr)
        dims = tuple(dp[i] for i in range(nd))
        cls = ctypes.cast(arr, ctypes.POINTER(ctypes.c_int))[0]
        dt = np.dtype(_DTYPE[cls])
        n = int(np.prod(dims))
        buf = (ctypes.c_char * (n * dt.itemsize)).from_address(self.lib.fm_data(arr))
        return np.frombuffer(buf, dtype=dt, count=n).reshape(dims, order="F").copy()

    def call_args(self, so_path: str, args, nlhs: int):
        """Run a mexFunction that takes its inputs as arguments (prhs) and
        returns nlhs outputs (plhs), as MATLAB's [a, b] = f(x, y, ...)."""
        eng = self.load(so_path)
        fn = ctypes.cast(eng.mexFunction, ctypes.c_void_p)
        prhs = (ctypes.c_void_p * max(1, len(args)))(*[self._numeric(np.asarray(a)) for a in args])
        plhs = (ctypes.c_void_p * max(1, nlhs))()
        rc = self.lib.fm_call_args(fn, nlhs, plhs, len(args), prhs)
        try:
            if rc != 0:
                raise MexError(self.lib.fm_last_error().decode())
            return [self._array(plhs[i]) for i in range(nlhs)]
        finally:
            for i in range(len(args)):
                self.lib.fm_free_array(prhs[i])
            for i in range(nlhs):
                if plhs[i]:
                    self.lib.fm_free_array(plhs[i])

    def call(self, so_path: str) -> None:
        """Run an engine's mexFunction against the current globals."""
        eng = self.load(so_path)
        fn = ctypes.cast(eng.mexFunction, ctypes.c_void_p)
        rc = self.lib.fm_call(fn)
        if rc != 0:
            raise MexError(self.lib.fm_last_error().decode())
