"""Build the native parts of mrilab_gb300 in-tree.

* ``libmrl_scan.so``: the C-ABI scan engine (``include/mrl_scan.h``), SAR
  engine (``include/mrl_sar.h``), reconstruction (``include/mrl_recon.h``)
  and sequence compiler (``include/mrl_seq.h``), CUDA for sm_103a only;
  translation units compile in parallel.
* ``mex/libfakemex.so``: the MATLAB stand-in used to drive the mex layer
  without MATLAB.
* ``mex/Do*ScanAtGPU.so``, ``mex/DoCalSARAtGPU.so``, ``mex/DoGridding.so``,
  ``mex/DoCartReconGPU.so``: the mex wrappers with the reference engine
  names (the SAR one named after the reference's DoCalSARAtCPU, for the
  GPU; DoCartReconGPU new, for the transform of DoCartRecon.m),
  linked against the stand-in (inside MATLAB they are built with ``mex``
  against MATLAB's own headers instead: ``mex -DMRL_WRAP_MODEL=<model>
  csrc/mex_wrappers.cpp -lmrl_scan``).

Nothing is built for the host's GPU or any other architecture:
``-gencode arch=compute_103a,code=sm_103a``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
MEX = os.path.join(HERE, "mex")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmrl_scan.so")
PEAKS = os.path.join(HERE, "libmrl_peaks.so")
FAKEMEX = os.path.join(MEX, "libfakemex.so")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
WRAPPERS = {
    "DoScanAtGPU": "MRL_MODEL_NORMAL",
    "DoMEScanAtGPU": "MRL_MODEL_ME",
    "DoMTScanAtGPU": "MRL_MODEL_MT",
    "DoCESTScanAtGPU": "MRL_MODEL_CEST",
    "DoGMScanAtGPU": "MRL_MODEL_GM",
}
# translation units of libmrl_scan.so and their extra flags; the reference-
# order integrators must not contract a*b+c into fused multiply-adds
UNITS = {
    "engine.cu": [],
    "scan_ref_normal.cu": ["-fmad=false"],
    "scan_ref_exch.cu": ["-fmad=false"],
    "scan_ref_mt.cu": ["-fmad=false"],
    "scan_ref_cest.cu": ["-fmad=false"],
    "scan_fast_normal.cu": [],
    "scan_fast_exch.cu": [],
    "scan_fast_mt.cu": [],
    "scan_fast_cest.cu": [],
    "adjoint.cu": [],
    "scan_fast_exact.cu": [],
    "scan_fast_exact_bound.cu": [],
    "scan_fast_tc.cu": [],
    "sar.cu": [],
    "recon.cu": [],
    "decode.cpp": None,  # host C++
    "seqc.cpp": None,  # host C++
}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", f) for f in ("mrl_scan.h", "mrl_sar.h", "mrl_recon.h", "mrl_seq.h")]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, jobs: int = 0) -> None:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    cmds = []
    objs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OBJ, unit + ".o")
        objs.append(obj)
        if not _stale(obj, [src] + hdrs):
            continue
        if extra is None:
            cmds.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", f"-I{_cuda_home()}/include", "-c", src, "-o", obj])
        else:
            cmds.append([nvcc, "-std=c++17", "-O3", *GENCODE, "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas",
                         "-warn-spills" if verbose else "-O3", *extra, "-c", src, "-o", obj])
    jobs = jobs or min(len(cmds), os.cpu_count() or 4) or 1
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for out in ex.map(_run, cmds):
            if verbose and out:
                print(out)
    if _stale(LIB, objs):
        _run([nvcc, "-shared", *GENCODE, "-o", LIB, *objs, "-lcudart", "-lcufft", "-lpthread"])
    peaks_src = os.path.join(CSRC, "peaks.cu")
    if _stale(PEAKS, [peaks_src]):
        _run([nvcc, "-std=c++17", "-O3", *GENCODE, "-Xcompiler", "-fPIC", "-shared", peaks_src, "-o", PEAKS])
    # MATLAB stand-in and the mex wrappers
    fm_src = os.path.join(MEX, "fakemex.c")
    if _stale(FAKEMEX, [fm_src, os.path.join(MEX, "mex.h"), os.path.join(MEX, "matrix.h")]):
        _run(["gcc", "-O2", "-fPIC", "-shared", f"-I{MEX}", fm_src, "-o", FAKEMEX])
    wsrc = os.path.join(CSRC, "mex_wrappers.cpp")
    sar_src = os.path.join(CSRC, "sar_mex.cpp")
    sar_out = os.path.join(MEX, "DoCalSARAtGPU.so")
    if _stale(sar_out, [sar_src, LIB, FAKEMEX] + hdrs):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-I{MEX}", sar_src, "-o", sar_out, f"-L{HERE}",
              "-lmrl_scan", f"-L{MEX}", "-lfakemex", "-Wl,-rpath,$ORIGIN/..", "-Wl,-rpath,$ORIGIN"])
    rsrc = os.path.join(CSRC, "recon_mex.cpp")
    for name, flag in (("DoGridding", "MRL_WRAP_GRID"), ("DoCartReconGPU", "MRL_WRAP_CART")):
        out = os.path.join(MEX, name + ".so")
        if _stale(out, [rsrc, LIB, FAKEMEX] + hdrs):
            _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-D{flag}", f"-I{MEX}", rsrc, "-o", out, f"-L{HERE}",
                  "-lmrl_scan", f"-L{MEX}", "-lfakemex", "-Wl,-rpath,$ORIGIN/..", "-Wl,-rpath,$ORIGIN"])
    for name, model in WRAPPERS.items():
        out = os.path.join(MEX, name + ".so")
        if _stale(out, [wsrc, LIB, FAKEMEX] + hdrs):
            _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", f"-DMRL_WRAP_MODEL={model}", f"-I{MEX}", wsrc,
                  "-o", out, f"-L{HERE}", "-lmrl_scan", f"-L{MEX}", "-lfakemex",
                  "-Wl,-rpath,$ORIGIN/..", "-Wl,-rpath,$ORIGIN"])


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print("built", LIB)
