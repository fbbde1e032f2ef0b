"""Regenerate the golden fixtures from the reference engine itself.

Runs the reference CPU engine (``Lib/src/engine/CPUEngine/DoScanAtCPU.cpp``,
compiled unmodified against the project's mex/IPP stand-ins into
``oracle/_ref`` -- available only where the reference tree is mounted) on
seeded single-pool scans and stores its outputs, together with the all-FP64
oracle's outputs on the same inputs, as small ``.npz`` files.  The scans are
rebuilt from their seeds by ``mrilab_gb300.phantoms`` at test time.

    MRILAB_REFERENCE_ROOT=<MRiLab tree> python tests/golden/make_golden.py [name ...]   # all, or the named ones
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mrilab_gb300 import phantoms  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

MULTIPOOL = {
    # name: small_multipool kwargs; the reference's own kernels (compiled as
    # host C, oracle/_ref/libmrl_refkern.so) produce the golden signal
    "mp_me_p2_s2_c2": dict(model="me", seed=3, pools=2, spins=2, coils=2, seq="gre"),
    "mp_me_p3_s1_c1": dict(model="me", seed=3, pools=3, spins=1, coils=1, seq="gre"),
    "mp_gm_p3_s2_c2": dict(model="gm", seed=3, pools=3, spins=2, coils=2, seq="sat"),
    "mp_mt_p2_s2_c2": dict(model="mt", seed=3, pools=2, spins=2, coils=2, seq="sat"),
    "mp_cest_p4_s2_c2": dict(model="cest", seed=3, pools=4, spins=2, coils=2, seq="sat"),
    "mp_cest_p5_s1_c2": dict(model="cest", seed=3, pools=5, spins=1, coils=2, seq="sat"),
}

# the MT + exchange EPI's tissue and sequence (general model with a bound
# pool, 8 ms MT pulse, single-shot EPI), small; reference kernels as above
MT_EPI = {
    "mt_epi_gm_p3_s2_c4": dict(seed=7, nx=6, ny=6, nz=2, spins=2, n_coils=4, n_read=8, n_pe=8),
}

# several transmit coils (B1 the complex sum over the coils): the
# reference CPU engine's multi-Tx branch (BlochKernel.h:62-110)
MULTI_TX = {
    "gre_tx2_n8_seed1": dict(seed=1, n=8, n_tr=2, tx_coils=2),
    "gre_tx3_n8_seed2": dict(seed=2, n=8, n_tr=2, tx_coils=3),
}

HISTORY = {
    # RunMode 1: the reference CPU engine's per-time-point state history
    "history_gre2d_n4_tr2_seed4": dict(seed=4, n=4, n_tr=2),
}

# the benchmark's two-pool multi-echo GRE at its full sequence length (256
# TRs, 220,416 steps) on a voxel subset spread over the field of view; the
# signal is stored at every SAMPLE_STRIDE-th sample of each (pool, coil)
# (the whole signal is 50 MB), with the relative L2 distances over the whole
# signal recorded beside it
FULL_LENGTH = {
    "config2_full_length_subset": dict(seed=0, step=8, offset=4),
}
SAMPLE_STRIDE = 127

# local SAR (the reference SAR engine DoCalSARAtCPU, compiled from its
# source): phantoms.sar_case kwargs
SAR = {
    "sar_tx1_n6_seed2": dict(seed=2, n=6, nz=1, tx_coils=1, n_tr=3),
    "sar_tx2_n8_seed1": dict(seed=1, n=8, nz=2, tx_coils=2, n_tr=2),
    "sar_tx3_n6_seed3": dict(seed=3, n=6, nz=3, tx_coils=3, n_tr=2, sample_fracs=(0.1, 0.45, 0.7)),
}

# gridding (the reference DoGridding mex, compiled from its source): inputs
# drawn from the seed by grid_inputs below
GRID = {
    "grid2d_n400_g32_seed0": dict(seed=0, n=400, grid=32, half_width=2.0, nk=101),
    "grid2d_n900_g48_seed1": dict(seed=1, n=900, grid=48, half_width=3.0, nk=201),
}


def grid_inputs(seed, n, grid, half_width, nk):
    """Seeded gridding inputs: k-space locations in [-0.5, 0.5], complex
    samples, density weights and a Gaussian-like kernel table."""
    rng = np.random.default_rng(seed)
    kx, ky = rng.uniform(-0.5, 0.5, n), rng.uniform(-0.5, 0.5, n)
    sx, sy = rng.normal(size=n), rng.normal(size=n)
    dcf = rng.uniform(0.2, 1.5, n)
    ker = np.exp(-3.0 * np.linspace(0.0, 1.0, nk) ** 2)
    return kx, ky, sx, sy, dcf, ker, grid, half_width


CASES = {
    # name: (builder kwargs)
    "gre2d_n16_tr4_seed1": dict(seed=1, n=16, n_tr=4),
    "gre2d_n32_tr8_seed2": dict(seed=2, n=32, n_tr=8),
    "gre2d_n64_full_seed0": dict(seed=0, n=64),
}


def main(only=()):
    def wanted(name):
        return not only or name in only

    oracle.build()
    if not oracle.ref_available():
        raise SystemExit("the reference engine is not built (needs the reference tree)")
    for name, kw in CASES.items():
        if not wanted(name):
            continue
        sc = phantoms.config1_gre(**kw)
        ref = oracle.run_ref_cpu(sc, threads=1)
        f64 = oracle.run_port(sc, "f64")
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            builder=np.array("config1_gre"), kwargs=np.array(repr(kw)),
            ref_Sx=ref["Sx"], ref_Sy=ref["Sy"], ref_Kx=ref["Kx"], ref_Ky=ref["Ky"], ref_Kz=ref["Kz"],
            ref_Mz=ref["Mz"], ref_Mx=ref["Mx"], ref_My=ref["My"],
            f64_Sx=f64["Sx"], f64_Sy=f64["Sy"],
        )
        s_ref = ref["Sx"] + 1j * ref["Sy"]
        s64 = f64["Sx"] + 1j * f64["Sy"]
        print(name, "reference vs FP64 oracle: %.3e" % (np.linalg.norm(s_ref - s64) / np.linalg.norm(s64)))
    for name, kw in MULTI_TX.items():
        if not wanted(name):
            continue
        sc = phantoms.multi_tx_gre(**kw)
        ref = oracle.run_ref_cpu(sc, threads=1)
        f64 = oracle.run_port(sc, "f64")
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            builder=np.array("multi_tx_gre"), kwargs=np.array(repr(kw)),
            ref_Sx=ref["Sx"], ref_Sy=ref["Sy"], ref_Kx=ref["Kx"], ref_Ky=ref["Ky"], ref_Kz=ref["Kz"],
            ref_Mz=ref["Mz"], ref_Mx=ref["Mx"], ref_My=ref["My"], f64_Sx=f64["Sx"], f64_Sy=f64["Sy"],
        )
        s_ref = ref["Sx"] + 1j * ref["Sy"]
        s64 = f64["Sx"] + 1j * f64["Sy"]
        print(name, "reference vs FP64 oracle: %.3e" % (np.linalg.norm(s_ref - s64) / np.linalg.norm(s64)))
    for name, kw in HISTORY.items():
        if not wanted(name):
            continue
        sc = phantoms.with_history(phantoms.config1_gre(**kw))
        ref = oracle.run_ref_cpu(sc, threads=1)
        f64 = oracle.run_port(sc, "f64")
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            builder=np.array("config1_gre"), kwargs=np.array(repr(kw)), history=np.array(True),
            ref_Sx=ref["Sx"], ref_Sy=ref["Sy"], ref_Mxs=ref["Mxs"], ref_Mys=ref["Mys"], ref_Mzs=ref["Mzs"],
            ref_Muts=ref["Muts"], f64_Mxs=f64["Mxs"], f64_Mys=f64["Mys"], f64_Mzs=f64["Mzs"],
        )
        print(name, "history: reference vs FP64 oracle max abs %.3e" % np.abs(ref["Mxs"] - f64["Mxs"]).max())
    for name, kw in FULL_LENGTH.items():
        if not wanted(name):
            continue
        import time

        sc = phantoms.config2_subset(**kw)
        P, C, A = int(sc.VObj["TypeNum"]), int(sc.VCoi["RxCoilNum"]), sc.signal_num
        keep = np.arange(0, A, SAMPLE_STRIDE)
        runs, secs = {}, {}
        for tag, fn in (("ref", oracle.run_ref_kernel), ("f64", lambda s: oracle.run_port(s, "f64")),
                        ("f32", lambda s: oracle.run_port(s, "f32"))):
            t0 = time.time()
            o = fn(sc)
            secs[tag] = time.time() - t0
            runs[tag] = (o["Sx"] + 1j * o["Sy"]).reshape(P, C, A)
        rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            builder=np.array("config2_subset"), kwargs=np.array(repr(kw)), sample_index=keep,
            ref_S=runs["ref"][..., keep].astype(np.complex64), f64_S=runs["f64"][..., keep].astype(np.complex64),
            full_ref_vs_f64=np.float64(rl(runs["ref"], runs["f64"])),
            full_f32_vs_f64=np.float64(rl(runs["f32"], runs["f64"])),
        )
        print(name, "reference kernels vs FP64 oracle: %.3e (sampled %.3e); FP32 port vs FP64 %.3e; seconds %s" % (
            rl(runs["ref"], runs["f64"]), rl(runs["ref"][..., keep], runs["f64"][..., keep]),
            rl(runs["f32"], runs["f64"]), secs))
    from oracle import recon as orc
    from oracle import sar as osar

    for name, kw in GRID.items():
        if not wanted(name):
            continue
        gx, gy = orc.run_ref_grid(*grid_inputs(**kw))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), builder=np.array("grid_inputs"),
                            kwargs=np.array(repr(kw)), ref_gx=gx, ref_gy=gy)
        print(name, "gridded points:", int(np.count_nonzero(gx)))

    for name, kw in SAR.items():
        if not wanted(name):
            continue
        sc = phantoms.sar_case(**kw)
        ref = osar.run_ref_sar(sc)
        f64 = osar.run_sar_port(sc, "f64")
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            builder=np.array("sar_case"), kwargs=np.array(repr(kw)),
            ref_SAR=ref["SAR"].astype(np.float32), ref_SARacc=ref["SARacc"].astype(np.float32),
            ref_Muts=ref["Muts"], ref_tRealSample=ref["tRealSample"],
            ref_cursor=np.array([ref["SARi"], ref["utsi"], ref["rfi"], ref["TRCount"]]),
            f64_SAR=f64["SAR"], f64_SARacc=f64["SARacc"],
        )
        print(name, "reference SAR engine vs FP64 oracle: %.3e" % (
            np.linalg.norm(ref["SAR"] - f64["SAR"]) / np.linalg.norm(f64["SAR"])))
    multi = [(n, "small_multipool", kw) for n, kw in MULTIPOOL.items()]
    multi += [(n, "config5_mt_epi", kw) for n, kw in MT_EPI.items()]
    for name, builder, kw in multi:
        if not wanted(name):
            continue
        sc = getattr(phantoms, builder)(**kw)
        ref = oracle.run_ref_kernel(sc)
        f64 = oracle.run_port(sc, "f64")
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            builder=np.array(builder), kwargs=np.array(repr(kw)),
            ref_Sx=ref["Sx"], ref_Sy=ref["Sy"], ref_Mz=ref["Mz"], ref_Mx=ref["Mx"], ref_My=ref["My"],
            f64_Sx=f64["Sx"], f64_Sy=f64["Sy"],
        )
        s_ref = ref["Sx"] + 1j * ref["Sy"]
        s64 = f64["Sx"] + 1j * f64["Sy"]
        print(name, "reference kernels vs FP64 oracle: %.3e" % (np.linalg.norm(s_ref - s64) / np.linalg.norm(s64)))


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
