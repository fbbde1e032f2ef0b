import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the engine and the CPU oracle in-tree (no-op when up to date);
    every session builds first: the phantoms' sequences come from the native
    sequence compiler in libmrl_scan.so."""
    import oracle
    from mrilab_gb300 import build

    build.build()
    oracle.build()
    return True


def rel_l2(a, b):
    import numpy as np

    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def signal(out):
    return out["Sx"] + 1j * out["Sy"]


def load_golden(name):
    import ast

    import numpy as np

    from mrilab_gb300 import phantoms

    path = os.path.join(ROOT, "tests", "golden", name + ".npz")
    z = np.load(path, allow_pickle=False)
    builder = str(z["builder"])
    kwargs = ast.literal_eval(str(z["kwargs"]))
    sc = getattr(phantoms, builder)(**kwargs)
    if "history" in z.files and bool(z["history"]):
        sc = phantoms.with_history(sc)
    return sc, {k: z[k] for k in z.files}
