"""Shared test setup: the `gpu` marker, import paths and fixture loading."""
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "vectorized-particle-in-cell-code-with-graphics_gb300")
for p in (PKG, os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases(mode=None):
    out = []
    for f in sorted(os.listdir(GOLDEN)):
        if f.endswith(".npz"):
            with np.load(os.path.join(GOLDEN, f)) as z:
                if "mode" not in z.files:   # a table, not a run or field case
                    continue
                if mode is None or str(z["mode"]) == mode:
                    out.append(f[:-4])
    return out


def load_golden(name):
    import picgb
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        rec = {k: z[k] for k in z.files}
    kw = json.loads(str(rec["params"]))
    rec["kw"] = kw
    rec["p"] = picgb.make_params(**kw)
    return rec


@pytest.fixture(scope="session")
def lib():
    """libpicgb.so, built in-tree if missing (no GPU needed to load it)."""
    import build_lib
    import picgb
    build_lib.build()
    return picgb.load_library()
