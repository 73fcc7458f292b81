import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "wpk_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN, allow_pickle=False)


def golden_cases(g):
    """Yields (name, rowptr, cols, vals, x, [(kind, threshold), ...])."""
    for name in g["names"]:
        name = str(name)
        yield (name, g[f"{name}/rowptr"], g[f"{name}/cols"], g[f"{name}/vals"], g[f"{name}/x"],
               [tuple(int(v) for v in r) for r in g[f"{name}/layouts"]])


def random_csr(rng, n, maxlen, p_empty=0.0, ncols=None, wpk2_safe=True):
    """Random CSR with ragged rows (lengths < n when wpk2_safe, the reference's
    structure2::scan asserts rowsize < nrows)."""
    ncols = n if ncols is None else ncols
    hi = min(maxlen, n - 1) if wpk2_safe else maxlen
    lens = rng.integers(0, max(hi, 0) + 1, n) if n > 1 or not wpk2_safe else np.zeros(n, np.int64)
    if p_empty:
        lens[rng.random(n) < p_empty] = 0
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    cols = rng.integers(0, ncols, int(rp[-1])).astype(np.int32)
    vals = rng.standard_normal(int(rp[-1]))
    return rp, cols, vals
