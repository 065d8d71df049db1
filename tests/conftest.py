import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        manifest = json.load(f)
    arrays = np.load(os.path.join(GOLDEN, "cases.npz"))
    return manifest, arrays


def bits_equal(a, b):
    """Bitwise equality of two float arrays, treating any NaN as equal to any NaN."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    an, bn = np.isnan(a), np.isnan(b)
    if not np.array_equal(an, bn):
        return False
    ia = a.view(np.uint64 if a.dtype == np.float64 else np.uint32)
    ib = b.view(np.uint64 if b.dtype == np.float64 else np.uint32)
    return bool(np.all((ia == ib) | an))


def first_diff(a, b):
    a, b = np.asarray(a), np.asarray(b)
    bad = ~((a == b) | (np.isnan(a) & np.isnan(b)) | ((a == 0) & (b == 0) & (np.signbit(a) == np.signbit(b))))
    idx = np.argwhere(bad)
    if idx.size == 0:
        return "no value difference (sign of zero or NaN payload only)"
    i = tuple(idx[0])
    return f"{idx.shape[0]} differing points, first at {i}: {a[i]!r} vs {b[i]!r}"
