import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")
GOLDEN_NEXT = os.path.join(ROOT, "tests", "golden", "golden_next.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 host)")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def golden_next():
    with np.load(GOLDEN_NEXT) as z:
        return {k: z[k] for k in z.files}


def bits_equal(a, b) -> bool:
    """Bit-for-bit equality; NaNs compare by position only (GPU adds return a
    canonical NaN where x86 propagates the payload)."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    if a.dtype.kind == "f":
        na, nb = np.isnan(a), np.isnan(b)
        if not np.array_equal(na, nb):
            return False
        ua = a.view(np.uint32 if a.itemsize == 4 else np.uint64)[~na]
        ub = b.view(np.uint32 if b.itemsize == 4 else np.uint64)[~nb]
        return np.array_equal(ua, ub)
    return np.array_equal(a, b)


def first_mismatch(a, b) -> str:
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return f"shape {a.shape} != {b.shape}"
    bad = np.argwhere(~((a == b) | (np.isnan(a) & np.isnan(b))))
    if len(bad) == 0:
        bad = np.argwhere(np.signbit(a) != np.signbit(b))
    if len(bad) == 0:
        return "equal"
    i = tuple(bad[0])
    return f"{len(bad)} mismatches; first at {i}: {a[i]!r} vs {b[i]!r}"


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle

    oracle.build()
    return oracle
