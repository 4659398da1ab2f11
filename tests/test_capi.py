"""The C ABI library loads and exports every symbol its header declares; its
argument checks return the documented status codes.  No GPU work is issued:
every call here fails validation before touching the device."""

import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"\b((?:adrt_gb300|adrtnet)_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from adrt_gb300 import _lib

    if not os.path.exists(_lib.LIB_PATH):
        from adrt_gb300 import build

        build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = _declared()
    assert "adrt_gb300_adrt" in names and "adrt_gb300_bdrt" in names
    assert len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    from adrt_gb300 import _lib

    assert set(_declared()) <= set(_lib.SIGNATURES)


def test_status_strings(lib):
    from adrt_gb300 import _lib

    for code in range(9):
        s = _lib.status_string(code)
        assert s and s != "unknown status"
    assert _lib.status_string(99) == "unknown status"


def test_num_iters(lib):
    for n, want in [(0, 0), (1, 0), (2, 1), (3, 2), (1024, 10), (2**40 + 1, 41)]:
        assert lib.adrt_gb300_num_iters(n) == want


def test_validation_codes(lib):
    from adrt_gb300 import _lib

    fake = ctypes.c_void_p(16)
    assert lib.adrt_gb300_adrt(None, fake, 1, 16, 0, None, 0, None) == _lib.ERR_NULL
    assert lib.adrt_gb300_adrt(fake, fake, 1, 12, 0, None, 0, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_adrt(fake, fake, 0, 16, 0, None, 0, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_adrt(fake, fake, 1, 16, 7, None, 0, None) == _lib.ERR_DTYPE
    assert lib.adrt_gb300_adrt(fake, fake, 1, 2**30, 0, None, 0, None) == _lib.ERR_TOO_LARGE
    # n = 1024 needs an intermediate buffer: refused without one.
    assert lib.adrt_gb300_adrt(fake, fake, 1, 1024, 0, None, 0, None) == _lib.ERR_WORKSPACE
    assert lib.adrt_gb300_adrt_step(fake, fake, 1, 16, 4, 0, None) == _lib.ERR_STEP
    assert lib.adrt_gb300_adrt_step(fake, fake, 1, 16, -1, 0, None) == _lib.ERR_STEP
    assert lib.adrt_gb300_bdrt_step(fake, fake, 1, 16, 4, 0, None) == _lib.ERR_STEP
    assert lib.adrt_gb300_bdrt(fake, fake, 1, 1024, 1, None, 0, None) == _lib.ERR_WORKSPACE
    assert lib.adrt_gb300_iadrt(fake, fake, 1, 64, 0, None, 0, None) == _lib.ERR_WORKSPACE
    assert lib.adrt_gb300_adjoint(fake, fake, 1, 64, 0, None, 0, None) == _lib.ERR_WORKSPACE
    assert lib.adrt_gb300_fmg_restriction(fake, fake, 1, 1, 0, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_fmg_highpass(fake, fake, 1, 1, 5, 0, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_fmg_prolongation(fake, fake, 1, 0, 5, 0, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_adrt_init(fake, fake, 1, 16, 3, None) == _lib.ERR_DTYPE
    assert lib.adrt_gb300_elementwise(2, fake, fake, fake, 4, 0, None) == _lib.ERR_SHAPE
    assert lib.adrt_gb300_sumsq(fake, 4, 0, None, fake, None) == _lib.ERR_NULL


def test_workspace_sizes(lib):
    from adrt_gb300 import _lib

    # One pass (n <= 32) needs no intermediate.
    assert _lib.workspace_size(_lib.OP_ADRT, 4, 32, _lib.F32) == 0
    # Two passes: one intermediate per image in the chunk; at n = 1024 the
    # fast float32 path keeps the 1056 offsets (n + 31 rounded up to 8) where a row
    # group can be non-zero after five stages.
    per = 4 * 32 * 32 * 1056 * 4
    got = _lib.workspace_size(_lib.OP_ADRT, 256, 1024, _lib.F32)
    assert got > 0 and got % per == 0
    # Below 1024 the first pass leaves L-5 stages done: rows end at n + n/32 - 1
    # (rounded up to 8 floats): 528 at n = 512, 72 at n = 64.
    for n, cs in ((512, 528), (256, 264), (128, 136), (64, 72)):
        assert _lib.workspace_size(_lib.OP_ADRT, 3, n, _lib.F32) == 3 * 4 * n * cs * 4
    per64 = 4 * 512 * 1023 * 8
    got64 = _lib.workspace_size(_lib.OP_ADRT, 8, 512, _lib.F64)
    assert got64 > 0 and got64 % per64 == 0
    assert _lib.workspace_size(_lib.OP_IADRT, 2, 64, _lib.F64) == 2 * 2 * 4 * 64 * 127 * 8
    # bdrt: one buffer between its two passes; on the float32 register path
    # (128 <= n <= 1024) its rows are padded from 2n - 1 to 2n floats.
    for n in (128, 256, 512, 1024):
        assert _lib.workspace_size(_lib.OP_BDRT, 3, n, _lib.F32) == 3 * 4 * n * (2 * n) * 4
    assert _lib.workspace_size(_lib.OP_BDRT, 3, 64, _lib.F32) == 3 * 4 * 64 * 127 * 4
    with pytest.raises(ValueError):
        _lib.workspace_size(_lib.OP_ADRT, 1, 12, _lib.F32)
