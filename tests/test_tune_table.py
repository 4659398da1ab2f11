"""The autotuner's configuration table (host side only: no GPU work)."""

import pytest

from adrt_gb300 import _lib


@pytest.fixture()
def tune():
    from adrt_gb300 import tune as t

    t.reset()
    yield t
    t.reset()


def test_defaults_and_round_trip(tune):
    assert tune.get("adrt", 1024, "float32") == tune.Config()
    cfg = tune.Config(width=128, max_fused=3, chunk_mb=24, use_fast=0)
    tune.set_config("adrt", 1024, "float32", cfg)
    assert tune.get("adrt", 1024, "float32") == cfg
    # other entries untouched
    assert tune.get("adrt", 1024, "float64") == tune.Config()
    assert tune.get("bdrt", 1024, "float32") == tune.Config()
    assert tune.get("adrt", 512, "float32") == tune.Config()
    tune.reset()
    assert tune.get("adrt", 1024, "float32") == tune.Config()


def test_validation(tune):
    lib = _lib.load()
    assert lib.adrt_gb300_tune_set(0, 0, 1000, 0, 0, 0, -1) == _lib.ERR_SHAPE  # n not a power of two
    assert lib.adrt_gb300_tune_set(2, 0, 64, 0, 0, 0, -1) == _lib.ERR_SHAPE  # op without a table
    assert lib.adrt_gb300_tune_set(0, 0, 64, 192, 0, 0, -1) == _lib.ERR_SHAPE  # width
    assert lib.adrt_gb300_tune_set(0, 0, 64, 0, 6, 0, -1) == _lib.ERR_SHAPE  # max_fused
    assert lib.adrt_gb300_tune_set(0, 0, 64, 0, 0, -1, -1) == _lib.ERR_SHAPE  # chunk
    assert lib.adrt_gb300_tune_set(0, 0, 64, 0, 0, 0, 2) == _lib.ERR_SHAPE  # use_fast
    assert lib.adrt_gb300_tune_set(0, 1, 64, 256, 4, 10, 0) == _lib.OK


def test_candidates(tune):
    c = tune.candidates("adrt", 1024, "float32")
    assert c[0] == tune.Config() and len(set(c)) == len(c)
    assert any(x.use_fast == 0 for x in c) and any(x.width == 128 for x in c)
    assert all(x.max_fused == 0 for x in c if x.use_fast == -1)
    c64 = tune.candidates("adrt", 1024, "float64")
    assert all(x.use_fast == -1 for x in c64)
    b = tune.candidates("bdrt", 1024, "float32")
    assert all(x.width == 0 for x in b) and len(b) > 1


def test_workspace_follows_table(tune):
    # Fewer fused stages per pass -> three passes -> two ping-pong buffers.
    w0 = _lib.workspace_size(_lib.OP_ADRT, 1, 1024, _lib.F64)
    tune.set_config("adrt", 1024, "float64", tune.Config(max_fused=3))
    w1 = _lib.workspace_size(_lib.OP_ADRT, 1, 1024, _lib.F64)
    assert w1 == 2 * w0


def test_select_keeps_builtin_within_noise():
    from adrt_gb300.tune import Config, select

    base, a, b = Config(), Config(128, 0, 0, -1), Config(256, 3, 96, 0)
    assert select([(base, 1.00), (a, 0.995), (b, 1.2)]) == (base, 1.00)      # 0.5 % faster: noise
    assert select([(base, 1.00), (a, 0.98), (b, 0.95)]) == (b, 0.95)        # clearly faster
    assert select([(base, 1.00), (a, 0.98)], min_gain=0.05) == (base, 1.00)
    assert select([(base, 1.00)]) == (base, 1.00)


def test_fast_forward_chunks_are_balanced():
    from adrt_gb300 import _lib

    lib_ws = lambda b: _lib.workspace_size(_lib.OP_ADRT, b, 1024, _lib.F32)  # noqa: E731
    per = 4 * 32 * 32 * 1056 * 4  # one image's intermediate at n = 1024
    assert lib_ws(8) == 8 * per                   # small batches: one chunk
    assert lib_ws(248) == 248 * per               # 4 GiB budget: 248 images
    assert lib_ws(249) == 125 * per               # two balanced chunks (125 + 124), not 248 + 1
    assert lib_ws(256) == 128 * per
    assert lib_ws(1000) == 200 * per              # five chunks of 200
