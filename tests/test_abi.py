"""CPU tests of the C ABI library: it builds, loads, exports every declared symbol, and
fails loudly (status codes + messages) without touching a GPU."""
import ctypes
import os
import re

import pytest

from conftest import REPO, GOLDEN


def _declared():
    with open(os.path.join(REPO, "include", "nnpgpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(nnpgpu_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(native_lib):
    names = _declared()
    assert len(names) >= 14
    for n in names:
        assert hasattr(native_lib, n), n
    from atomnn_gb300 import engine
    assert set(engine.EXPORTS) == set(names)


def _create(lib, path):
    from atomnn_gb300 import engine
    ctx = ctypes.c_void_p()
    rc = lib.nnpgpu_create(path.encode(), None, ctypes.byref(ctx))
    msg = lib.nnpgpu_last_error(ctx).decode() if ctx else ""
    if ctx:
        lib.nnpgpu_destroy(ctx)
    return rc, msg


def test_missing_potential_is_io_error(native_lib, tmp_path):
    from atomnn_gb300 import engine
    rc, msg = _create(native_lib, str(tmp_path / "nope.nnp"))
    assert rc == engine.ERR_IO and "could not open" in msg


def test_truncated_potential_is_io_error(native_lib, tmp_path):
    from atomnn_gb300 import engine
    src = open(os.path.join(GOLDEN, "small64.nnp")).read().splitlines()
    p = tmp_path / "cut.nnp"
    p.write_text("\n".join(src[:40]) + "\n")
    rc, msg = _create(native_lib, str(p))
    assert rc == engine.ERR_IO, msg


def _with_zeta(zeta):
    lines = open(os.path.join(GOLDEN, "small64.nnp")).read().splitlines()
    out, done = [], False
    for ln in lines:
        parts = ln.split()
        if not done and len(parts) == 3 and ln.startswith("\t") and parts[1] == "1.000000":
            ln = "\t%s %s %s" % (parts[0], zeta, parts[2])
            done = True
        out.append(ln)
    assert done
    return "\n".join(out) + "\n"


def test_unsupported_forms_are_reported(native_lib, tmp_path):
    """A real zeta is supported (per-function angular path); a zeta below 1 is refused with
    NNPGPU_ERR_UNSUPPORTED, since the force term's cw^(zeta-1) diverges at cw = 0."""
    from atomnn_gb300 import engine
    p = tmp_path / "z05.nnp"
    p.write_text(_with_zeta("0.500000"))
    rc, msg = _create(native_lib, str(p))
    assert rc == engine.ERR_UNSUPPORTED and "zeta" in msg
    p = tmp_path / "z3.nnp"
    p.write_text(_with_zeta("3.000000"))
    rc, msg = _create(native_lib, str(p))
    assert rc != engine.ERR_UNSUPPORTED, msg  # without a GPU the context fails later, with ERR_CUDA


def test_no_gpu_fails_loudly(native_lib, pot_small64):
    """Without a CUDA device the engine refuses to run: there is no CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from atomnn_gb300 import engine
    with pytest.raises(engine.NNPGPUError) as ei:
        engine.Engine(pot_small64)
    assert ei.value.code == engine.ERR_CUDA


def test_tune_shapes_validated(native_lib):
    """nnpgpu_set_tune accepts only the shapes the kernels are built for, and nnpgpu_get_tune
    reads back what was set; a context without a device still holds its settings."""
    from atomnn_gb300 import engine
    ctx = ctypes.c_void_p()
    native_lib.nnpgpu_create(os.path.join(GOLDEN, "small64.nnp").encode(), None, ctypes.byref(ctx))
    assert ctx
    try:
        assert native_lib.nnpgpu_set_tune(ctx, 3, 4, 4, 32) == engine.ERR_INVALID
        assert native_lib.nnpgpu_set_tune(ctx, 4, 4, 4, 48) == engine.ERR_INVALID
        assert native_lib.nnpgpu_set_tune(ctx, 2, 1, 4, 64) == engine.OK
        v = [ctypes.c_int() for _ in range(4)]
        assert native_lib.nnpgpu_get_tune(ctx, *[ctypes.byref(x) for x in v]) == engine.OK
        assert [x.value for x in v] == [2, 1, 4, 64]
        assert native_lib.nnpgpu_autotune(ctx, 0, None, None, None, None, 0, None, 0) == engine.ERR_INVALID
    finally:
        native_lib.nnpgpu_destroy(ctx)


def _ctx_without_device(lib, path):
    """A context whose potential is parsed; on a machine without a GPU nnpgpu_create returns
    NNPGPU_ERR_CUDA together with it."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: covered by tests/test_gpu_train.py")
    from atomnn_gb300 import engine
    ctx = ctypes.c_void_p()
    rc = lib.nnpgpu_create(path.encode(), None, ctypes.byref(ctx))
    assert rc == engine.ERR_CUDA and ctx
    return ctx


def test_write_potential_reproduces_the_file(native_lib, tmp_path):
    """nnpgpu_write_potential writes NNP::write's format: the file the workload writer made (the
    same tokens and number formats) comes back byte for byte."""
    from atomnn_gb300 import engine
    src = os.path.join(GOLDEN, "mixed512.nnp")
    ctx = _ctx_without_device(native_lib, src)
    try:
        out = tmp_path / "copy.nnp"
        assert native_lib.nnpgpu_write_potential(ctx, str(out).encode()) == engine.OK
        assert out.read_bytes() == open(src, "rb").read()
        assert native_lib.nnpgpu_write_potential(ctx, str(tmp_path / "no" / "dir.nnp").encode()) == engine.ERR_IO
    finally:
        native_lib.nnpgpu_destroy(ctx)


def test_params_roundtrip_through_the_potential_file(native_lib, oracle_lib, tmp_path):
    """get_params gives the oracle's parameters in the reference's order; set_params followed by
    write_potential gives a file whose networks carry the new values (to the 15 decimals of
    ANN::write)."""
    import numpy as np
    from atomnn_gb300 import engine
    src = os.path.join(GOLDEN, "mixed512.nnp")
    orc = oracle_lib.OracleNNP(src)
    ctx = _ctx_without_device(native_lib, src)
    try:
        for t in range(orc.ntypes):
            n = native_lib.nnpgpu_nparams(ctx, t)
            p = np.zeros(n)
            assert native_lib.nnpgpu_get_params(ctx, t, p.ctypes.data_as(ctypes.c_void_p)) == engine.OK
            np.testing.assert_array_equal(p, orc.params(t))
            q = p + np.random.default_rng(t).normal(0.0, 0.01, n)
            assert native_lib.nnpgpu_set_params(ctx, t, q.ctypes.data_as(ctypes.c_void_p)) == engine.OK
        bad = np.full(native_lib.nnpgpu_nparams(ctx, 0), np.nan)
        assert native_lib.nnpgpu_set_params(ctx, 0, bad.ctypes.data_as(ctypes.c_void_p)) == engine.ERR_INVALID
        out = str(tmp_path / "new.nnp")
        assert native_lib.nnpgpu_write_potential(ctx, out.encode()) == engine.OK
        orc2 = oracle_lib.OracleNNP(out)
        for t in range(orc.ntypes):
            q = orc.params(t) + np.random.default_rng(t).normal(0.0, 0.01, len(orc.params(t)))
            np.testing.assert_allclose(orc2.params(t), q, rtol=0, atol=1e-14)
    finally:
        native_lib.nnpgpu_destroy(ctx)
