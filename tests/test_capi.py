"""C ABI checks that need no GPU: the library loads, exports every entry point
include/gpu_determ.h declares, builds the host grid bit-exactly like the
oracle's restatement of velocity_grid.cu, and rejects bad arguments."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle.pyoracle import Oracle

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(HEADER):
        if fn.endswith(".h"):
            src = open(os.path.join(HEADER, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(gd_\w+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("gd_ctx_create", "gd_collision", "gd_project", "gd_relax", "gd_step",
                 "gd_grid_fill", "gd_export_tables", "gd_correction_basis", "gd_last_error"):
        assert must in syms


def test_library_exports_every_declared_symbol(gdlib):
    L = gdlib.lib()
    for name in declared_symbols():
        assert hasattr(L, name), name
        assert isinstance(getattr(L, name), C._CFuncPtr)


SPECS = [
    dict(nx=16, R=16.5), dict(nx=16, R=4.8), dict(nx=12, R=4.8), dict(nx=20, R=4.8),
    dict(nx=24, R=4.8), dict(nx=32, R=5.5), dict(nx=8, ny=10, nz=6, R=3.0),
    dict(nx=16, vmin=(-3, -4, -5), vmax=(4, 3, 5), R=4.0), dict(nx=10, R=0.0), dict(nx=14, R=-1.0),
]


@pytest.mark.parametrize("kw", SPECS)
def test_host_grid_bit_exact(gdlib, kw):
    spec = gdlib.GridSpec(**kw)
    g = spec.fill()
    o = Oracle(spec.nx, spec.ny, spec.nz, spec.vmin, spec.vmax, spec.R)
    assert spec.count() == o.n_pnt
    for k in ("u", "v", "w", "ui", "vi", "wi"):
        assert np.array_equal(g[k], getattr(o, k)), k
    assert np.array_equal(g["steps"], o.steps)


@pytest.mark.parametrize("bad", [dict(nx=15), dict(nx=0), dict(nx=16, vmin=(5, 5, 5), vmax=(-5, -5, -5)),
                                 dict(nx=66)])
def test_bad_spec_rejected(gdlib, bad):
    spec = gdlib.GridSpec(**bad)
    with pytest.raises(gdlib.GDError) as e:
        spec.count()
    assert e.value.code in (1, 4)
    assert gdlib.lib().gd_last_error()


def test_null_arguments_rejected(gdlib):
    L = gdlib.lib()
    assert L.gd_ctx_create(None, 0, None) == 1
    assert L.gd_collision(None, None, 1, 1, None, None, None) == 1
    assert L.gd_ctx_destroy(None) == 0
    out = C.c_void_p()
    # surrogate, batch and autotuner arguments are checked before any CUDA call
    assert L.gd_mlp_create(0, 10, 64, 0, 0, C.byref(out)) == 1
    assert L.gd_mlp_create(10, 10, 100, 0, 0, C.byref(out)) == 1        # cap not a multiple of 64
    assert L.gd_mlp_create(10, 10, 64, 2, 0, C.byref(out)) == 1         # output scaling needs input scaling
    assert L.gd_mlp_create(10, 10, 64, 64, 0, C.byref(out)) == 1        # unknown flag
    assert L.gd_mlp_forward(None, None, 1, 1, None, 1, None) == 1
    assert L.gd_mlp_train_step(None, None, 64, None, 64, None, 0, 64, 0.0, 0.0, None, None) == 1
    assert L.gd_surrogate_create(None, None, None, 1, C.byref(out)) == 1
    assert L.gd_surrogate_gain(None, None, 1, 1, 1.0, None, None, None, None, None) == 1
    assert L.gd_cell_rel_l2(None, 1, None, 1, 1, 1, None, None) == 1
    assert L.gd_batch_add(None, None, None, 1, 1, 0, 1.0, None, None, None) == 1
    assert L.gd_batch_step(None, 1, None) == 1
    assert L.gd_ctx_autotune(None, None, 1, 1, 1, 0.0, None, None) == 1
    assert L.gd_mlp_destroy(None) == 0 and L.gd_surrogate_destroy(None) == 0 and L.gd_batch_destroy(None) == 0
    assert L.gd_ctx_check(None, None) == 1
    # a memory cap refuses the surrogate network before any CUDA call
    try:
        assert L.gd_set_memory_limit(1 << 20) == 0
        assert L.gd_mlp_create(3648, 3648, 4096, 3, 0, C.byref(out)) == 3
        assert b"memory limit" in L.gd_last_error()
    finally:
        L.gd_set_memory_limit(0)


def test_missing_library_fails_loudly(gdlib, monkeypatch):
    import gpu_determ_gb300 as gd
    monkeypatch.setattr(gd, "_LIB_PATH", "/nonexistent/libgpu_determ.so")
    monkeypatch.setattr(gd, "_lib", None)
    with pytest.raises(ImportError):
        gd.lib()


def test_python_constants_match_header(gdlib):
    """The binding's enum constants equal the header's (gain paths, matrix
    modes, network flags)."""
    src = open(os.path.join(HEADER, "gpu_determ.h")).read()
    vals = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(GD_[A-Z0-9_]+)\s*=\s*(\d+)", src)}
    for name, py in (("GD_GAIN_PAIR", "GAIN_PAIR"), ("GD_GAIN_CMATRIX_BF16", "GAIN_CMATRIX_BF16"),
                     ("GD_GAIN_CMATRIX_BF16X3", "GAIN_CMATRIX_BF16X3"), ("GD_GAIN_PAIR_TC", "GAIN_PAIR_TC"),
                     ("GD_CMATRIX_BF16", "CMATRIX_BF16"), ("GD_CMATRIX_BF16X3", "CMATRIX_BF16X3"),
                     ("GD_MLP_SCALE_INPUT", "MLP_SCALE_INPUT"), ("GD_MLP_SCALE_OUTPUT", "MLP_SCALE_OUTPUT"),
                     ("GD_MLP_LOSS_MSE", "MLP_LOSS_MSE"), ("GD_MLP_LOSS_BATCH", "MLP_LOSS_BATCH")):
        assert name in vals, name
        assert getattr(gdlib, py) == vals[name], (name, vals[name], getattr(gdlib, py))
