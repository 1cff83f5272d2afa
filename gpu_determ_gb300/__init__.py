"""GB300 collision-integral library: Python view of the C ABI in include/gpu_determ.h.

The compute path is libgpu_determ.so (hand-written sm_103a kernels) built in
tree by ``gpu_determ_gb300.build``.  There is no CPU fallback: if the library
is missing or cannot be loaded, importing the bindings raises.

Arrays passed to the operator are CUDA tensors (torch) or raw device
pointers (int); distributions are laid out [node][cell] with the compact
in-sphere node index and leading dimension ``ld``.
"""
from __future__ import annotations

import ctypes as C
import os

__all__ = ["GDError", "GridSpec", "Context", "CollisionMatrix", "Mlp", "Surrogate", "Batch", "cell_rel_l2", "fma_peak", "lib", "library_path", "load_options",
           "DT_COURANT", "DT_FIXED", "CMATRIX_BF16", "CMATRIX_BF16X3",
           "MLP_SCALE_INPUT", "MLP_SCALE_OUTPUT", "MLP_LOSS_MSE", "MLP_LOSS_BATCH"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgpu_determ.so")
_lib = None

DT_COURANT = 0
DT_FIXED = 1
CMATRIX_BF16 = 0
CMATRIX_BF16X3 = 1
GAIN_PAIR = 0
GAIN_CMATRIX_BF16 = 1
GAIN_CMATRIX_BF16X3 = 2
GAIN_PAIR_TC = 3
BATCH_STREAMS = 0
BATCH_FUSED_PAIR_TC = 1
BATCH_FUSED_CMATRIX = 2
MLP_SCALE_INPUT = 1
MLP_SCALE_OUTPUT = 2
MLP_LOSS_MSE = 4
MLP_LOSS_BATCH = 8

_ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "unsupported",
           5: "singular system", 6: "I/O error"}


class GDError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gpu_determ error {code} ({_ERRORS.get(code, '?')}): {msg}")
        self.code = code


class _Spec(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("vmin", C.c_float * 3), ("vmax", C.c_float * 3), ("R", C.c_float)]


class _Options(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nyz", C.c_int), ("nxyz", C.c_int),
                ("npx", C.c_int)]


class _Info(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("n_pnt", C.c_int),
                ("du", C.c_float), ("dv", C.c_float), ("dw", C.c_float), ("d3v", C.c_float),
                ("nonzero_weights", C.c_int64), ("table_a_elems", C.c_int64),
                ("pair_products", C.c_int64), ("contraction_terms", C.c_int64),
                ("scatter_terms", C.c_int64), ("cmatrix_tiles", C.c_int64),
                ("cmatrix_slices", C.c_int64), ("cmatrix_node_tiles", C.c_int64)]


class _PairSizes(C.Structure):
    _fields_ = [("n_groups", C.c_int), ("nclass", C.c_int), ("n_entries", C.c_int64), ("n_items", C.c_int64),
                ("n_members", C.c_int64)]


class _MlpInfo(C.Structure):
    _fields_ = [("n_in", C.c_int), ("n_out", C.c_int), ("n_in_padded", C.c_int), ("n_out_padded", C.c_int),
                ("batch_cap", C.c_int), ("flags", C.c_int), ("steps", C.c_int64), ("num_params", C.c_int64),
                ("forward_flop_per_cell", C.c_double), ("in_gain", C.c_float), ("out_gain", C.c_float)]


class _Autotune(C.Structure):
    _fields_ = [("path", C.c_int), ("waves", C.c_int), ("best_ms", C.c_float), ("n_candidates", C.c_int),
                ("cand_path", C.c_int * 8), ("cand_waves", C.c_int * 8), ("cand_ms", C.c_float * 8),
                ("cluster", C.c_int), ("cand_cluster", C.c_int * 8)]


def library_path() -> str:
    return _LIB_PATH


def lib():
    """Load libgpu_determ.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise ImportError(
            f"{_LIB_PATH} is missing: build it with `python -m gpu_determ_gb300.build` "
            "(there is no CPU fallback)")
    L = C.CDLL(_LIB_PATH)
    vp, i, f, P = C.c_void_p, C.c_int, C.c_float, C.POINTER
    L.gd_version.restype = i
    L.gd_last_error.restype = C.c_char_p
    L.gd_grid_count.argtypes = [P(_Spec), P(i)]
    L.gd_grid_fill.argtypes = [P(_Spec), vp, vp, vp, vp, vp, vp, vp]
    L.gd_ctx_create.argtypes = [P(_Spec), i, P(vp)]
    L.gd_ctx_destroy.argtypes = [vp]
    L.gd_ctx_info.argtypes = [vp, P(_Info)]
    L.gd_export_tables.argtypes = [vp, vp, vp, vp]
    L.gd_correction_basis.argtypes = [vp, vp, vp]
    L.gd_collision.argtypes = [vp, vp, i, i, vp, vp, vp]
    L.gd_project.argtypes = [vp, vp, vp, vp, i, i, vp, vp, vp, vp]
    L.gd_relax.argtypes = [vp, vp, vp, vp, i, i, i, f, vp, vp, vp]
    L.gd_step.argtypes = [vp, vp, i, i, i, f, vp, vp, vp, vp, vp, vp, vp]
    L.gd_moments.argtypes = [vp, vp, i, i, vp, vp]
    L.gd_ctx_check.argtypes = [vp, vp]
    L.gd_set_memory_limit.argtypes = [C.c_size_t]
    L.gd_gain_noalloc.argtypes = [vp, vp, i, i, vp, vp]
    L.gd_load_options.argtypes = [C.c_char_p, P(_Options)]
    L.gd_cmatrix_create.argtypes = [vp, i, P(vp)]
    L.gd_cmatrix_gain.argtypes = [vp, vp, i, i, vp, vp]
    L.gd_cmatrix_destroy.argtypes = [vp]
    L.gd_cmatrix_set_cluster.argtypes = [vp, i]
    L.gd_cmatrix_set_chain.argtypes = [vp, i]
    L.gd_ctx_set_gain_path.argtypes = [vp, i]
    L.gd_box_to_compact.argtypes = [vp, vp, i, i, vp, i, vp]
    L.gd_compact_to_box.argtypes = [vp, vp, i, i, vp, i, vp]
    L.gd_mlp_create.argtypes = [i, i, i, i, C.c_uint64, P(vp)]
    L.gd_mlp_destroy.argtypes = [vp]
    L.gd_mlp_set_io_scale.argtypes = [vp, f, f]
    L.gd_mlp_info.argtypes = [vp, P(_MlpInfo)]
    L.gd_mlp_forward.argtypes = [vp, vp, i, i, vp, i, vp]
    L.gd_mlp_train_step.argtypes = [vp, vp, i, vp, i, vp, i, i, f, f, vp, vp]
    L.gd_mlp_loss.argtypes = [vp, vp, i, vp, i, vp, i, i, vp, vp]
    L.gd_mlp_check.argtypes = [vp, vp]
    L.gd_mlp_get_params.argtypes = [vp, vp]
    L.gd_mlp_set_params.argtypes = [vp, vp]
    L.gd_mlp_get_grads.argtypes = [vp, vp]
    L.gd_surrogate_create.argtypes = [vp, vp, vp, i, P(vp)]
    L.gd_surrogate_destroy.argtypes = [vp]
    L.gd_surrogate_gain.argtypes = [vp, vp, i, i, f, vp, vp, vp, P(i), vp]
    L.gd_cell_rel_l2.argtypes = [vp, i, vp, i, i, i, vp, vp]
    L.gd_cmatrix_check.argtypes = [vp, vp]
    L.gd_batch_create.argtypes = [P(vp)]
    L.gd_batch_destroy.argtypes = [vp]
    L.gd_batch_add.argtypes = [vp, vp, vp, i, i, i, f, vp, vp, vp]
    L.gd_batch_step.argtypes = [vp, i, vp]
    L.gd_batch_set_mode.argtypes = [vp, i]
    L.gd_batch_check.argtypes = [vp]
    L.gd_batch_info.argtypes = [vp, P(i), P(i), P(i), P(C.c_int64)]
    L.gd_ctx_autotune.argtypes = [vp, vp, i, i, i, C.c_double, P(_Autotune), vp]
    L.gd_fma_peak.argtypes = [i, i, P(C.c_double)]
    L.gd_mlp_inject_timeout.argtypes = [vp, i]
    L.gd_pair_tables.argtypes = [vp, P(_PairSizes), vp, vp, vp, vp, vp, vp]
    L.gd_pair_tc_table.argtypes = [vp, P(C.c_int64), vp, vp, vp]
    L.gd_ctx_inject_timeout.argtypes = [vp, i]
    for name in ("gd_grid_count", "gd_grid_fill", "gd_ctx_create", "gd_ctx_destroy", "gd_ctx_info",
                 "gd_export_tables", "gd_correction_basis", "gd_collision", "gd_project",
                 "gd_relax", "gd_step", "gd_moments", "gd_ctx_check", "gd_set_memory_limit", "gd_gain_noalloc",
                 "gd_box_to_compact", "gd_compact_to_box", "gd_load_options", "gd_cmatrix_create",
                 "gd_cmatrix_gain", "gd_cmatrix_destroy", "gd_cmatrix_set_cluster", "gd_cmatrix_set_chain", "gd_ctx_set_gain_path",
                 "gd_mlp_create", "gd_mlp_destroy", "gd_mlp_set_io_scale", "gd_mlp_info", "gd_mlp_forward", "gd_mlp_train_step",
                 "gd_mlp_loss", "gd_mlp_check", "gd_mlp_get_params", "gd_mlp_set_params", "gd_mlp_get_grads",
                 "gd_surrogate_create", "gd_surrogate_destroy", "gd_surrogate_gain", "gd_cell_rel_l2",
                 "gd_cmatrix_check", "gd_batch_create", "gd_batch_destroy", "gd_batch_add", "gd_batch_step",
                 "gd_batch_check", "gd_batch_info", "gd_batch_set_mode", "gd_ctx_autotune", "gd_fma_peak",
                 "gd_mlp_inject_timeout", "gd_ctx_inject_timeout", "gd_pair_tables", "gd_pair_tc_table"):
        getattr(L, name).restype = i
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        raise GDError(rc, lib().gd_last_error().decode(errors="replace"))


def _ptr(x):
    """Device pointer of a tensor (or an int / None)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream


def set_memory_limit(nbytes: int):
    """Cap the large device allocations of one object (0 = no cap)."""
    _check(lib().gd_set_memory_limit(int(nbytes)))


def load_options(path: str) -> dict:
    """Parse a reference options file (gpu.conf): nx, ny, nz, npx, nyz, nxyz."""
    o = _Options()
    _check(lib().gd_load_options(str(path).encode(), C.byref(o)))
    return {k: getattr(o, k) for k, _ in _Options._fields_}


class GridSpec:
    """Velocity lattice [vmin, vmax]^3 with n points per axis, cut to |xi| < R."""

    def __init__(self, nx, ny=None, nz=None, vmin=(-5.0, -5.0, -5.0), vmax=(5.0, 5.0, 5.0), R=16.5):
        self.nx, self.ny, self.nz = nx, (nx if ny is None else ny), (nx if nz is None else nz)
        self.vmin = tuple(float(v) for v in vmin)
        self.vmax = tuple(float(v) for v in vmax)
        self.R = float(R)

    def _c(self) -> _Spec:
        return _Spec(self.nx, self.ny, self.nz, (C.c_float * 3)(*self.vmin),
                     (C.c_float * 3)(*self.vmax), self.R)

    def count(self) -> int:
        n = C.c_int(0)
        _check(lib().gd_grid_count(C.byref(self._c()), C.byref(n)))
        return n.value

    def fill(self):
        """Host grid: dict of numpy arrays u, v, w, ui, vi, wi, steps."""
        import numpy as np
        n = self.count()
        out = {"u": np.zeros(self.nx, np.float32), "v": np.zeros(self.ny, np.float32),
               "w": np.zeros(self.nz, np.float32), "ui": np.zeros(n, np.int32),
               "vi": np.zeros(n, np.int32), "wi": np.zeros(n, np.int32),
               "steps": np.zeros(4, np.float32)}
        _check(lib().gd_grid_fill(C.byref(self._c()), *(out[k].ctypes.data for k in
                                                        ("u", "v", "w", "ui", "vi", "wi", "steps"))))
        return out


class Context:
    """Device tables for one velocity grid and the collision operator on it."""

    def __init__(self, spec: GridSpec, device: int = 0):
        self.spec = spec
        self._h = C.c_void_p()
        _check(lib().gd_ctx_create(C.byref(spec._c()), int(device), C.byref(self._h)))
        self.device = device
        self.info = self._info()
        self.n_pnt = self.info["n_pnt"]

    def _info(self) -> dict:
        inf = _Info()
        _check(lib().gd_ctx_info(self._h, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in _Info._fields_}

    def close(self):
        if self._h:
            lib().gd_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_gain_path(self, path: int):
        """GAIN_PAIR (FP32 pair-product kernel), GAIN_CMATRIX_BF16, GAIN_CMATRIX_BF16X3 or
        GAIN_PAIR_TC (pair products with the weight contraction on the tensor cores)."""
        _check(lib().gd_ctx_set_gain_path(self._h, int(path)))

    # tables -----------------------------------------------------------------
    def export_tables(self, b=None, a=None, stream=None):
        _check(lib().gd_export_tables(self._h, _ptr(b), _ptr(a), _stream(stream)))

    def correction_basis(self, basis, stream=None):
        _check(lib().gd_correction_basis(self._h, _ptr(basis), _stream(stream)))

    # operator ---------------------------------------------------------------
    def collision(self, f, ncells, ld, nu=None, gain=None, stream=None):
        _check(lib().gd_collision(self._h, _ptr(f), int(ncells), int(ld), _ptr(nu), _ptr(gain),
                                  _stream(stream)))

    def project(self, f, nu, gain, ncells, ld, nu_corr=None, q=None, x=None, stream=None):
        _check(lib().gd_project(self._h, _ptr(f), _ptr(nu), _ptr(gain), int(ncells), int(ld),
                                _ptr(nu_corr), _ptr(q), _ptr(x), _stream(stream)))

    def relax(self, f, nu_corr, gain, ncells, ld, mode, param, time=None, dt=None, stream=None):
        _check(lib().gd_relax(self._h, _ptr(f), _ptr(nu_corr), _ptr(gain), int(ncells), int(ld),
                              int(mode), float(param), _ptr(time), _ptr(dt), _stream(stream)))

    def step(self, f, ncells, ld, mode, param, nu=None, gain=None, q=None, m5=None, time=None,
             dt=None, stream=None):
        _check(lib().gd_step(self._h, _ptr(f), int(ncells), int(ld), int(mode), float(param),
                             _ptr(nu), _ptr(gain), _ptr(q), _ptr(m5), _ptr(time), _ptr(dt),
                             _stream(stream)))

    def autotune(self, f, ncells, ld, path_mask=1 << GAIN_PAIR, mem_budget=0.0, stream=None) -> dict:
        """Time the gain candidates on these cells and keep the fastest."""
        r = _Autotune()
        _check(lib().gd_ctx_autotune(self._h, _ptr(f), int(ncells), int(ld), int(path_mask), float(mem_budget),
                                     C.byref(r), _stream(stream)))
        names = {GAIN_PAIR: "pair", GAIN_CMATRIX_BF16: "cmatrix_bf16", GAIN_CMATRIX_BF16X3: "cmatrix_bf16x3",
                 GAIN_PAIR_TC: "pair_tc"}
        cands = [{"path": names[r.cand_path[k]], "waves": r.cand_waves[k], "cluster": r.cand_cluster[k],
                  "ms": r.cand_ms[k]} for k in range(r.n_candidates)]
        return {"path": names[r.path], "waves": r.waves, "cluster": r.cluster, "best_ms": r.best_ms,
                "candidates": cands}

    def box_to_compact(self, box, ncells, ld_box, compact, ld, stream=None):
        _check(lib().gd_box_to_compact(self._h, _ptr(box), int(ncells), int(ld_box), _ptr(compact), int(ld),
                                       _stream(stream)))

    def compact_to_box(self, compact, ncells, ld, box, ld_box, stream=None):
        _check(lib().gd_compact_to_box(self._h, _ptr(compact), int(ncells), int(ld), _ptr(box), int(ld_box),
                                       _stream(stream)))

    def check(self, stream=None):
        """Raise GDError when a projection met non-finite data or a singular system."""
        _check(lib().gd_ctx_check(self._h, _stream(stream)))

    def moments(self, f, ncells, ld, m5, stream=None):
        _check(lib().gd_moments(self._h, _ptr(f), int(ncells), int(ld), _ptr(m5), _stream(stream)))

    def pair_tables(self) -> dict:
        """The pair-product tables the gain kernels read (gd_pair_tables), as
        numpy arrays."""
        import numpy as np
        sz = _PairSizes()
        _check(lib().gd_pair_tables(self._h, C.byref(sz), None, None, None, None, None, None))
        nxyz = self.spec.nx * self.spec.ny * self.spec.nz
        out = {"grp_row_off": np.zeros(sz.n_groups + 1, np.int32),
               "entry_class": np.zeros(sz.n_entries, np.int32), "entry_w": np.zeros(sz.n_entries, np.float32),
               "item_off": np.zeros(nxyz + 1, np.int32), "items": np.zeros((sz.n_items, 3), np.int32),
               "members": np.zeros(sz.n_members, np.uint32)}
        _check(lib().gd_pair_tables(self._h, C.byref(sz), *(out[k].ctypes.data for k in
                                                            ("grp_row_off", "entry_class", "entry_w", "item_off",
                                                             "items", "members"))))
        out["nclass"] = sz.nclass
        return out

    def pair_tc_table(self) -> dict:
        """The per-D weight table of the pair path on tensor cores (raw BF16
        bits of the hi and lo parts, [rows][64]) and each D's first row."""
        import numpy as np
        rows = C.c_int64(0)
        _check(lib().gd_pair_tc_table(self._h, C.byref(rows), None, None, None))
        nxyz = self.spec.nx * self.spec.ny * self.spec.nz
        out = {"wrow": np.zeros(nxyz, np.int32), "wh": np.zeros((rows.value, 64), np.uint16),
               "wl": np.zeros((rows.value, 64), np.uint16)}
        _check(lib().gd_pair_tc_table(self._h, C.byref(rows), out["wrow"].ctypes.data, out["wh"].ctypes.data,
                                      out["wl"].ctypes.data))
        return out

    def inject_timeout(self, polls: int):
        """Failure-detection test hook: the next tensor-core loss GEMM's bounded
        wait runs out after `polls` polls; check() then reports it."""
        _check(lib().gd_ctx_inject_timeout(self._h, int(polls)))


class CollisionMatrix:
    """Dense collision matrices G_i of a context on the device and the
    tensor-core gain I_i = f^T G_i f (modes CMATRIX_BF16, CMATRIX_BF16X3)."""

    def __init__(self, ctx: Context, mode: int = CMATRIX_BF16X3):
        self.ctx = ctx
        self.mode = mode
        self._h = C.c_void_p()
        _check(lib().gd_cmatrix_create(ctx._h, int(mode), C.byref(self._h)))

    def gain(self, f, ncells, ld, gain, stream=None):
        _check(lib().gd_cmatrix_gain(self._h, _ptr(f), int(ncells), int(ld), _ptr(gain), _stream(stream)))

    def set_cluster(self, ctas: int):
        """CTAs per tensor-core MMA: 2 (default; CTA pair, M = 256 cells) or 1."""
        _check(lib().gd_cmatrix_set_cluster(self._h, int(ctas)))

    def set_chain(self, tiles: int):
        """Most stored tiles per tensor-memory accumulation (even; 0 = unlimited)."""
        _check(lib().gd_cmatrix_set_chain(self._h, int(tiles)))

    def close(self):
        if self._h:
            lib().gd_cmatrix_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mlp:
    """Surrogate network n_in -> 256 -> 512 -> 512 -> 256 (+residual) -> n_out
    on the tensor cores (BF16 weights, FP32 accumulation); arrays are
    [feature][cell] device tensors with leading dimension ld."""

    def __init__(self, n_in: int, n_out: int, batch_cap: int, flags: int = MLP_SCALE_INPUT | MLP_SCALE_OUTPUT,
                 seed: int = 0):
        self._h = C.c_void_p()
        _check(lib().gd_mlp_create(int(n_in), int(n_out), int(batch_cap), int(flags), int(seed),
                                   C.byref(self._h)))
        inf = _MlpInfo()
        _check(lib().gd_mlp_info(self._h, C.byref(inf)))
        self.info = {k: getattr(inf, k) for k, _ in _MlpInfo._fields_}
        self.n_in, self.n_out, self.cap = n_in, n_out, batch_cap

    def set_io_scale(self, in_gain: float, out_gain: float):
        """Global gains on the scaled input and on the network output."""
        _check(lib().gd_mlp_set_io_scale(self._h, float(in_gain), float(out_gain)))
        self.info["in_gain"], self.info["out_gain"] = float(in_gain), float(out_gain)

    def layer_shapes(self):
        """[(out, in)] of the five layers with the padded feature counts."""
        i, o = self.info["n_in_padded"], self.info["n_out_padded"]
        return [(256, i), (512, 256), (512, 512), (256, 512), (o, 256)]

    def forward(self, x, ldx, batch, y, ldy, stream=None):
        _check(lib().gd_mlp_forward(self._h, _ptr(x), int(ldx), int(batch), _ptr(y), int(ldy), _stream(stream)))

    def train_step(self, x, ldx, t, ldt, batch, lr, weight_decay=0.0, loss=None, tden=None, ldd=0, stream=None):
        _check(lib().gd_mlp_train_step(self._h, _ptr(x), int(ldx), _ptr(t), int(ldt), _ptr(tden), int(ldd),
                                       int(batch), float(lr), float(weight_decay), _ptr(loss), _stream(stream)))

    def loss(self, x, ldx, t, ldt, batch, row_loss, tden=None, ldd=0, stream=None):
        _check(lib().gd_mlp_loss(self._h, _ptr(x), int(ldx), _ptr(t), int(ldt), _ptr(tden), int(ldd),
                                 int(batch), _ptr(row_loss), _stream(stream)))

    def check(self, stream=None):
        _check(lib().gd_mlp_check(self._h, _stream(stream)))

    def inject_timeout(self, polls: int):
        """Failure-detection test hook: the next forward pass's first GEMM has
        its bounded wait run out after `polls` polls; check() then reports it."""
        _check(lib().gd_mlp_inject_timeout(self._h, int(polls)))

    def get_params(self):
        import numpy as np
        out = np.zeros(self.info["num_params"], np.float32)
        _check(lib().gd_mlp_get_params(self._h, out.ctypes.data))
        return out

    def set_params(self, p):
        import numpy as np
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.info["num_params"]
        _check(lib().gd_mlp_set_params(self._h, p.ctypes.data))

    def get_grads(self):
        import numpy as np
        out = np.zeros(self.info["num_params"], np.float32)
        _check(lib().gd_mlp_get_grads(self._h, out.ctypes.data))
        return out

    def close(self):
        if self._h:
            lib().gd_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Surrogate:
    """Gain from the trained network `net` for cells whose estimated error
    (network `est`) is within tol, the context's plain gain for the rest."""

    def __init__(self, ctx: Context, net: Mlp, est: Mlp | None, max_cells: int):
        self.ctx, self.net, self.est = ctx, net, est
        self._h = C.c_void_p()
        _check(lib().gd_surrogate_create(ctx._h, net._h, est._h if est is not None else None, int(max_cells),
                                         C.byref(self._h)))

    def gain(self, f, ncells, ld, tol, nu, gain, est_out=None, stream=None) -> int:
        """Returns the number of cells that took the plain method."""
        n = C.c_int(0)
        _check(lib().gd_surrogate_gain(self._h, _ptr(f), int(ncells), int(ld), float(tol), _ptr(nu), _ptr(gain),
                                       _ptr(est_out), C.byref(n), _stream(stream)))
        return n.value

    def close(self):
        if self._h:
            lib().gd_surrogate_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fma_peak(device: int = 0, precision: int = 32) -> float:
    """Measured FP32 (precision 32) or FP64 (64) FMA throughput of the device
    in FLOP/s: the roofline denominator of the SIMT kernels."""
    v = C.c_double(0.0)
    _check(lib().gd_fma_peak(int(device), int(precision), C.byref(v)))
    return v.value


def cell_rel_l2(a, lda, b, ldb, n, ncells, out, stream=None):
    """out[c] = ||a[:,c] - b[:,c]|| / ||b[:,c]|| (FP64 device arrays)."""
    _check(lib().gd_cell_rel_l2(_ptr(a), int(lda), _ptr(b), int(ldb), int(n), int(ncells), _ptr(out),
                                _stream(stream)))


class Batch:
    """Groups (context, cells) stepped together; with use_graph every step
    after the second is one CUDA graph launch."""

    def __init__(self):
        self._h = C.c_void_p()
        _check(lib().gd_batch_create(C.byref(self._h)))
        self._keep = []

    def add(self, ctx: Context, f, ncells, ld, mode, param, m5=None, time=None, dt=None):
        _check(lib().gd_batch_add(self._h, ctx._h, _ptr(f), int(ncells), int(ld), int(mode), float(param),
                                  _ptr(m5), _ptr(time), _ptr(dt)))
        self._keep.append((ctx, f, m5, time, dt))

    def step(self, use_graph=True, stream=None):
        _check(lib().gd_batch_step(self._h, int(bool(use_graph)), _stream(stream)))

    def set_mode(self, mode: int):
        """BATCH_STREAMS (per-group steps on forked streams),
        BATCH_FUSED_PAIR_TC (every group's gain in one persistent launch of the
        pair-product kernel) or BATCH_FUSED_CMATRIX (every group's gain in one
        launch of the collision-matrix kernel)."""
        _check(lib().gd_batch_set_mode(self._h, int(mode)))

    def check(self):
        _check(lib().gd_batch_check(self._h))

    def info(self) -> dict:
        g, s, n, k = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int64(0)
        _check(lib().gd_batch_info(self._h, C.byref(g), C.byref(s), C.byref(n), C.byref(k)))
        return {"groups": g.value, "streams": s.value, "graph_nodes": n.value, "steps": k.value}

    def close(self):
        if self._h:
            lib().gd_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
