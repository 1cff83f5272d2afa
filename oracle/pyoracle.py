"""numpy/ctypes view of the oracle library (test infrastructure only).

Imported by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py, as the oracle results are compared with.  The product path never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.or_grid_count.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_float]
        L.or_grid_count.restype = C.c_int
        L.or_grid_fill.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_float,
                                   _f32p, _f32p, _f32p, _i32p, _i32p, _i32p, _f32p]
        L.or_grid_fill.restype = C.c_int
        L.or_relative_speed.argtypes = [C.c_float] * 3 + [C.c_int] * 3
        L.or_relative_speed.restype = C.c_float
        L.or_box_sphere_area.argtypes = [C.c_double] * 3 + [C.c_int] * 3 + [C.c_double]
        L.or_box_sphere_area.restype = C.c_double
        L.or_build_dense_tables.argtypes = [C.c_int] * 3 + [C.c_float] * 4 + [_f32p, _f32p]
        L.or_create.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_float]
        L.or_create.restype = C.c_void_p
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_n_pnt.argtypes = [C.c_void_p]
        L.or_n_pnt.restype = C.c_int
        L.or_table_a.argtypes = [C.c_void_p]
        L.or_table_a.restype = C.POINTER(C.c_float)
        L.or_table_b.argtypes = [C.c_void_p]
        L.or_table_b.restype = C.POINTER(C.c_float)
        L.or_compact_of_box.argtypes = [C.c_void_p]
        L.or_compact_of_box.restype = C.POINTER(C.c_int)
        L.or_count_work.argtypes = [C.c_void_p, _i64p]
        L.or_index_map_digest.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")]
        for name, outp in (("or_loss_f64", _f64p), ("or_gain_f64", _f64p),
                           ("or_loss_f32", _f32p), ("or_gain_f32", _f32p)):
            getattr(L, name).argtypes = [C.c_void_p, _f32p, C.c_int, _i32p, C.c_int, outp]
        for name in ("or_loss_literal", "or_gain_literal"):
            getattr(L, name).argtypes = [C.c_void_p, _f32p, C.c_int, C.c_int, _i32p, C.c_int, _f32p]
        L.or_project.argtypes = [C.c_void_p, _f32p, _f32p, _f32p, C.c_int, _f64p, _f64p, _f64p]
        L.or_project.restype = C.c_int
        L.or_moments.argtypes = [C.c_void_p, _f64p, C.c_int, _f64p]
        _lib = L
    return _lib


def ref_weights():
    """The reference's own calc_matrix_element compiled for the host, or None
    when the reference checkout is not available on this machine."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_calc_matrix_element.argtypes = [C.c_double] * 3 + [C.c_int] * 3 + [C.c_double]
        L.ref_calc_matrix_element.restype = C.c_double
        _ref = L
    return _ref


def _vec3(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(3))


class Oracle:
    """Grid, dense tables and the CPU collision operator for one velocity grid."""

    def __init__(self, nx, ny=None, nz=None, vmin=(-5.0, -5.0, -5.0), vmax=(5.0, 5.0, 5.0),
                 R=16.5):
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        L = lib()
        self.nx, self.ny, self.nz = nx, ny, nz
        self.nyz, self.nxyz = ny * nz, nx * ny * nz
        self.vmin, self.vmax, self.R = _vec3(vmin), _vec3(vmax), float(R)
        self._c = L.or_create(nx, ny, nz, self.vmin, self.vmax, self.R)
        if not self._c:
            raise ValueError("grid sizes must be even and >= 2")
        np_ = L.or_n_pnt(self._c)
        self.u = np.zeros(nx, np.float32)
        self.v = np.zeros(ny, np.float32)
        self.w = np.zeros(nz, np.float32)
        self.ui = np.zeros(np_, np.int32)
        self.vi = np.zeros(np_, np.int32)
        self.wi = np.zeros(np_, np.int32)
        steps = np.zeros(4, np.float32)
        L.or_grid_fill(nx, ny, nz, self.vmin, self.vmax, self.R, self.u, self.v, self.w,
                       self.ui, self.vi, self.wi, steps)
        self.du, self.dv, self.dw, self.d3v = (float(s) for s in steps)
        self.steps = steps
        self.n_pnt = np_
        self.box_of_compact = ((self.ui * ny + self.vi) * nz + self.wi).astype(np.int32)
        self.compact_of_box = np.ctypeslib.as_array(L.or_compact_of_box(self._c),
                                                    shape=(self.nxyz,)).copy()

    def __del__(self):
        if getattr(self, "_c", None):
            lib().or_destroy(self._c)
            self._c = None

    # tables -------------------------------------------------------------
    @property
    def a_size(self):
        return (self.nx // 2) * self.nx * (self.ny // 2) * (self.nz // 2) * self.nyz

    def table_a(self):
        return np.ctypeslib.as_array(lib().or_table_a(self._c), shape=(self.a_size,)).copy()

    def table_b(self):
        return np.ctypeslib.as_array(lib().or_table_b(self._c), shape=(self.nxyz,)).copy()

    def count_work(self):
        out = np.zeros(3, np.int64)
        lib().or_count_work(self._c, out)
        return {"nonzero_weights": int(out[0]), "terms": int(out[1]), "subterms": int(out[2])}

    def index_map_digest(self):
        """Digest of the gain's index map: (count, sum mix_a, xor mix_b,
        FP64 weight sum) over keys i << 32 | s << 15 | n (or_index_map_digest)."""
        out = np.zeros(4, np.uint64)
        lib().or_index_map_digest(self._c, out)
        return int(out[0]), int(out[1]), int(out[2]), float(out[3:4].view(np.float64)[0])

    # layouts --------------------------------------------------------------
    def to_box(self, f_compact):
        """[n_pnt][cells] -> [nxyz][cells] with zeros outside the sphere."""
        f_compact = np.asarray(f_compact, np.float32)
        out = np.zeros((self.nxyz,) + f_compact.shape[1:], np.float32)
        out[self.box_of_compact] = f_compact
        return out

    def _nodes(self, nodes):
        if nodes is None:
            nodes = self.box_of_compact
        return np.ascontiguousarray(np.asarray(nodes, dtype=np.int32).ravel())

    # operator -------------------------------------------------------------
    def _run(self, name, f_box, nodes, dtype):
        f_box = np.ascontiguousarray(f_box, dtype=np.float32)
        if f_box.ndim == 1:
            f_box = f_box[:, None]
        nodes = self._nodes(nodes)
        out = np.zeros((len(nodes), f_box.shape[1]), dtype)
        getattr(lib(), name)(self._c, f_box, f_box.shape[1], nodes, len(nodes), out)
        return out

    def loss_f64(self, f_box, nodes=None):
        return self._run("or_loss_f64", f_box, nodes, np.float64)

    def gain_f64(self, f_box, nodes=None):
        return self._run("or_gain_f64", f_box, nodes, np.float64)

    def loss_f32(self, f_box, nodes=None):
        return self._run("or_loss_f32", f_box, nodes, np.float32)

    def gain_f32(self, f_box, nodes=None):
        return self._run("or_gain_f32", f_box, nodes, np.float32)

    def _literal(self, name, f_box, cell, nodes):
        f_box = np.ascontiguousarray(f_box, dtype=np.float32)
        nodes = self._nodes(nodes)
        out = np.zeros(len(nodes), np.float32)
        getattr(lib(), name)(self._c, f_box.ravel(), f_box.shape[1], int(cell), nodes,
                             len(nodes), out)
        return out

    def loss_literal(self, f_box, cell, nodes):
        return self._literal("or_loss_literal", f_box, cell, nodes)

    def gain_literal(self, f_box, cell, nodes):
        return self._literal("or_gain_literal", f_box, cell, nodes)

    def project(self, f, nu, gain):
        """FP64 conservation projection over compact [n_pnt][cells] arrays."""
        f = np.ascontiguousarray(f, np.float32)
        nu = np.ascontiguousarray(nu, np.float32)
        gain = np.ascontiguousarray(gain, np.float32)
        nc = f.shape[1]
        nu_c = np.zeros(f.shape, np.float64)
        q = np.zeros(f.shape, np.float64)
        x = np.zeros((nc, 5), np.float64)
        sing = lib().or_project(self._c, f, nu, gain, nc, nu_c, q, x)
        return nu_c, q, x, sing

    def project_f64(self, f, nu, gain):
        """The conservation projection with FP64 nu and gain (no FP32 rounding
        of its inputs), in numpy: A X = B with A_kl = sum_i f nu phi_k phi_l,
        B_k = sum_i (I - f nu) phi_k, nu' = nu (1 + X.phi), Q = I - f nu'
        (the intended per-cell system of collision_integral.cu:217-526 over
        the basis of velocity.cu:17-50).  Returns Q, [n_pnt][cells] float64."""
        phi = self.phi()
        f64 = np.asarray(f, np.float64)
        fnu = f64 * nu
        A = np.einsum("ic,ik,il->ckl", fnu, phi, phi)
        B = np.einsum("ic,ik->ck", gain - fnu, phi)
        X = np.linalg.solve(A, B[..., None])[..., 0]
        return gain - f64 * nu * (1.0 + phi @ X.T)

    def moments(self, f):
        f = np.ascontiguousarray(f, np.float64)
        m = np.zeros((f.shape[1], 5), np.float64)
        lib().or_moments(self._c, f, f.shape[1], m)
        return m

    def phi(self):
        """Per compact node basis (1, u, v, w, u^2+v^2+w^2) in FP64."""
        xu = self.u[self.ui].astype(np.float64)
        xv = self.v[self.vi].astype(np.float64)
        xw = self.w[self.wi].astype(np.float64)
        return np.stack([np.ones_like(xu), xu, xv, xw, xu * xu + xv * xv + xw * xw], axis=1)


def maxwellian(o: Oracle, n=1.0, u=(0.0, 0.0, 0.0), T=1.0):
    """n (pi T)^{-3/2} exp(-|xi - u|^2 / T) at the compact nodes, FP64."""
    xu = o.u[o.ui].astype(np.float64)
    xv = o.v[o.vi].astype(np.float64)
    xw = o.w[o.wi].astype(np.float64)
    c2 = (xu - u[0]) ** 2 + (xv - u[1]) ** 2 + (xw - u[2]) ** 2
    return n * (np.pi * T) ** -1.5 * np.exp(-c2 / T)
