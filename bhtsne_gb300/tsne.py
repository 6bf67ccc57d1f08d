"""Python mirror of the reference builder `tSNE<'data, T, U, const D>`
(bhtsne 0.7.10, src/lib.rs:149-1249) over the CUDA library's C ABI.

Same method names, defaults and error messages as the Rust builder; the
reference's panics surface as `BhtsneError` with code EINVAL and the
reference's message text. The dataset is given at construction like
`tSNE::new(&data)`; the Euclidean metric is selected by the finisher, and any
other metric enters through `*_with_neighbors` (a precomputed kNN table) or,
for `exact`, through a dense distance matrix.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Callable, Optional, Sequence

import numpy as np

from . import _lib as L


@dataclass(frozen=True)
class Neighbor:
    """`Neighbor<T>` (src/lib.rs:108-111): an index and its distance."""
    index: int
    distance: float


@dataclass
class SparseAffinities:
    """`SparseAffinities<T>` (src/lib.rs:117-144)."""
    rows: np.ndarray
    columns: np.ndarray
    values: np.ndarray
    perplexity: float


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def _dtype_code(dt) -> int:
    dt = np.dtype(dt)
    if dt == np.float32:
        return L.F32
    if dt == np.float64:
        return L.F64
    raise TypeError("dtype must be float32 or float64")


def neighbors_to_arrays(neighbors, dtype=np.float32):
    """Accepts a (indices, distances) pair of arrays or a sequence of rows of
    Neighbor; checks the row shape like check_neighbors (src/lib.rs:781-798)."""
    if isinstance(neighbors, tuple) and len(neighbors) == 2:
        idx = np.ascontiguousarray(neighbors[0], dtype=np.uint64)
        dist = np.ascontiguousarray(neighbors[1], dtype=dtype)
        if idx.ndim != 2 or idx.shape != dist.shape:
            raise L.BhtsneError(L.EINVAL, "error: every neighbors row must have the same length, greater than zero.")
        return idx, dist
    rows = list(neighbors)
    k = len(rows[0]) if rows else 0
    if k == 0 or any(len(r) != k for r in rows):
        raise L.BhtsneError(L.EINVAL, "error: every neighbors row must have the same length, greater than zero.")
    idx = np.array([[nb.index for nb in r] for r in rows], dtype=np.uint64)
    dist = np.array([[nb.distance for nb in r] for r in rows], dtype=dtype)
    return idx, dist


class TSNE:
    """t-SNE builder on one GPU. `data` is an (n_samples, dim) array (or just
    n_samples when only the `*_with_neighbors` / `with_affinities` entry
    points are used); `dtype` is the reference's T; `D` its const generic."""

    def __init__(self, data, D: int = 2, dtype=np.float32, ctx: Optional[L.Context] = None):
        self.ctx = ctx or L.default_context()
        self.lib = self.ctx.lib
        self.dtype = np.dtype(dtype)
        self.D = int(D)
        if isinstance(data, (int, np.integer)):
            self.data = None
            self.n = int(data)
        else:
            self.data = np.ascontiguousarray(np.asarray(data, dtype=self.dtype))
            if self.data.ndim == 1:
                self.data = self.data.reshape(-1, 1)
            self.n = self.data.shape[0]
        h = C.c_void_p()
        self._check_ctx(self.lib.bhtsne_tsne_new(self.ctx.handle, _dtype_code(self.dtype), self.D, self.n, C.byref(h)))
        self.handle = h
        self._cb = None

    # -- plumbing -------------------------------------------------------------
    def _check_ctx(self, rc):
        if rc != L.OK:
            raise L.BhtsneError(rc, self.lib.bhtsne_ctx_last_error(self.ctx.handle).decode())

    def _check(self, rc):
        if rc != L.OK:
            raise L.BhtsneError(rc, self.lib.bhtsne_tsne_last_error(self.handle).decode())
        return self

    def close(self):
        if getattr(self, "handle", None):
            self.lib.bhtsne_tsne_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- setters: src/lib.rs:277-435 -------------------------------------------
    def learning_rate(self, v):
        return self._check(self.lib.bhtsne_tsne_learning_rate(self.handle, float(v)))

    def epochs(self, v):
        return self._check(self.lib.bhtsne_tsne_epochs(self.handle, int(v)))

    def momentum(self, v):
        return self._check(self.lib.bhtsne_tsne_momentum(self.handle, float(v)))

    def final_momentum(self, v):
        return self._check(self.lib.bhtsne_tsne_final_momentum(self.handle, float(v)))

    def momentum_switch_epoch(self, v):
        return self._check(self.lib.bhtsne_tsne_momentum_switch_epoch(self.handle, int(v)))

    def stop_lying_epoch(self, v):
        return self._check(self.lib.bhtsne_tsne_stop_lying_epoch(self.handle, int(v)))

    def early_exaggeration(self, v):
        return self._check(self.lib.bhtsne_tsne_early_exaggeration(self.handle, float(v)))

    def perplexity(self, v):
        return self._check(self.lib.bhtsne_tsne_perplexity(self.handle, float(v)))

    def random_seed(self, seed: int):
        return self._check(self.lib.bhtsne_tsne_random_seed(self.handle, int(seed)))

    def initial_embedding(self, y):
        y = np.ascontiguousarray(np.asarray(y, dtype=self.dtype).ravel())
        return self._check(self.lib.bhtsne_tsne_initial_embedding(self.handle, _ptr(y), y.size))

    def epoch_callback(self, fn: Callable[[int, np.ndarray], None]):
        n, D, dt = self.n, self.D, self.dtype

        def tramp(epoch, yptr, user):
            buf = (C.c_char * (n * D * dt.itemsize)).from_address(yptr)
            fn(int(epoch), np.frombuffer(buf, dtype=dt).copy())

        self._cb = L.EPOCH_CB(tramp)
        return self._check(self.lib.bhtsne_tsne_epoch_callback(self.handle, C.cast(self._cb, C.c_void_p), None))

    # -- finishers --------------------------------------------------------------
    def _need_data(self):
        if self.data is None:
            raise L.BhtsneError(L.EINVAL, "error: this finisher needs the dataset given at construction.")
        return self.data

    def exact(self, metric="sqeuclidean"):
        """exact (src/lib.rs:489-646). metric: 'sqeuclidean', 'euclidean', or a
        dense (n, n) distance matrix (only its strict upper triangle is read)."""
        if isinstance(metric, str):
            X = self._need_data()
            sq = {"sqeuclidean": 1, "euclidean": 0}[metric]
            return self._check(self.lib.bhtsne_tsne_exact_euclidean(self.handle, _ptr(X), X.shape[1], sq))
        d = np.ascontiguousarray(np.asarray(metric, dtype=self.dtype))
        if d.shape != (self.n, self.n):
            raise L.BhtsneError(L.EINVAL, "error: the distance matrix must be n_samples x n_samples.")
        return self._check(self.lib.bhtsne_tsne_exact_distances(self.handle, _ptr(d)))

    def barnes_hut(self, theta, metric="euclidean"):
        """barnes_hut (src/lib.rs:701-742) with the Euclidean metric. With
        cached affinities (with_affinities or an earlier fit) the dataset is not
        read, as in the reference."""
        if metric != "euclidean":
            raise L.BhtsneError(L.EINVAL, "error: other metrics enter through barnes_hut_with_neighbors.")
        X = self.data
        return self._check(self.lib.bhtsne_tsne_barnes_hut_euclidean(
            self.handle, float(theta), _ptr(X), 0 if X is None else X.shape[1]))

    def barnes_hut_with_neighbors(self, theta, neighbors):
        """barnes_hut_with_neighbors (src/lib.rs:757-772)."""
        if not (float(theta) > 0):
            return self._check(self.lib.bhtsne_tsne_barnes_hut_with_neighbors(self.handle, float(theta), None, None,
                                                                              0, 0))
        idx, dist = neighbors_to_arrays(neighbors, self.dtype)
        return self._check(self.lib.bhtsne_tsne_barnes_hut_with_neighbors(self.handle, float(theta), _ptr(idx),
                                                                          _ptr(dist), idx.shape[0], idx.shape[1]))

    def fit_sne(self, metric="euclidean"):
        """fit_sne (src/lib.rs:835-871) with the Euclidean metric."""
        if metric != "euclidean":
            raise L.BhtsneError(L.EINVAL, "error: other metrics enter through fit_sne_with_neighbors.")
        X = self.data
        return self._check(self.lib.bhtsne_tsne_fit_sne_euclidean(self.handle, _ptr(X), 0 if X is None else X.shape[1]))

    def fit_sne_with_neighbors(self, neighbors):
        """fit_sne_with_neighbors (src/lib.rs:884-894)."""
        idx, dist = neighbors_to_arrays(neighbors, self.dtype)
        return self._check(self.lib.bhtsne_tsne_fit_sne_with_neighbors(self.handle, _ptr(idx), _ptr(dist),
                                                                       idx.shape[0], idx.shape[1]))

    def advance(self, epochs: int):
        """Continues the last fit for `epochs` more epochs (no reference counterpart)."""
        return self._check(self.lib.bhtsne_tsne_advance(self.handle, int(epochs)))

    # -- getters ------------------------------------------------------------------
    def embedding(self) -> np.ndarray:
        out = np.zeros(self.n * self.D, self.dtype)
        self._check(self.lib.bhtsne_tsne_embedding(self.handle, _ptr(out)))
        return out

    def embedding_into(self, out: np.ndarray) -> np.ndarray:
        """embedding() into a caller buffer (for instance page-locked memory)
        of n * D values of the handle's type."""
        if out.dtype != self.dtype or out.size != self.n * self.D or not out.flags.c_contiguous:
            raise L.BhtsneError(L.EINVAL, "error: the output buffer must hold n_samples * D contiguous values.")
        self._check(self.lib.bhtsne_tsne_embedding(self.handle, _ptr(out)))
        return out

    def kl_divergence(self, quirk: bool = True) -> Optional[float]:
        v = C.c_double()
        has = C.c_int32()
        self._check(self.lib.bhtsne_tsne_kl_divergence(self.handle, 1 if quirk else 0, C.byref(v), C.byref(has)))
        return v.value if has.value else None

    def affinities(self) -> Optional[SparseAffinities]:
        nnz = C.c_int64()
        perp = C.c_double()
        has = C.c_int32()
        self._check(self.lib.bhtsne_tsne_affinities(self.handle, None, None, None, C.byref(nnz), C.byref(perp),
                                                    C.byref(has)))
        if not has.value:
            return None
        rows = np.zeros(self.n + 1, np.uint64)
        cols = np.zeros(nnz.value, np.uint32)
        vals = np.zeros(nnz.value, self.dtype)
        self._check(self.lib.bhtsne_tsne_affinities(self.handle, _ptr(rows), _ptr(cols), _ptr(vals), C.byref(nnz),
                                                    C.byref(perp), C.byref(has)))
        return SparseAffinities(rows, cols, vals, perp.value)

    def with_affinities(self, aff: SparseAffinities):
        rows = np.ascontiguousarray(aff.rows, dtype=np.uint64)
        cols = np.ascontiguousarray(aff.columns, dtype=np.uint32)
        vals = np.ascontiguousarray(aff.values, dtype=self.dtype)
        return self._check(self.lib.bhtsne_tsne_with_affinities(self.handle, _ptr(rows), rows.size, _ptr(cols),
                                                                _ptr(vals), vals.size, float(aff.perplexity)))

    def write_csv(self, path: str):
        """write_csv (src/csv.rs:31-58): the embedding, one point per record,
        headers x,y (D = 2) or x,y,z (D = 3)."""
        return self._check(self.lib.bhtsne_tsne_write_csv(self.handle, os.fsencode(path)))

    def profile(self, enable: bool = True):
        """Per-phase CUDA-event timing of subsequent epochs (no reference counterpart)."""
        return self._check(self.lib.bhtsne_tsne_profile(self.handle, 1 if enable else 0))

    def phase_times(self):
        ms = (C.c_double * 4)()
        e = C.c_int64()
        self.lib.bhtsne_tsne_phase_times(self.handle, ms, C.byref(e))
        return {"tree": ms[0], "repulsion": ms[1], "attractive": ms[2], "update": ms[3], "epochs": e.value}

    def relayout_times(self):
        """Device ms and count of the locality re-layouts of the last finisher
        or advance call (no reference counterpart)."""
        ms, c = C.c_double(), C.c_int64()
        self._check(self.lib.bhtsne_tsne_relayout_times(self.handle, C.byref(ms), C.byref(c)))
        return {"ms": ms.value, "count": c.value}

    def layout_info(self):
        """The last fit's layout (no reference counterpart): whether the points
        were grouped by connected component of P, and P's largest component."""
        comp, big = C.c_int32(), C.c_int64()
        self._check(self.lib.bhtsne_tsne_layout_info(self.handle, C.byref(comp), C.byref(big)))
        return {"component_layout": bool(comp.value), "largest_component": big.value}

    def timings(self):
        a, lp, e = C.c_double(), C.c_double(), C.c_int64()
        self.lib.bhtsne_tsne_timings(self.handle, C.byref(a), C.byref(lp), C.byref(e))
        return {"affinity_ms": a.value, "loop_ms": lp.value, "loop_epochs": e.value}


# ---- stage entry points ---------------------------------------------------------
def knn_euclidean(X: np.ndarray, k: int, ctx: Optional[L.Context] = None):
    ctx = ctx or L.default_context()
    X = np.ascontiguousarray(X)
    n, d = X.shape
    idx = np.zeros((n, k), np.uint32)
    dist = np.zeros((n, k), X.dtype)
    ctx.check(ctx.lib.bhtsne_knn_euclidean(ctx.handle, _dtype_code(X.dtype), _ptr(X), n, d, int(k), _ptr(idx),
                                           _ptr(dist)))
    return idx, dist


def conditional_p(dist: np.ndarray, perplexity: float, ctx: Optional[L.Context] = None):
    ctx = ctx or L.default_context()
    dist = np.ascontiguousarray(dist)
    n, k = dist.shape
    p = np.zeros_like(dist)
    its = np.zeros(n, np.int32)
    ctx.check(ctx.lib.bhtsne_conditional_p(ctx.handle, _dtype_code(dist.dtype), _ptr(dist), n, k, float(perplexity),
                                           _ptr(p), _ptr(its)))
    return p, its


def symmetrize(cols: np.ndarray, p: np.ndarray, ctx: Optional[L.Context] = None):
    ctx = ctx or L.default_context()
    cols = np.ascontiguousarray(cols, dtype=np.uint32)
    p = np.ascontiguousarray(p)
    n, k = cols.shape
    nnz = C.c_int64()
    ctx.check(ctx.lib.bhtsne_symmetrize(ctx.handle, _dtype_code(p.dtype), _ptr(cols), _ptr(p), n, k, None, None, None,
                                        C.byref(nnz)))
    rows = np.zeros(n + 1, np.uint64)
    c = np.zeros(nnz.value, np.uint32)
    v = np.zeros(nnz.value, p.dtype)
    ctx.check(ctx.lib.bhtsne_symmetrize(ctx.handle, _dtype_code(p.dtype), _ptr(cols), _ptr(p), n, k, _ptr(rows),
                                        _ptr(c), _ptr(v), C.byref(nnz)))
    return rows, c, v


def gradient(method: int, y: np.ndarray, rows=None, cols=None, vals=None, theta: float = 0.5,
             ctx: Optional[L.Context] = None):
    """Attractive forces, repulsive forces and Z at a fixed embedding."""
    ctx = ctx or L.default_context()
    y = np.ascontiguousarray(y)
    n, D = y.shape
    pos = np.zeros_like(y)
    neg = np.zeros_like(y)
    z = C.c_double()
    vals = np.ascontiguousarray(vals, dtype=y.dtype)
    nnz = vals.size
    if rows is not None:
        rows = np.ascontiguousarray(rows, dtype=np.uint64)
        cols = np.ascontiguousarray(cols, dtype=np.uint32)
    ctx.check(ctx.lib.bhtsne_gradient(ctx.handle, _dtype_code(y.dtype), int(method), D, _ptr(y), n, _ptr(rows),
                                      _ptr(cols), _ptr(vals), nnz, float(theta), _ptr(pos), _ptr(neg), C.byref(z)))
    return pos, neg, z.value


def update(y, pos, neg, uy, gains, learning_rate, momentum, inverse_z, ctx: Optional[L.Context] = None):
    """gradient_descent_step + zero_mean on copies; returns (y, uy, gains)."""
    ctx = ctx or L.default_context()
    y = np.array(y, copy=True, order="C")
    uy = np.array(uy, copy=True, order="C")
    gains = np.array(gains, copy=True, order="C")
    pos = np.ascontiguousarray(pos, dtype=y.dtype)
    neg = None if neg is None else np.ascontiguousarray(neg, dtype=y.dtype)
    n, D = y.shape
    ctx.check(ctx.lib.bhtsne_update(ctx.handle, _dtype_code(y.dtype), D, _ptr(y), _ptr(pos), _ptr(neg), _ptr(uy),
                                    _ptr(gains), n, float(learning_rate), float(momentum), float(inverse_z)))
    return y, uy, gains


# ---- CSV input and output (src/csv.rs) -------------------------------------------
def load_csv(path: str, has_headers: bool = False, skip=None, dtype=np.float32) -> np.ndarray:
    """load_csv (src/csv.rs:61-118) for numeric fields: every field except the
    columns in `skip`, parsed as `dtype`, flattened in file order (the
    reference's Vec<T>)."""
    lib = L.load()
    code = _dtype_code(dtype)
    sk = np.ascontiguousarray(np.asarray(list(skip or []), dtype=np.int64))
    count, records = C.c_int64(0), C.c_int64(0)
    p = os.fsencode(path)
    rc = lib.bhtsne_load_csv(p, 1 if has_headers else 0, _ptr(sk) if sk.size else None, sk.size, code, None,
                             C.byref(count), C.byref(records))
    if rc != L.OK:
        raise L.BhtsneError(rc, lib.bhtsne_io_last_error().decode())
    out = np.zeros(count.value, np.dtype(dtype))
    rc = lib.bhtsne_load_csv(p, 1 if has_headers else 0, _ptr(sk) if sk.size else None, sk.size, code, _ptr(out),
                             C.byref(count), C.byref(records))
    if rc != L.OK:
        raise L.BhtsneError(rc, lib.bhtsne_io_last_error().decode())
    return out


def load_npz(path: str, name: str, dtype=np.float32) -> np.ndarray:
    """Array `name` of an .npz archive (the input format of the reference's
    example, examples/mnist_pca_tsne.rs:39-44) in C order, converted to
    `dtype`, with its shape."""
    lib = L.load()
    code = _dtype_code(dtype)
    count, ndim = C.c_int64(0), C.c_int32(0)
    shape = (C.c_int64 * 8)()
    p, nm = os.fsencode(path), name.encode()
    rc = lib.bhtsne_load_npz(p, nm, code, None, C.byref(count), C.byref(ndim), shape)
    if rc != L.OK:
        raise L.BhtsneError(rc, lib.bhtsne_io_last_error().decode())
    out = np.zeros(count.value, np.dtype(dtype))
    rc = lib.bhtsne_load_npz(p, nm, code, _ptr(out), C.byref(count), None, None)
    if rc != L.OK:
        raise L.BhtsneError(rc, lib.bhtsne_io_last_error().decode())
    if ndim.value > 8:
        return out
    return out.reshape(tuple(shape[k] for k in range(ndim.value)))


def write_csv(embedding: np.ndarray, path: str, D: int = 2):
    """write_csv of an embedding held by the caller (n x D values)."""
    lib = L.load()
    e = np.ascontiguousarray(embedding)
    rc = lib.bhtsne_write_csv(_ptr(e), e.size // D, D, _dtype_code(e.dtype), os.fsencode(path))
    if rc != L.OK:
        raise L.BhtsneError(rc, lib.bhtsne_io_last_error().decode())
