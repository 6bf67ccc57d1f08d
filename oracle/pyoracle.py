"""ctypes driver for the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py for the CPU baseline. The product package never
imports this module.

The oracle restates the bhtsne 0.7.10 fitting path in C++ (see
bhtsne_oracle.cpp for the reference file:line of each routine).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bhtsne_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")

FIT_EXACT, FIT_BH, FIT_INTERP = 1, 2, 3


def build(force: bool = False) -> str:
    """Compile liboracle.so next to its source (g++, OpenMP, no FMA contraction)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           SRC, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i64, i32, u64p, u32p, dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_double
        sig = {
            "orc_num_threads": (C.c_int, []),
            "orc_set_threads": (None, [C.c_int]),
            "orc_knn": (None, [C.c_int, vp, i64, i32, i32, u32p, vp]),
            "orc_knn_rows": (None, [C.c_int, vp, i64, i32, i32, vp, i64, u32p, vp]),
            "orc_search_beta": (C.c_int, [C.c_int, vp, i64, i32, dbl, vp, vp]),
            "orc_symmetrize": (i64, [C.c_int, u32p, vp, i64, i32, u64p, u32p, vp]),
            "orc_normalize": (None, [C.c_int, vp, i64, dbl]),
            "orc_edge_forces": (C.c_int, [C.c_int, i32, vp, i64, u64p, u32p, vp, vp]),
            "orc_bh_repulsion": (C.c_int, [C.c_int, i32, vp, i64, dbl, vp, vp, C.POINTER(C.c_double)]),
            "orc_bh_interactions": (C.c_int, [C.c_int, i32, vp, i64, dbl, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
            "orc_bh_tree": (i64, [C.c_int, i32, vp, i64, vp, vp, vp, vp, vp, vp, vp]),
            "orc_fit_repulsion": (C.c_int, [C.c_int, i32, vp, i64, vp, C.POINTER(C.c_double), vp]),
            "orc_gradient_step": (None, [C.c_int, vp, vp, vp, vp, vp, i64, dbl, dbl, dbl]),
            "orc_zero_mean": (None, [C.c_int, vp, i64, i32]),
            "orc_exact_affinities": (C.c_int, [C.c_int, vp, i64, dbl, vp]),
            "orc_exact_gradient": (dbl, [C.c_int, i32, vp, vp, i64, vp]),
            "orc_sparse_kl": (dbl, [C.c_int, i32, u64p, u32p, vp, vp, i64, dbl, C.c_int]),
            "orc_morton": (C.c_int, [i32, vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
            "orc_morton2": (C.c_uint64, [C.c_uint32, C.c_uint32]),
            "orc_morton3": (C.c_uint64, [C.c_uint32, C.c_uint32, C.c_uint32]),
            "orc_quantize_f32": (C.c_uint32, [C.c_float, C.c_float, C.c_float, C.c_uint32]),
            "orc_next_smooth": (i64, [i64]),
            "orc_fft_f64": (None, [vp, vp, i32, i32, i32]),
            "orc_lagrange_weights": (None, [dbl, vp]),
            "orc_tsne_new": (vp, [C.c_int, i32, i64]),
            "orc_tsne_free": (None, [vp]),
            "orc_tsne_last_error": (C.c_char_p, [vp]),
            "orc_tsne_set": (C.c_int, [vp, C.c_char_p, dbl]),
            "orc_tsne_get": (dbl, [vp, C.c_char_p]),
            "orc_tsne_set_initial_embedding": (None, [vp, vp, i64]),
            "orc_tsne_set_epoch_callback": (None, [vp, vp, vp]),
            "orc_tsne_fit_euclidean": (C.c_int, [vp, C.c_int, dbl, vp, i32]),
            "orc_tsne_fit_with_neighbors": (C.c_int, [vp, C.c_int, dbl, u64p, vp, i64, i64]),
            "orc_tsne_exact": (C.c_int, [vp, vp]),
            "orc_tsne_embedding": (None, [vp, vp]),
            "orc_tsne_kl": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double)]),
            "orc_tsne_affinities": (i64, [vp, u64p, u32p, vp, C.POINTER(C.c_double)]),
            "orc_tsne_with_affinities": (None, [vp, u64p, i64, u32p, vp, i64, dbl]),
            "orc_tsne_p_values": (i64, [vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dt(a: np.ndarray) -> int:
    return 0 if a.dtype == np.float32 else 1


def _p(a):
    return None if a is None else a.ctypes.data


def set_threads(t: int) -> None:
    lib().orc_set_threads(int(t))


def num_threads() -> int:
    return lib().orc_num_threads()


def knn(X: np.ndarray, k: int):
    X = np.ascontiguousarray(X)
    n, d = X.shape
    idx = np.empty((n, k), np.uint32)
    dist = np.empty((n, k), X.dtype)
    lib().orc_knn(_dt(X), _p(X), n, d, k, _p(idx), _p(dist))
    return idx, dist


def knn_rows(X: np.ndarray, k: int, rows):
    """Brute-force neighbours of the listed query rows over all n points."""
    X = np.ascontiguousarray(X)
    n, d = X.shape
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    idx = np.empty((rows.size, k), np.uint32)
    dist = np.empty((rows.size, k), X.dtype)
    lib().orc_knn_rows(_dt(X), _p(X), n, d, k, _p(rows), rows.size, _p(idx), _p(dist))
    return idx, dist


def search_beta(dist: np.ndarray, perplexity: float):
    dist = np.ascontiguousarray(dist)
    n, k = dist.shape
    p = np.empty_like(dist)
    its = np.empty(n, np.int32)
    lib().orc_search_beta(_dt(dist), _p(dist), n, k, float(perplexity), _p(p), _p(its))
    return p, its


def symmetrize(cols: np.ndarray, p: np.ndarray):
    cols = np.ascontiguousarray(cols, dtype=np.uint32)
    p = np.ascontiguousarray(p)
    n, k = cols.shape
    nnz = lib().orc_symmetrize(_dt(p), _p(cols), _p(p), n, k, None, None, None)
    rows = np.empty(n + 1, np.uint64)
    c = np.empty(nnz, np.uint32)
    v = np.empty(nnz, p.dtype)
    lib().orc_symmetrize(_dt(p), _p(cols), _p(p), n, k, _p(rows), _p(c), _p(v))
    return rows, c, v


def normalize(vals: np.ndarray, exaggeration: float) -> np.ndarray:
    v = np.array(vals, copy=True)
    lib().orc_normalize(_dt(v), _p(v), v.size, float(exaggeration))
    return v


def edge_forces(y, rows, cols, vals):
    y = np.ascontiguousarray(y)
    n, D = y.shape
    pos = np.zeros_like(y)
    rc = lib().orc_edge_forces(_dt(y), D, _p(y), n, _p(rows), _p(cols), _p(vals), _p(pos))
    assert rc == 0
    return pos


def bh_repulsion(y, theta):
    y = np.ascontiguousarray(y)
    n, D = y.shape
    neg = np.zeros_like(y)
    q = np.zeros(n, y.dtype)
    z = C.c_double()
    rc = lib().orc_bh_repulsion(_dt(y), D, _p(y), n, float(theta), _p(neg), _p(q), C.byref(z))
    assert rc == 0
    return neg, q, z.value


def bh_interactions(y, theta):
    """Theta tests and accepted cells of one Barnes-Hut repulsion pass at y."""
    y = np.ascontiguousarray(y)
    n, D = y.shape
    vis, inter = C.c_int64(), C.c_int64()
    rc = lib().orc_bh_interactions(_dt(y), D, _p(y), n, float(theta), C.byref(vis), C.byref(inter))
    assert rc == 0
    return vis.value, inter.value


def bh_tree(y):
    y = np.ascontiguousarray(y)
    n, D = y.shape
    L = lib()
    nn = L.orc_bh_tree(_dt(y), D, _p(y), n, None, None, None, None, None, None, None)
    com = np.zeros((max(nn, 0), D), y.dtype)
    count = np.zeros(max(nn, 0), np.uint32)
    level = np.zeros(max(nn, 0), np.uint8)
    first = np.zeros(max(nn, 0), np.uint32)
    cc = np.zeros(max(nn, 0), np.uint8)
    rs = np.zeros(max(nn, 0), np.uint32)
    re = np.zeros(max(nn, 0), np.uint32)
    L.orc_bh_tree(_dt(y), D, _p(y), n, _p(com), _p(count), _p(level), _p(first), _p(cc), _p(rs), _p(re))
    return dict(com=com, count=count, level=level, first_child=first, child_count=cc,
                range_start=rs, range_end=re)


def fit_repulsion(y):
    y = np.ascontiguousarray(y)
    n, D = y.shape
    neg = np.zeros_like(y)
    z = C.c_double()
    grid = np.zeros(6, np.float64)
    rc = lib().orc_fit_repulsion(_dt(y), D, _p(y), n, _p(neg), C.byref(z), _p(grid))
    assert rc == 0
    info = dict(boxes=int(grid[0]), nodes=int(grid[1]), fft_len=int(grid[2]), min=grid[3],
                box_width=grid[4], spacing=grid[5])
    return neg, z.value, info


def gradient_step(y, pos, neg, uy, gains, lr, momentum, inv_norm):
    """In-place fused update on copies; returns (y, uy, gains)."""
    y = np.array(y, copy=True)
    uy = np.array(uy, copy=True)
    gains = np.array(gains, copy=True)
    lib().orc_gradient_step(_dt(y), _p(y), _p(np.ascontiguousarray(pos)), _p(np.ascontiguousarray(neg)),
                            _p(uy), _p(gains), y.size, float(lr), float(momentum), float(inv_norm))
    return y, uy, gains


def zero_mean(y):
    y = np.array(y, copy=True)
    n, D = y.shape
    lib().orc_zero_mean(_dt(y), _p(y), n, D)
    return y


def exact_affinities(dist_matrix, perplexity):
    """The exact method's joint P before normalisation: search_beta over each
    full row of the mirrored distance matrix (diagonal included), then
    p_ij + p_ji on both sides."""
    d = np.ascontiguousarray(dist_matrix)
    n = d.shape[0]
    p = np.zeros_like(d)
    lib().orc_exact_affinities(_dt(d), _p(d), n, float(perplexity), _p(p))
    return p


def exact_gradient(p, y):
    """One exact gradient dy at a fixed y and dense P; returns (dy, Z)."""
    y = np.ascontiguousarray(y)
    p = np.ascontiguousarray(p, dtype=y.dtype)
    n, D = y.shape
    dy = np.zeros_like(y)
    z = lib().orc_exact_gradient(_dt(y), D, _p(p), _p(y), n, _p(dy))
    return dy, z


def sparse_kl(rows, cols, vals, y, inv_q_sum, quirk=True):
    y = np.ascontiguousarray(y)
    n, D = y.shape
    return lib().orc_sparse_kl(_dt(y), D, _p(rows), _p(cols), _p(vals), _p(y), n, float(inv_q_sum),
                               1 if quirk else 0)


def morton(coords):
    """Morton code of D = len(coords) quantised coordinates (D = 2..7) as an int."""
    c = np.ascontiguousarray(coords, dtype=np.uint32)
    lo, hi = C.c_uint64(), C.c_uint64()
    rc = lib().orc_morton(len(c), _p(c), C.byref(lo), C.byref(hi))
    assert rc == 0
    return (hi.value << 64) | lo.value


def morton2(a, b):
    return lib().orc_morton2(a, b)


def morton3(a, b, c):
    return lib().orc_morton3(a, b, c)


def next_smooth(n):
    return lib().orc_next_smooth(n)


def fft(re, im, inverse=False):
    re = np.array(re, dtype=np.float64, copy=True)
    im = np.array(im, dtype=np.float64, copy=True)
    dims = re.ndim
    lib().orc_fft_f64(_p(re), _p(im), re.shape[0], dims, 1 if inverse else 0)
    return re, im


def lagrange_weights(local):
    out = np.zeros(3, np.float64)
    lib().orc_lagrange_weights(float(local), _p(out))
    return out


EPOCH_CB = C.CFUNCTYPE(None, C.c_int64, C.c_void_p, C.c_void_p)


class TSNE:
    """The oracle's mirror of the reference builder (src/lib.rs:149-1249)."""

    def __init__(self, n: int, D: int = 2, dtype=np.float32):
        self.n, self.D, self.dtype = n, D, np.dtype(dtype)
        self._h = lib().orc_tsne_new(0 if self.dtype == np.float32 else 1, D, n)
        self._cb = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_tsne_free(h)
            self._h = None

    def _set(self, what, v):
        rc = lib().orc_tsne_set(self._h, what.encode(), float(v))
        assert rc == 0, what
        return self

    def learning_rate(self, v): return self._set("learning_rate", v)
    def epochs(self, v): return self._set("epochs", v)
    def momentum(self, v): return self._set("momentum", v)
    def final_momentum(self, v): return self._set("final_momentum", v)
    def momentum_switch_epoch(self, v): return self._set("momentum_switch_epoch", v)
    def stop_lying_epoch(self, v): return self._set("stop_lying_epoch", v)
    def early_exaggeration(self, v): return self._set("early_exaggeration", v)
    def perplexity(self, v): return self._set("perplexity", v)
    def seed(self, v): return self._set("seed", v)

    def get(self, what):
        return lib().orc_tsne_get(self._h, what.encode())

    def initial_embedding(self, y):
        y = np.ascontiguousarray(np.asarray(y, dtype=self.dtype).ravel())
        lib().orc_tsne_set_initial_embedding(self._h, _p(y), y.size)
        return self

    def epoch_callback(self, fn):
        n, D, dt = self.n, self.D, self.dtype

        def tramp(epoch, yptr, user):
            buf = (C.c_char * (n * D * dt.itemsize)).from_address(yptr)
            fn(int(epoch), np.frombuffer(buf, dtype=dt).copy())

        self._cb = EPOCH_CB(tramp)
        lib().orc_tsne_set_epoch_callback(self._h, C.cast(self._cb, C.c_void_p), None)
        return self

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(lib().orc_tsne_last_error(self._h).decode())
        return self

    def barnes_hut(self, theta, X):
        X = np.ascontiguousarray(X, dtype=self.dtype)
        return self._check(lib().orc_tsne_fit_euclidean(self._h, FIT_BH, float(theta), _p(X), X.shape[1]))

    def fit_sne(self, X):
        X = np.ascontiguousarray(X, dtype=self.dtype)
        return self._check(lib().orc_tsne_fit_euclidean(self._h, FIT_INTERP, 0.0, _p(X), X.shape[1]))

    def _with_neighbors(self, method, theta, idx, dist):
        idx = np.ascontiguousarray(idx, dtype=np.uint64)
        dist = np.ascontiguousarray(dist, dtype=self.dtype)
        rows, k = idx.shape
        return self._check(lib().orc_tsne_fit_with_neighbors(self._h, method, float(theta), _p(idx),
                                                             _p(dist), rows, k))

    def barnes_hut_with_neighbors(self, theta, idx, dist):
        return self._with_neighbors(FIT_BH, theta, idx, dist)

    def fit_sne_with_neighbors(self, idx, dist):
        return self._with_neighbors(FIT_INTERP, 0.0, idx, dist)

    def exact(self, dist_matrix):
        d = np.ascontiguousarray(dist_matrix, dtype=self.dtype)
        return self._check(lib().orc_tsne_exact(self._h, _p(d)))

    def embedding(self):
        out = np.zeros(self.n * self.D, self.dtype)
        lib().orc_tsne_embedding(self._h, _p(out))
        return out

    def kl_divergence(self, quirk=True):
        v = C.c_double()
        has = lib().orc_tsne_kl(self._h, 1 if quirk else 0, C.byref(v))
        return v.value if has else None

    def affinities(self):
        pp = C.c_double()
        nnz = lib().orc_tsne_affinities(self._h, None, None, None, C.byref(pp))
        if nnz < 0:
            return None
        rows = np.zeros(self.n + 1, np.uint64)
        cols = np.zeros(nnz, np.uint32)
        vals = np.zeros(nnz, self.dtype)
        lib().orc_tsne_affinities(self._h, _p(rows), _p(cols), _p(vals), C.byref(pp))
        return rows, cols, vals, pp.value

    def with_affinities(self, rows, cols, vals, perplexity):
        rows = np.ascontiguousarray(rows, dtype=np.uint64)
        cols = np.ascontiguousarray(cols, dtype=np.uint32)
        vals = np.ascontiguousarray(vals, dtype=self.dtype)
        lib().orc_tsne_with_affinities(self._h, _p(rows), rows.size, _p(cols), _p(vals), vals.size,
                                       float(perplexity))
        return self

    def p_values(self):
        nnz = lib().orc_tsne_p_values(self._h, None)
        v = np.zeros(nnz, self.dtype)
        lib().orc_tsne_p_values(self._h, _p(v))
        return v
