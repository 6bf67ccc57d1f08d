"""Many independent Barnes-Hut fits stepped together on one GPU.

Each job is what `TSNE(X).barnes_hut(theta)` (src/lib.rs:701-742) would fit on
its own: its own affinities, learning rate, tree, Z and mean. The jobs share
one launch per stage each epoch (the bhtsne_batch handle of the C ABI), so
thousands of small embeddings do not pay one launch sequence each. The
reference has no batch entry point: a caller there loops over `tSNE`
builders.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L
from .tsne import _dtype_code, neighbors_to_arrays

_FIELDS = [f for f, _ in L.BatchParams._fields_]


class Batch:
    """`Batch(D=2, dtype=np.float32, perplexity=30, epochs=500, ...)`; keyword
    arguments are the builder settings shared by every job (the fields of
    bhtsne_batch_params; `learning_rate` <= 0 means the reference's automatic
    max(n / exaggeration / 4, 50) per job)."""

    def __init__(self, D: int = 2, dtype=np.float32, ctx: Optional[L.Context] = None, **params):
        self.ctx = ctx or L.default_context()
        self.lib = self.ctx.lib
        self.dtype = np.dtype(dtype)
        self.D = int(D)
        p = L.BatchParams()
        self.lib.bhtsne_batch_params_default(C.byref(p))
        for k, v in params.items():
            if k not in _FIELDS:
                raise TypeError(f"unknown batch parameter {k!r}")
            setattr(p, k, v)
        self.params = p
        h = C.c_void_p()
        rc = self.lib.bhtsne_batch_new(self.ctx.handle, _dtype_code(self.dtype), self.D, C.byref(p), C.byref(h))
        if rc != L.OK:
            raise L.BhtsneError(rc, self.lib.bhtsne_ctx_last_error(self.ctx.handle).decode())
        self.handle = h
        self.sizes: list[int] = []

    def _check(self, rc):
        if rc != L.OK:
            raise L.BhtsneError(rc, self.lib.bhtsne_batch_last_error(self.handle).decode())
        return self

    def close(self):
        if getattr(self, "handle", None):
            self.lib.bhtsne_batch_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, data) -> int:
        """Adds a job from an (n, dim) array (device kNN, Euclidean)."""
        X = np.ascontiguousarray(np.asarray(data, dtype=self.dtype))
        if X.ndim == 1:
            X = X.reshape(-1, 1)
        j = C.c_int64(-1)
        self._check(self.lib.bhtsne_batch_add_euclidean(self.handle, X.ctypes.data, X.shape[0], X.shape[1],
                                                        C.byref(j)))
        self.sizes.append(X.shape[0])
        return j.value

    def add_with_neighbors(self, neighbors) -> int:
        """Adds a job from a kNN table ((indices, distances) or rows of Neighbor)."""
        idx, dist = neighbors_to_arrays(neighbors, self.dtype)
        j = C.c_int64(-1)
        self._check(self.lib.bhtsne_batch_add_with_neighbors(self.handle, idx.ctypes.data, dist.ctypes.data,
                                                             idx.shape[0], idx.shape[1], C.byref(j)))
        self.sizes.append(idx.shape[0])
        return j.value

    def initial_embedding(self, job: int, y) -> "Batch":
        y = np.ascontiguousarray(np.asarray(y, dtype=self.dtype).reshape(-1))
        if y.size != self.sizes[job] * self.D:
            raise L.BhtsneError(L.EINVAL, f"error: initial embedding has {y.size} values, expected "
                                          f"n_samples * D = {self.sizes[job] * self.D}")
        return self._check(self.lib.bhtsne_batch_initial_embedding(self.handle, int(job), y.ctypes.data))

    def fit(self) -> "Batch":
        return self._check(self.lib.bhtsne_batch_fit(self.handle))

    def __len__(self) -> int:
        return int(self.lib.bhtsne_batch_jobs(self.handle))

    def embedding(self, job: int) -> np.ndarray:
        out = np.empty(self.sizes[job] * self.D, dtype=self.dtype)
        self._check(self.lib.bhtsne_batch_embedding(self.handle, int(job), out.ctypes.data))
        return out

    def kl_divergence(self, job: int, quirk: bool = True) -> float:
        v = C.c_double(0)
        self._check(self.lib.bhtsne_batch_kl_divergence(self.handle, int(job), 1 if quirk else 0, C.byref(v)))
        return v.value

    def timings(self):
        a, b = C.c_double(0), C.c_double(0)
        self._check(self.lib.bhtsne_batch_timings(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value
