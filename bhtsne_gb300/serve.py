"""Serving: embedding requests fitted concurrently on one GPU (bhtsne_server).

Requests are admitted in order while their estimated device footprint fits
the server's byte budget; Barnes-Hut requests join one running batch (each
with its own epoch count), FIt-SNE requests run on worker streams. Every
request uses the reference's optimiser defaults (src/lib.rs:241-266) with the
server's perplexity and theta. The reference has no server: a caller there
fits one `tSNE` builder after another.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L
from .tsne import _dtype_code

_STATES = {L.JOB_QUEUED: "queued", L.JOB_RUNNING: "running", L.JOB_DONE: "done", L.JOB_FAILED: "failed"}
_METHODS = {"bh": L.METHOD_BARNES_HUT, "barnes_hut": L.METHOD_BARNES_HUT, "fit": L.METHOD_FIT_SNE,
            "fit_sne": L.METHOD_FIT_SNE}


class Server:
    """`Server(D=2, dtype=np.float32, perplexity=30, theta=0.5, hbm_budget_bytes=0,
    round_epochs=25, fit_workers=2)`."""

    def __init__(self, D: int = 2, dtype=np.float32, ctx: Optional[L.Context] = None, **params):
        self.ctx = ctx or L.default_context()
        self.lib = self.ctx.lib
        self.dtype = np.dtype(dtype)
        self.D = int(D)
        p = L.ServerParams()
        self.lib.bhtsne_server_params_default(C.byref(p))
        names = [f for f, _ in L.ServerParams._fields_]
        for k, v in params.items():
            if k not in names:
                raise TypeError(f"unknown server parameter {k!r}")
            setattr(p, k, v)
        h = C.c_void_p()
        rc = self.lib.bhtsne_server_new(self.ctx.handle, _dtype_code(self.dtype), self.D, C.byref(p), C.byref(h))
        if rc != L.OK:
            raise L.BhtsneError(rc, "bhtsne_server_new failed (invalid parameters or no device)")
        self.handle = h
        self.sizes: dict[int, int] = {}

    def _check(self, rc):
        if rc != L.OK:
            raise L.BhtsneError(rc, self.lib.bhtsne_server_last_error(self.handle).decode())

    def close(self):
        if getattr(self, "handle", None):
            self.lib.bhtsne_server_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, data, method: str = "bh", epochs: int = 750, seed: int = 0, want_kl: bool = True) -> int:
        X = np.ascontiguousarray(np.asarray(data, dtype=self.dtype))
        if X.ndim == 1:
            X = X.reshape(-1, 1)
        r = L.Request(X.ctypes.data, X.shape[0], X.shape[1], _METHODS[method], int(epochs), int(seed),
                      1 if want_kl else 0)
        i = C.c_int64(-1)
        self._check(self.lib.bhtsne_server_submit(self.handle, C.byref(r), C.byref(i)))
        self.sizes[i.value] = X.shape[0]
        return i.value

    def poll(self, job: int) -> str:
        st = C.c_int32(-1)
        self._check(self.lib.bhtsne_server_poll(self.handle, int(job), C.byref(st)))
        return _STATES[st.value]

    def wait(self, job: int, timeout: Optional[float] = None) -> bool:
        rc = self.lib.bhtsne_server_wait(self.handle, int(job), -1.0 if timeout is None else float(timeout))
        if rc == L.ETIMEDOUT:
            return False
        self._check(rc)
        return True

    def result(self, job: int):
        """(embedding (n, D), KL or nan, submit-to-done latency in ms); forgets the job."""
        n = self.sizes.pop(int(job), None)
        if n is None:
            raise L.BhtsneError(L.EINVAL, "error: no request with that id.")
        out = np.empty(n * self.D, dtype=self.dtype)
        kl, lat = C.c_double(np.nan), C.c_double(0)
        self._check(self.lib.bhtsne_server_result(self.handle, int(job), out.ctypes.data, C.byref(kl), C.byref(lat)))
        return out.reshape(n, self.D), kl.value, lat.value

    def stats(self):
        d, f, p, m = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        self._check(self.lib.bhtsne_server_stats(self.handle, C.byref(d), C.byref(f), C.byref(p), C.byref(m)))
        a, b, c, e = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        self._check(self.lib.bhtsne_server_timings(self.handle, C.byref(a), C.byref(b), C.byref(c), C.byref(e)))
        return {"done": d.value, "in_flight": f.value, "peak_bytes": p.value, "mean_batch_points": m.value,
                "round_s": a.value, "repack_s": b.value, "prepare_s": c.value, "fit_worker_s": e.value}
