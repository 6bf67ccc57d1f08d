"""ctypes binding of libbhtsne_gpu.so (the C ABI in include/bhtsne_gpu.h).

The library is built in-tree (bhtsne_gb300/build.py). There is no fallback:
if the library cannot be built or loaded, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

OK, EIO, ENOMEM, EINVAL, ETIMEDOUT, ECUDA, EINTERNAL = 0, 5, 12, 22, 110, 1001, 1002
F32, F64 = 0, 1
METHOD_EXACT, METHOD_BARNES_HUT, METHOD_FIT_SNE = 1, 2, 3

EPOCH_CB = C.CFUNCTYPE(None, C.c_int64, C.c_void_p, C.c_void_p)

# Every symbol declared in include/bhtsne_gpu.h with its (restype, argtypes).
_vp, _i64, _i32, _dbl, _u64p, _u32p, _i32p, _i64p, _dblp = (
    C.c_void_p, C.c_int64, C.c_int32, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p)
SIGNATURES = {
    "bhtsne_version": (C.c_char_p, []),
    "bhtsne_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "bhtsne_ctx_destroy": (C.c_int, [_vp]),
    "bhtsne_ctx_last_error": (C.c_char_p, [_vp]),
    "bhtsne_ctx_knn_fallback_rows": (C.c_int, [_vp, _i64p]),
    "bhtsne_ctx_knn_brute_rows": (C.c_int, [_vp, _i64p]),
    "bhtsne_tsne_new": (C.c_int, [_vp, C.c_int, _i32, _i64, C.POINTER(C.c_void_p)]),
    "bhtsne_tsne_free": (C.c_int, [_vp]),
    "bhtsne_tsne_last_error": (C.c_char_p, [_vp]),
    "bhtsne_tsne_learning_rate": (C.c_int, [_vp, _dbl]),
    "bhtsne_tsne_epochs": (C.c_int, [_vp, _i64]),
    "bhtsne_tsne_momentum": (C.c_int, [_vp, _dbl]),
    "bhtsne_tsne_final_momentum": (C.c_int, [_vp, _dbl]),
    "bhtsne_tsne_momentum_switch_epoch": (C.c_int, [_vp, _i64]),
    "bhtsne_tsne_stop_lying_epoch": (C.c_int, [_vp, _i64]),
    "bhtsne_tsne_early_exaggeration": (C.c_int, [_vp, _dbl]),
    "bhtsne_tsne_perplexity": (C.c_int, [_vp, _dbl]),
    "bhtsne_tsne_epoch_callback": (C.c_int, [_vp, _vp, _vp]),
    "bhtsne_tsne_initial_embedding": (C.c_int, [_vp, _vp, _i64]),
    "bhtsne_tsne_random_seed": (C.c_int, [_vp, C.c_uint64]),
    "bhtsne_tsne_exact_euclidean": (C.c_int, [_vp, _vp, _i32, _i32]),
    "bhtsne_tsne_exact_distances": (C.c_int, [_vp, _vp]),
    "bhtsne_tsne_barnes_hut_euclidean": (C.c_int, [_vp, _dbl, _vp, _i32]),
    "bhtsne_tsne_barnes_hut_with_neighbors": (C.c_int, [_vp, _dbl, _u64p, _vp, _i64, _i64]),
    "bhtsne_tsne_fit_sne_euclidean": (C.c_int, [_vp, _vp, _i32]),
    "bhtsne_tsne_fit_sne_with_neighbors": (C.c_int, [_vp, _u64p, _vp, _i64, _i64]),
    "bhtsne_tsne_embedding": (C.c_int, [_vp, _vp]),
    "bhtsne_tsne_kl_divergence": (C.c_int, [_vp, _i32, _dblp, _i32p]),
    "bhtsne_tsne_affinities": (C.c_int, [_vp, _u64p, _u32p, _vp, _i64p, _dblp, _i32p]),
    "bhtsne_tsne_with_affinities": (C.c_int, [_vp, _u64p, _i64, _u32p, _vp, _i64, _dbl]),
    "bhtsne_tsne_advance": (C.c_int, [_vp, _i64]),
    "bhtsne_tsne_timings": (C.c_int, [_vp, _dblp, _dblp, _i64p]),
    "bhtsne_tsne_profile": (C.c_int, [_vp, _i32]),
    "bhtsne_tsne_phase_times": (C.c_int, [_vp, _dblp, _i64p]),
    "bhtsne_tsne_relayout_times": (C.c_int, [_vp, _dblp, _i64p]),
    "bhtsne_tsne_layout_info": (C.c_int, [_vp, C.POINTER(_i32), _i64p]),
    "bhtsne_launch_count": (C.c_int64, []),
    "bhtsne_knn_euclidean": (C.c_int, [_vp, C.c_int, _vp, _i64, _i32, _i32, _u32p, _vp]),
    "bhtsne_conditional_p": (C.c_int, [_vp, C.c_int, _vp, _i64, _i32, _dbl, _vp, _i32p]),
    "bhtsne_symmetrize": (C.c_int, [_vp, C.c_int, _u32p, _vp, _i64, _i32, _u64p, _u32p, _vp, _i64p]),
    "bhtsne_gradient": (C.c_int, [_vp, C.c_int, _i32, _i32, _vp, _i64, _u64p, _u32p, _vp, _i64, _dbl, _vp, _vp,
                                  _dblp]),
    "bhtsne_update": (C.c_int, [_vp, C.c_int, _i32, _vp, _vp, _vp, _vp, _vp, _i64, _dbl, _dbl, _dbl]),
    "bhtsne_load_csv": (C.c_int, [C.c_char_p, _i32, _i64p, _i64, C.c_int, _vp, _i64p, _i64p]),
    "bhtsne_tsne_write_csv": (C.c_int, [_vp, C.c_char_p]),
    "bhtsne_write_csv": (C.c_int, [_vp, _i64, _i32, C.c_int, C.c_char_p]),
    "bhtsne_load_npz": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, _vp, _i64p, C.POINTER(_i32), _i64p]),
    "bhtsne_io_last_error": (C.c_char_p, []),
    "bhtsne_tune": (C.c_int, [_vp, C.c_int, _i32, _i64, _i32, _i32]),
    "bhtsne_tune_config": (C.c_int, [C.c_int, _i32, _i64, C.c_char_p, _i64]),
    "bhtsne_tune_load": (C.c_int, [C.c_char_p]),
    "bhtsne_tune_save": (C.c_int, [C.c_char_p]),
    "bhtsne_bh_repulsion_noalloc": (C.c_int, [_vp, _i64, _dbl, _vp, _vp, _vp]),
    "bhtsne_batch_params_default": (None, [_vp]),
    "bhtsne_batch_new": (C.c_int, [_vp, C.c_int, _i32, _vp, C.POINTER(C.c_void_p)]),
    "bhtsne_batch_free": (C.c_int, [_vp]),
    "bhtsne_batch_last_error": (C.c_char_p, [_vp]),
    "bhtsne_batch_add_euclidean": (C.c_int, [_vp, _vp, _i64, _i32, _i64p]),
    "bhtsne_batch_add_with_neighbors": (C.c_int, [_vp, _u64p, _vp, _i64, _i64, _i64p]),
    "bhtsne_batch_initial_embedding": (C.c_int, [_vp, _i64, _vp]),
    "bhtsne_batch_fit": (C.c_int, [_vp]),
    "bhtsne_batch_jobs": (C.c_int64, [_vp]),
    "bhtsne_batch_embedding": (C.c_int, [_vp, _i64, _vp]),
    "bhtsne_batch_kl_divergence": (C.c_int, [_vp, _i64, _i32, _dblp]),
    "bhtsne_batch_timings": (C.c_int, [_vp, _dblp, _dblp]),
    "bhtsne_server_params_default": (None, [_vp]),
    "bhtsne_server_new": (C.c_int, [_vp, C.c_int, _i32, _vp, C.POINTER(C.c_void_p)]),
    "bhtsne_server_free": (C.c_int, [_vp]),
    "bhtsne_server_last_error": (C.c_char_p, [_vp]),
    "bhtsne_server_submit": (C.c_int, [_vp, _vp, _i64p]),
    "bhtsne_server_poll": (C.c_int, [_vp, _i64, _i32p]),
    "bhtsne_server_wait": (C.c_int, [_vp, _i64, _dbl]),
    "bhtsne_server_result": (C.c_int, [_vp, _i64, _vp, _dblp, _dblp]),
    "bhtsne_server_stats": (C.c_int, [_vp, _i64p, _i64p, _i64p, _dblp]),
    "bhtsne_server_timings": (C.c_int, [_vp, _dblp, _dblp, _dblp, _dblp]),
}

JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class ServerParams(C.Structure):
    """Mirror of struct bhtsne_server_params."""
    _fields_ = [
        ("perplexity", C.c_double),
        ("theta", C.c_double),
        ("hbm_budget_bytes", C.c_int64),
        ("round_epochs", C.c_int32),
        ("fit_workers", C.c_int32),
    ]


class Request(C.Structure):
    """Mirror of struct bhtsne_request."""
    _fields_ = [
        ("data", C.c_void_p),
        ("n", C.c_int64),
        ("dim", C.c_int32),
        ("method", C.c_int32),
        ("epochs", C.c_int64),
        ("seed", C.c_uint64),
        ("want_kl", C.c_int32),
    ]


class BatchParams(C.Structure):
    """Mirror of struct bhtsne_batch_params."""
    _fields_ = [
        ("perplexity", C.c_double),
        ("epochs", C.c_int64),
        ("learning_rate", C.c_double),
        ("momentum", C.c_double),
        ("final_momentum", C.c_double),
        ("momentum_switch_epoch", C.c_int64),
        ("stop_lying_epoch", C.c_int64),
        ("early_exaggeration", C.c_double),
        ("theta", C.c_double),
        ("seed", C.c_uint64),
    ]

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_needed: bool = True):
    """Loads (building first if needed) the CUDA library. Raises on failure."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build() if build_if_needed else _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(f"libbhtsne_gpu.so is missing at {path}; run bhtsne_gb300/build.py")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return _lib


class BhtsneError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class Context:
    """One CUDA device and stream (bhtsne_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.bhtsne_ctx_create(int(device), C.byref(h))
        if rc != OK:
            raise BhtsneError(rc, f"bhtsne_ctx_create failed with status {rc} (is a CUDA device visible?)")
        self.handle = h
        self.device = device

    def check(self, rc: int) -> None:
        if rc != OK:
            raise BhtsneError(rc, self.lib.bhtsne_ctx_last_error(self.handle).decode())

    def tune(self, dtype: int, embed_dim: int, n: int, k: int, dim: int = 0) -> str:
        """Autotunes the launch shapes for fits of that shape on this device
        (bhtsne_tune); returns the candidates' timings."""
        self.check(self.lib.bhtsne_tune(self.handle, int(dtype), int(embed_dim), int(n), int(k), int(dim)))
        return self.lib.bhtsne_ctx_last_error(self.handle).decode()

    def knn_fallback_rows(self) -> int:
        """Rows of the last Euclidean kNN on this context that failed the
        candidate pass's exactness certificate and were recomputed."""
        v = C.c_int64()
        self.check(self.lib.bhtsne_ctx_knn_fallback_rows(self.handle, C.byref(v)))
        return v.value

    def knn_brute_rows(self) -> int:
        """Of those, the rows recomputed by exact brute force."""
        v = C.c_int64()
        self.check(self.lib.bhtsne_ctx_knn_brute_rows(self.handle, C.byref(v)))
        return v.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.bhtsne_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def tune_config(dtype: int, embed_dim: int, n: int) -> dict:
    """The launch shapes a fit of (dtype, embed_dim, n) would use on the current device."""
    import json
    lib = load()
    buf = C.create_string_buffer(1024)
    rc = lib.bhtsne_tune_config(int(dtype), int(embed_dim), int(n), buf, len(buf))
    if rc != OK:
        raise BhtsneError(rc, lib.bhtsne_io_last_error().decode())
    return json.loads(buf.value.decode())


def tune_load(path: str) -> None:
    lib = load()
    rc = lib.bhtsne_tune_load(os.fsencode(path))
    if rc != OK:
        raise BhtsneError(rc, lib.bhtsne_io_last_error().decode())


def tune_save(path: str) -> None:
    lib = load()
    rc = lib.bhtsne_tune_save(os.fsencode(path))
    if rc != OK:
        raise BhtsneError(rc, lib.bhtsne_io_last_error().decode())
