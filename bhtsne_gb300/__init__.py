"""bhtsne_gb300: t-SNE fitting (exact, Barnes-Hut, FIt-SNE) on one GB300 GPU.

A from-scratch sm_103a implementation of the fitting path of the Rust crate
bhtsne 0.7.10 behind a C ABI (include/bhtsne_gpu.h); this package is the
Python mirror of the reference's `tSNE` builder over that ABI.
"""
from ._lib import (BhtsneError, Context, F32, F64, METHOD_BARNES_HUT, METHOD_EXACT, METHOD_FIT_SNE, SIGNATURES,
                   default_context, library_path, load, tune_config, tune_load, tune_save)
from .batch import Batch
from .serve import Server
from .tsne import (Neighbor, SparseAffinities, TSNE, conditional_p, gradient, knn_euclidean, load_csv,
                   load_npz, neighbors_to_arrays, symmetrize, update, write_csv)

__all__ = [
    "Batch", "BhtsneError", "Server", "Context", "F32", "F64", "METHOD_BARNES_HUT", "METHOD_EXACT", "METHOD_FIT_SNE", "SIGNATURES",
    "default_context", "library_path", "load", "Neighbor", "SparseAffinities", "TSNE", "conditional_p", "gradient",
    "knn_euclidean", "load_csv", "load_npz", "neighbors_to_arrays", "symmetrize", "tune_config", "tune_load", "tune_save",
    "update", "write_csv",
]
