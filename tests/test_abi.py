"""The C ABI library builds, loads without a GPU, and exports exactly the
entry points declared in include/bhtsne_gpu.h. CPU only: no compute calls."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bhtsne_gpu.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bhtsne_[a-z0-9_]+)\s*\(", text)) - {"bhtsne_epoch_cb"})


def test_header_declares_the_builder_surface():
    syms = declared_symbols()
    for name in ["bhtsne_tsne_new", "bhtsne_tsne_barnes_hut_euclidean", "bhtsne_tsne_barnes_hut_with_neighbors",
                 "bhtsne_tsne_fit_sne_euclidean", "bhtsne_tsne_fit_sne_with_neighbors",
                 "bhtsne_tsne_exact_euclidean", "bhtsne_tsne_embedding", "bhtsne_tsne_kl_divergence",
                 "bhtsne_tsne_affinities", "bhtsne_tsne_with_affinities", "bhtsne_knn_euclidean"]:
        assert name in syms


def test_library_loads_and_exports_every_declared_symbol():
    from bhtsne_gb300 import _lib
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), f"{name} not exported"
    assert set(declared_symbols()) == set(_lib.SIGNATURES), "Python binding and header disagree"
    assert b"bhtsne" in lib.bhtsne_version()


def test_context_creation_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from bhtsne_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.bhtsne_ctx_create(0, ctypes.byref(h))
    assert rc != 0 and not h.value


def test_neighbor_table_shape_checks():
    import numpy as np

    from bhtsne_gb300 import BhtsneError, Neighbor, neighbors_to_arrays
    rows = [[Neighbor(1, 0.5), Neighbor(2, 0.7)], [Neighbor(0, 0.5), Neighbor(2, 0.9)], [Neighbor(0, 0.7)]]
    with pytest.raises(BhtsneError, match="same length"):
        neighbors_to_arrays(rows)
    with pytest.raises(BhtsneError, match="same length"):
        neighbors_to_arrays([[], []])
    idx, dist = neighbors_to_arrays(rows[:2] + [[Neighbor(0, 0.7), Neighbor(1, 0.9)]])
    assert idx.dtype == np.uint64 and idx.shape == (3, 2) and dist.dtype == np.float32


def _c_params(decl):
    """Parameter count of a C declaration's argument list."""
    inner = decl[decl.index("(") + 1:decl.rindex(")")].strip()
    return 0 if inner in ("", "void") else len(inner.split(","))


def test_rust_sys_crate_declares_every_header_function():
    """bindings/rust/bhtsne-gpu-sys/src/lib.rs (not compiled here: no cargo)
    declares every function of the header with the same number of parameters,
    and the three #[repr(C)] structs with the header's fields in order."""
    sys_rs = open(os.path.join(ROOT, "bindings", "rust", "bhtsne-gpu-sys", "src", "lib.rs")).read()
    header = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    decls = {m.group(1): m.group(0) for m in re.finditer(r"\b(bhtsne_[a-z0-9_]+)\s*\([^;]*\)\s*;", header)}
    decls.pop("bhtsne_epoch_cb", None)
    rust = {m.group(1): m.group(0) for m in re.finditer(r"pub fn (bhtsne_[a-z0-9_]+)\s*\((.*?)\)", sys_rs, flags=re.S)}
    assert set(decls) == set(rust), set(decls) ^ set(rust)
    for name, decl in decls.items():
        inner = rust[name][rust[name].index("(") + 1:-1].strip()
        n_rust = 0 if not inner else len([p for p in inner.split(",") if p.strip()])
        assert n_rust == _c_params(decl), name
    for struct in ("bhtsne_batch_params", "bhtsne_server_params", "bhtsne_request"):
        c_body = re.search(r"typedef struct %s \{(.*?)\}" % struct, header, flags=re.S).group(1)
        c_fields = re.findall(r"\b([a-z_]+)\s*;", c_body)
        r_body = re.search(r"pub struct %s \{(.*?)\}" % struct, sys_rs, flags=re.S).group(1)
        r_fields = re.findall(r"pub ([a-z_]+):", r_body)
        assert c_fields == r_fields, struct
