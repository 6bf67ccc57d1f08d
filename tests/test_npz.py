"""npz input through the C ABI, on the CPU: the archive format the reference's
example reads its data from (examples/mnist_pca_tsne.rs:39-44, through npyz's
NpzArchive::by_name + into_vec). Archives written by numpy (np.savez: stored
entries; np.savez_compressed: deflated entries), every supported element type,
Fortran order, 0-d to 3-d shapes, the fixture's own layout (float32 data of
shape (70000, 20) and uint8 labels, deflated), and the error paths."""
import io
import zipfile

import numpy as np
import pytest


@pytest.mark.parametrize("compressed", [False, True])
@pytest.mark.parametrize("dt", ["<f4", "<f8", "|i1", "<i2", "<i4", "<i8", "|u1", "<u2", "<u4", "<u8", "|b1"])
def test_load_npz_element_types(tmp_path, compressed, dt):
    from bhtsne_gb300 import load_npz
    rng = np.random.default_rng(3)
    if dt == "|b1":
        a = rng.random((37, 5)) > 0.5
    elif dt[1] == "f":
        a = rng.normal(0, 100, size=(37, 5)).astype(dt)
    else:
        info = np.iinfo(np.dtype(dt))
        a = rng.integers(max(info.min, -(2 ** 40)), min(info.max, 2 ** 40), size=(37, 5), endpoint=True).astype(dt)
    p = tmp_path / "a.npz"
    (np.savez_compressed if compressed else np.savez)(p, data=a, other=np.arange(3))
    for dtype in (np.float32, np.float64):
        v = load_npz(str(p), "data", dtype=dtype)
        assert v.dtype == dtype and v.shape == a.shape
        assert np.array_equal(v, a.astype(dtype))


def test_load_npz_fixture_layout(tmp_path):
    """The shapes and types of the reference's data/mnist_pca20.npz (float32
    (70000, 20) 'data', uint8 (70000,) 'labels', deflated), with synthetic
    values."""
    from bhtsne_gb300 import load_npz
    rng = np.random.default_rng(4)
    data = rng.uniform(-6.2, 9.4, size=(70000, 20)).astype(np.float32)
    labels = rng.integers(0, 10, size=70000).astype(np.uint8)
    p = tmp_path / "mnist_like.npz"
    np.savez_compressed(p, data=data, labels=labels)
    with zipfile.ZipFile(p) as z:
        assert all(i.compress_type == zipfile.ZIP_DEFLATED for i in z.infolist())
    v = load_npz(str(p), "data")
    assert v.shape == (70000, 20) and np.array_equal(v, data)
    lab = load_npz(str(p), "labels", dtype=np.float64)
    assert lab.shape == (70000,) and np.array_equal(lab, labels.astype(np.float64))


@pytest.mark.parametrize("shape", [(), (7,), (4, 6), (3, 4, 5)])
def test_load_npz_shapes_and_fortran_order(tmp_path, shape):
    from bhtsne_gb300 import load_npz
    a = np.arange(int(np.prod(shape)), dtype=np.float64).reshape(shape) * 1.5 - 3
    f = np.asfortranarray(a)
    p = tmp_path / "s.npz"
    np.savez(p, c=a, f=f)
    for name, ref in (("c", a), ("f", f)):  # (asfortranarray makes a 0-d array 1-d)
        v = load_npz(str(p), name, dtype=np.float64)
        assert v.shape == ref.shape and np.array_equal(v, ref)


def test_load_npz_deflate_block_kinds(tmp_path):
    """Deflate streams with stored, fixed-Huffman and dynamic-Huffman blocks
    (zlib levels 0, 1 and 9 on data of different entropy), long back
    references included."""
    from bhtsne_gb300 import load_npz
    rng = np.random.default_rng(5)
    arrays = {
        "random": rng.normal(size=4096).astype(np.float32),         # high entropy: dynamic or stored
        "repeats": np.tile(np.arange(16, dtype=np.float32), 4096),  # long matches
        "tiny": np.array([1.0, 2.0], np.float32),                   # fixed Huffman
    }
    for level in (0, 1, 9):
        p = tmp_path / f"l{level}.npz"
        with zipfile.ZipFile(p, "w", compression=zipfile.ZIP_DEFLATED, compresslevel=level) as z:
            for k, a in arrays.items():
                buf = io.BytesIO()
                np.save(buf, a)
                z.writestr(k + ".npy", buf.getvalue())
        for k, a in arrays.items():
            assert np.array_equal(load_npz(str(p), k), a)


def test_load_npz_zip64(tmp_path):
    """Entries written with ZIP64 records (zipfile's force_zip64)."""
    from bhtsne_gb300 import load_npz
    a = np.linspace(-1, 1, 1000, dtype=np.float32)
    p = tmp_path / "z64.npz"
    buf = io.BytesIO()
    np.save(buf, a)
    with zipfile.ZipFile(p, "w", compression=zipfile.ZIP_DEFLATED) as z:
        with z.open("x.npy", "w", force_zip64=True) as f:
            f.write(buf.getvalue())
    assert np.array_equal(load_npz(str(p), "x"), a)


def test_load_npz_errors(tmp_path):
    from bhtsne_gb300 import load_npz, _lib as L
    p = tmp_path / "a.npz"
    np.savez(p, data=np.zeros(3, np.float32), cplx=np.zeros(2, np.complex64),
             big=np.zeros(2, dtype=">f4"))
    with pytest.raises(L.BhtsneError) as e:
        load_npz(str(p), "missing")
    assert e.value.code == L.EINVAL and "no array 'missing'" in str(e.value)
    for name in ("cplx", "big"):
        with pytest.raises(L.BhtsneError) as e:
            load_npz(str(p), name)
        assert e.value.code == L.EINVAL and "unsupported .npy dtype" in str(e.value)
    with pytest.raises(L.BhtsneError) as e:
        load_npz(str(tmp_path / "nope.npz"), "data")
    assert e.value.code == L.EIO
    q = tmp_path / "not.npz"
    q.write_bytes(b"plain text, not a zip archive" * 10)
    with pytest.raises(L.BhtsneError) as e:
        load_npz(str(q), "data")
    assert e.value.code == L.EINVAL
    # a flipped byte inside a stored entry's data fails the CRC-32 check
    raw = bytearray(p.read_bytes())
    with zipfile.ZipFile(p) as z:
        info = z.getinfo("data.npy")
    hdr = info.header_offset
    name_len = int.from_bytes(raw[hdr + 26:hdr + 28], "little")
    extra_len = int.from_bytes(raw[hdr + 28:hdr + 30], "little")
    raw[hdr + 30 + name_len + extra_len + info.file_size - 1] ^= 0x40
    r = tmp_path / "bad.npz"
    r.write_bytes(bytes(raw))
    with pytest.raises(L.BhtsneError) as e:
        load_npz(str(r), "data")
    assert e.value.code == L.EINVAL and "CRC-32" in str(e.value)
