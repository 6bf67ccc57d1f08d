"""CSV input and output (src/csv.rs:31-118) through the C ABI, on the CPU:
load_csv with and without headers and skipped columns, the csv crate's
quoting, empty lines and ragged-record error, Rust's number parsing; and
write_csv's headers and number format (Rust's Display of a float: the
shortest round-trip decimal, no exponent)."""
import numpy as np
import pytest


def rust_display(x):
    """Rust's Display for f32 / f64, restated: shortest round-trip digits in
    positional notation; NaN, inf, -inf."""
    if np.isnan(x):
        return "NaN"
    if np.isinf(x):
        return "-inf" if x < 0 else "inf"
    return np.format_float_positional(x, unique=True, trim="-")


def test_load_csv_headers_and_skip(tmp_path):
    from bhtsne_gb300 import load_csv
    p = tmp_path / "data.csv"
    p.write_text("id,a,b,label\n0,1.5,-2,7\n1,3e2,.25,8\n\n2,+4,-0.0,9\r\n")
    v = load_csv(str(p), has_headers=True, skip=[0, 3])
    assert v.dtype == np.float32
    assert np.array_equal(v, np.array([1.5, -2, 300, 0.25, 4, -0.0], np.float32))
    assert np.signbit(v[5])
    w = load_csv(str(p), has_headers=True, dtype=np.float64)
    assert w.dtype == np.float64 and w.size == 12 and w[8] == 2 and w[11] == 9


def test_load_csv_quotes_and_special_values(tmp_path):
    from bhtsne_gb300 import load_csv
    p = tmp_path / "q.csv"
    p.write_text('"1.0","2"\n"inf",NaN\n-Infinity,"3.5e-1"\n')
    v = load_csv(str(p))
    assert v[0] == 1.0 and v[1] == 2.0 and np.isinf(v[2]) and np.isnan(v[3]) and v[4] == -np.inf
    assert v[5] == np.float32(0.35)


@pytest.mark.parametrize("text,what", [("1,2\n3\n", "fields"), ("1,x\n", "invalid float"), ("1, 2\n", "invalid float"),
                                       ("--1\n", "invalid float"), ('"1\n', "unterminated")])
def test_load_csv_errors(tmp_path, text, what):
    from bhtsne_gb300 import BhtsneError, load_csv
    p = tmp_path / "bad.csv"
    p.write_text(text)
    with pytest.raises(BhtsneError, match=what):
        load_csv(str(p))


def test_load_csv_missing_file(tmp_path):
    from bhtsne_gb300 import BhtsneError, load_csv
    with pytest.raises(BhtsneError) as e:
        load_csv(str(tmp_path / "none.csv"))
    assert e.value.code == 5


@pytest.mark.parametrize("D,header", [(2, "x,y"), (3, "x,y,z"), (4, None)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_write_csv_format(tmp_path, D, header, dtype):
    from bhtsne_gb300 import load_csv, write_csv
    rng = np.random.default_rng(D)
    e = (rng.normal(size=(50, D)) * 10.0 ** rng.integers(-9, 9, size=(50, D))).astype(dtype)
    e[0, 0], e[1, 0], e[2, 0] = dtype(0.1), dtype(-0.0), dtype(1e20)
    p = tmp_path / "e.csv"
    write_csv(e.ravel(), str(p), D=D)
    lines = p.read_text().split("\n")
    assert lines[-1] == ""
    body = lines[1:-1] if header else lines[:-1]
    if header:
        assert lines[0] == header
    assert len(body) == 50
    assert body[0].split(",")[0] == "0.1" and body[1].split(",")[0] == "-0"
    assert body[2].split(",")[0] == "100000000000000000000"
    for row, vals in zip(body, e):
        assert row == ",".join(rust_display(x) for x in vals)
    # and it reads back exactly
    back = load_csv(str(p), has_headers=header is not None, dtype=dtype)
    assert np.array_equal(back.view(np.uint8), e.ravel().view(np.uint8))
