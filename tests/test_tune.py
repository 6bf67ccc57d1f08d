"""The autotuner's table (no reference counterpart), on the CPU: defaults
before any tuning, the JSON file round trip, and errors. The timing sweep
itself runs on the GPU (tests/test_gpu_tune.py)."""
import json

import pytest


def test_defaults_without_tuning():
    import bhtsne_gb300 as bg
    cfg = bg.tune_config(bg.F32, 2, 1_000_000)
    assert cfg["knobs"] == {"attr_task_len": 128, "bh_threads": 256, "knn_pass": "default", "tuned": False}
    assert cfg["key"].endswith("|f32|D2|n2^19")


def test_table_file_round_trip(tmp_path):
    import bhtsne_gb300 as bg
    key = bg.tune_config(bg.F32, 3, 5000)["key"]  # this machine's key for the 2^12 bucket
    p = tmp_path / "tune.json"
    p.write_text(json.dumps({key: {"attr_task_len": 64, "bh_threads": 512, "knn_pass": 1}}))
    bg.tune_load(str(p))
    cfg = bg.tune_config(bg.F32, 3, 4096)
    assert cfg["knobs"] == {"attr_task_len": 64, "bh_threads": 512, "knn_pass": "cuda_cores", "tuned": True}
    # another bucket, D or type keeps the defaults
    assert bg.tune_config(bg.F32, 3, 9000)["knobs"]["tuned"] is False
    assert bg.tune_config(bg.F64, 3, 4096)["knobs"]["tuned"] is False
    out = tmp_path / "saved.json"
    bg.tune_save(str(out))
    saved = json.loads(out.read_text())
    assert saved[key] == {"attr_task_len": 64, "bh_threads": 512, "knn_pass": 1}


def test_table_errors(tmp_path):
    import bhtsne_gb300 as bg
    with pytest.raises(bg.BhtsneError):
        bg.tune_load(str(tmp_path / "missing.json"))
    bad = tmp_path / "bad.json"
    bad.write_text('{"k": {"attr_task_len": 64}}')
    with pytest.raises(bg.BhtsneError, match="not a tuning table"):
        bg.tune_load(str(bad))
