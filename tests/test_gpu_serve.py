"""Serving (bhtsne_server): requests fitted concurrently give the same result
alone and in a mix, match the plain builder's fits, and respect admission."""
import time

import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu


def request_data(i, n, dim=20):
    X, _ = blobs(n, dim, 4 + i % 5, 500 + i)
    return X


def test_result_alone_equals_result_in_a_mix(gpu):
    """Per job, the batched epoch computes its tree, Z, mean and update from
    its own rows only, so a Barnes-Hut request's embedding is bit-identical
    whether it runs alone or joins a batch of other requests mid-flight; a
    FIt-SNE request runs the deterministic builder path either way."""
    target = request_data(0, 1500)
    alone = gpu.Server(perplexity=10.0, round_epochs=20, fit_workers=1)
    j = alone.submit(target, "bh", epochs=300, seed=7)
    f = alone.submit(target, "fit", epochs=120, seed=8)
    alone.wait(j)
    alone.wait(f)
    e_alone, kl_alone, _ = alone.result(j)
    fe_alone, fkl_alone, _ = alone.result(f)
    alone.close()

    mix = gpu.Server(perplexity=10.0, round_epochs=20, fit_workers=2)
    early = [mix.submit(request_data(i, 600 + 300 * i), "bh", epochs=200 + 60 * i, seed=i) for i in range(1, 4)]
    time.sleep(0.05)  # the target joins a batch already in flight
    j = mix.submit(target, "bh", epochs=300, seed=7)
    f = mix.submit(target, "fit", epochs=120, seed=8)
    late = [mix.submit(request_data(i, 900), "bh" if i % 2 else "fit", epochs=150, seed=i) for i in range(4, 7)]
    for r in early + late + [j, f]:
        assert mix.wait(r, timeout=600)
    e_mix, kl_mix, _ = mix.result(j)
    fe_mix, fkl_mix, _ = mix.result(f)
    for r in early + late:
        e, kl, lat = mix.result(r)
        assert np.all(np.isfinite(e)) and np.isfinite(kl) and lat > 0
    st = mix.stats()
    mix.close()
    assert np.array_equal(e_alone, e_mix)
    assert kl_alone == kl_mix
    assert np.array_equal(fe_alone, fe_mix)
    assert fkl_alone == fkl_mix
    assert st["done"] == 8 and st["in_flight"] == 0 and st["mean_batch_points"] > 1500


def test_server_matches_plain_builder(gpu):
    """Against the plain builder with the same seed: the batched job sums Z and
    the mean in another order, so the final costs agree within 2 %, not bit
    for bit."""
    X = request_data(9, 2500)
    sv = gpu.Server(perplexity=20.0)
    j = sv.submit(X, "bh", epochs=500, seed=21)
    sv.wait(j)
    e, kl, _ = sv.result(j)
    sv.close()
    t = gpu.TSNE(X).perplexity(20.0).epochs(500).random_seed(21)
    t.barnes_hut(0.5)
    ref = t.kl_divergence()
    assert abs(kl - ref) / ref < 0.02, (kl, ref)


def test_admission_respects_the_budget(gpu):
    """With a budget that holds one request at a time, requests still all
    finish, in order, and the admitted footprint never exceeds the budget."""
    sizes = [700, 800, 900]
    sv = gpu.Server(perplexity=10.0, hbm_budget_bytes=1, round_epochs=10)
    ids = [sv.submit(request_data(i, n), "bh", epochs=60, seed=i) for i, n in enumerate(sizes)]
    assert sv.poll(ids[-1]) in ("queued", "running")
    for i in ids:
        assert sv.wait(i, timeout=600)
    lat = [sv.result(i)[2] for i in ids]
    st = sv.stats()
    sv.close()
    assert lat[0] < lat[1] < lat[2]
    assert st["done"] == 3


def test_server_errors(gpu):
    sv = gpu.Server(perplexity=30.0)
    with pytest.raises(gpu.BhtsneError, match="perplexity is too large"):
        sv.submit(np.zeros((50, 4), np.float32))
    with pytest.raises(gpu.BhtsneError, match="no request"):
        sv.result(12345)
    j = sv.submit(request_data(1, 3000), "bh", epochs=2000, seed=1)
    assert sv.wait(j, timeout=0.001) is False
    sv.close()
    with pytest.raises(gpu.BhtsneError):
        gpu.Server(D=3).submit(request_data(1, 500), "fit")
