"""Batched fits (bhtsne_batch): every job must fit as the same job would on
its own through the builder (src/lib.rs:701-772), which the other GPU tests
pin against the oracle; and one job of the batch against the oracle
directly."""
import numpy as np
import pytest

from conftest import blobs

pytestmark = pytest.mark.gpu

SIZES = [180, 700, 1500, 2600]


def jobs(dim=16, seed=70):
    out = []
    for j, n in enumerate(SIZES):
        X, lab = blobs(n, dim, 4 + j, seed + j)
        out.append((X, lab))
    return out


def seeds(D=2):
    return [np.random.default_rng(900 + j).normal(0, 1e-4, size=(n, D)).astype(np.float32)
            for j, n in enumerate(SIZES)]


def single(gpu, X, y0, epochs, D=2, perplexity=10.0):
    t = gpu.TSNE(X, D=D).perplexity(perplexity).epochs(epochs).initial_embedding(y0)
    t.barnes_hut(0.5)
    return t


@pytest.mark.parametrize("D", [2, 3])
def test_first_epochs_match_single_fits(gpu, D):
    """Per job the tree, traversal and attractive pass are those of a single
    fit; only Z's and the mean's summation order differ, so a few epochs agree
    to rounding."""
    data, y0 = jobs(), seeds(D)
    b = gpu.Batch(D=D, perplexity=10.0, epochs=3)
    for (X, _), y in zip(data, y0):
        j = b.add(X)
        b.initial_embedding(j, y)
    b.fit()
    assert len(b) == len(SIZES)
    for j, ((X, _), y) in enumerate(zip(data, y0)):
        ref = single(gpu, X, y, 3, D).embedding().astype(np.float64)
        got = b.embedding(j).astype(np.float64)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-4, (j, err)


def test_full_fits_match_single_fits(gpu):
    """1000 epochs: trajectories are chaotic (the single fit sums its
    attractive forces in another order once its layout is renumbered), so
    compare the final costs and the cluster structure. The summed cost of all
    jobs agrees within 1 %; a single job within 5 % (the smallest, 180 points,
    varies most between equally valid runs)."""
    data, y0 = jobs(), seeds()
    b = gpu.Batch(perplexity=10.0, epochs=1000)
    for (X, _), y in zip(data, y0):
        b.initial_embedding(b.add(X), y)
    b.fit()
    tot_b = tot_s = 0.0
    for j, ((X, lab), y) in enumerate(zip(data, y0)):
        t = single(gpu, X, y, 1000)
        for quirk in (True, False):
            kb, ks = b.kl_divergence(j, quirk), t.kl_divergence(quirk)
            assert abs(kb - ks) / abs(ks) < 0.05, (j, quirk, kb, ks)
            if not quirk:
                tot_b += kb
                tot_s += ks
        e = b.embedding(j).reshape(-1, 2).astype(np.float64)
        d = ((e[:, None, :] - e[None, :, :]) ** 2).sum(-1)
        np.fill_diagonal(d, np.inf)
        assert np.mean(lab == lab[d.argmin(1)]) > 0.95
    assert abs(tot_b - tot_s) / tot_s < 0.01, (tot_b, tot_s)


def test_one_job_against_the_oracle(gpu, oracle):
    X, _ = blobs(1200, 30, 6, 333)
    idx, dist = oracle.knn(X, 60)
    y = np.random.default_rng(8).normal(0, 1e-4, size=(1200, 2)).astype(np.float32)
    o = oracle.TSNE(1200).perplexity(20).epochs(1000).initial_embedding(y)
    o.barnes_hut_with_neighbors(0.5, idx.astype(np.uint64), dist)
    b = gpu.Batch(perplexity=20.0, epochs=1000)
    b.add_with_neighbors((idx, dist))
    b.initial_embedding(0, y)
    other, _ = blobs(500, 30, 3, 334)
    b.add(other)
    b.fit()
    for quirk in (True, False):
        kb, ko = b.kl_divergence(0, quirk), o.kl_divergence(quirk)
        assert abs(kb - ko) / abs(ko) < 0.01, (quirk, kb, ko)


def test_neighbors_job_equals_euclidean_job(gpu, oracle):
    X, _ = blobs(900, 12, 5, 21)
    idx, dist = oracle.knn(X, 30)
    y = np.random.default_rng(3).normal(0, 1e-4, size=(900, 2)).astype(np.float32)
    outs = []
    for how in ("euclidean", "neighbors"):
        b = gpu.Batch(perplexity=10.0, epochs=60)
        j = b.add(X) if how == "euclidean" else b.add_with_neighbors((idx, dist))
        b.initial_embedding(j, y)
        b.fit()
        outs.append(b.embedding(j))
    assert np.array_equal(outs[0], outs[1])


def test_batch_is_deterministic(gpu):
    data = jobs()
    outs = []
    for _ in range(2):
        b = gpu.Batch(perplexity=10.0, epochs=120, seed=77)
        for X, _ in data:
            b.add(X)
        b.fit()
        outs.append(np.concatenate([b.embedding(j) for j in range(len(data))]))
    assert np.array_equal(outs[0], outs[1])
    assert np.all(np.isfinite(outs[0]))


def test_batch_errors(gpu):
    b = gpu.Batch(perplexity=30.0, epochs=10)
    X, _ = blobs(60, 4, 2, 1)
    with pytest.raises(gpu.BhtsneError, match="perplexity is too large"):
        b.add(X)
    with pytest.raises(gpu.BhtsneError, match="no jobs"):
        b.fit()
    Y, _ = blobs(200, 4, 2, 2)
    b.add(Y)
    with pytest.raises(gpu.BhtsneError, match="initial embedding"):
        b.initial_embedding(0, np.zeros(10, np.float32))
    t = gpu.Batch(perplexity=10.0, epochs=10, theta=0.0)
    t.add(Y)
    with pytest.raises(gpu.BhtsneError, match="theta value must be greater than 0.0"):
        t.fit()
    with pytest.raises(gpu.BhtsneError, match="no fitted job"):
        t.embedding(0)


def test_mixed_inputs_in_one_batch(gpu, oracle):
    """Euclidean jobs and kNN-table jobs (of another k) are prepared as separate
    groups and fitted together; a job given as data and the same job given as
    its kNN table end identical."""
    X, _ = blobs(800, 20, 4, 31)
    Z, _ = blobs(400, 20, 3, 32)
    idx, dist = oracle.knn(X, 30)
    idx2, dist2 = oracle.knn(Z, 45)
    y = np.random.default_rng(4).normal(0, 1e-4, size=(800, 2)).astype(np.float32)
    b = gpu.Batch(perplexity=10.0, epochs=80)
    a0 = b.add(X)
    a1 = b.add_with_neighbors((idx, dist))
    a2 = b.add_with_neighbors((idx2, dist2))
    a3 = b.add(Z)
    b.initial_embedding(a0, y)
    b.initial_embedding(a1, y)
    b.fit()
    assert np.array_equal(b.embedding(a0), b.embedding(a1))
    for j in (a2, a3):
        assert np.all(np.isfinite(b.embedding(j)))
    # a second fit of the same batch restarts from fresh seeds and matches the first
    first = [b.embedding(j) for j in range(4)]
    b.initial_embedding(a0, y)
    b.initial_embedding(a1, y)
    b.fit()
    for j in range(4):
        assert np.array_equal(first[j], b.embedding(j))
