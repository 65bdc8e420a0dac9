"""GPU parity at the edges of the supported shapes and on the fallback
paths, against the oracle: 4096 samples (the largest labelling drawn on the
device), more than 4096 samples (labellings generated on the host), the
512-gene maximum, a general-path queue that overflows (the batch is then
decided by the popcount kernel) and networks with more changed nodes than
the first pass records (the units are re-run)."""
import numpy as np
import pytest

from test_gpu_parity import js_close, make_labels, planted

pytestmark = pytest.mark.gpu


def _oracle(oracle_lib, data, labs, mp=3, bonf=True, pw=0.5, prior=None):
    prm = oracle_lib.params(mp=mp, bonferroni=bonf, pw=pw)
    return oracle_lib.units(data, labs, prior, prm)


def test_many_samples_counter_stream(eddy_lib, oracle_lib):
    """n = 4500 (> 4096): the counter labellings come from the host
    (permutations 0..3 of the stream, no stop at a NaN JS)."""
    rng = np.random.default_rng(31)
    g, n, nA = 8, 4500, 2000
    data = planted(rng, g, n, nA=nA, planted=3)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    R, seed = 4, 99
    ctx = eddy_lib.Context(max_parents=3, permutations=R, rng=eddy_lib.RNG_COUNTER, seed=seed)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    js, U = ctx.run_permutations(sid, 0, R)
    ojs, oU = _oracle(oracle_lib, data, oracle_lib.counter_labels(seed, sid, labels0, R))
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)


def test_largest_device_labelling(eddy_lib, oracle_lib):
    """n = 4096, the largest sample count whose counter labellings are drawn
    on the device (radix select over 4096 keys): labels, U and JS as the
    oracle's sorted Philox keys give them."""
    rng = np.random.default_rng(35)
    g, n, nA = 6, 4096, 1500
    data = planted(rng, g, n, nA=nA, planted=3)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    R, seed = 6, 123
    ctx = eddy_lib.Context(max_parents=3, permutations=R, rng=eddy_lib.RNG_COUNTER, seed=seed)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    js, U = ctx.run_permutations(sid, 0, R)
    ojs, oU = _oracle(oracle_lib, data, oracle_lib.counter_labels(seed, sid, labels0, R))
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)


def test_maximum_set_size(eddy_lib, oracle_lib):
    """g = 512 genes (130816 pairs), the largest set the GPU path takes."""
    rng = np.random.default_rng(32)
    g, n, nA = 512, 60, 30
    data = planted(rng, g, n, nA=nA, planted=40)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    labs = np.stack([labels0] + [make_labels(rng, n, nA) for _ in range(2)])
    ctx = eddy_lib.Context(max_parents=3, rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    js, U = ctx.run_labellings(sid, labs)
    ojs, oU = _oracle(oracle_lib, data, labs)
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)


def test_general_queue_overflow_falls_back(eddy_lib, oracle_lib, monkeypatch):
    """Classes below 32 samples leave every table to the general path; a
    queue of one entry overflows and the batch is decided by the popcount
    kernel instead, with the same results."""
    rng = np.random.default_rng(33)
    g, n, nA = 30, 40, 20
    data = planted(rng, g, n, nA=nA)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    labs = np.stack([labels0] + [make_labels(rng, n, nA) for _ in range(40)])
    ctx = eddy_lib.Context(max_parents=3, bonferroni=False, rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    monkeypatch.setenv("EDDY_GENERAL_QUEUE_CAP", "1")
    js, U = ctx.run_labellings(sid, labs)
    ojs, oU = _oracle(oracle_lib, data, labs, bonf=False)
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)


def test_changed_node_overflow_reruns(eddy_lib, oracle_lib, monkeypatch):
    """With room for one changed node per network, every network that
    changes more is re-run with room for all of them."""
    rng = np.random.default_rng(34)
    g, n, nA = 24, 60, 30
    data = planted(rng, g, n, nA=nA, planted=8, w=0.9, noise=0.4)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    labs = np.stack([labels0] + [make_labels(rng, n, nA) for _ in range(60)])
    ctx = eddy_lib.Context(max_parents=3, bonferroni=False, rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    monkeypatch.setenv("EDDY_KMAX", "1")
    js, U = ctx.run_labellings(sid, labs)
    ojs, oU = _oracle(oracle_lib, data, labs, bonf=False)
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)
    assert U.max() > 2  # networks with changes occurred
