"""GPU parity: libeddy_gpu (through its C ABI) against the oracle.

Integer results (edge decisions of every leave-one-out network, unique
networks, capped parent lists, unique counts) must be identical.  Floating
results: node-summed BDeu within 1e-9 relative (fixed-point sums of a
long-double lgamma table vs the oracle's FP64 lgamma), normalised
likelihoods within 1e-6 relative, JS within 1e-5 relative + 1e-9 absolute
(JS values of identical distributions are rounding noise near 0).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JS_RTOL, JS_ATOL = 1e-5, 1e-9


def planted(rng, g, n, planted=4, w=0.8, noise=0.5, nA=None, invalid=0.0):
    from eddy_gpu import synth
    x = rng.standard_normal((g, n))
    nA = n // 2 if nA is None else nA
    for k in range(min(planted, g // 2)):
        x[g - 1 - k, :nA] = w * x[k, :nA] + noise * rng.standard_normal(nA)
    d = synth.tertiles(x)
    if invalid:
        m = rng.random(d.shape) < invalid
        d[m] = 2
    return d


def make_labels(rng, n, nA):
    lab = np.ones(n, np.uint8)
    lab[rng.choice(n, nA, replace=False)] = 0
    return lab


def js_close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return (np.isclose(a, b, rtol=JS_RTOL, atol=JS_ATOL) | (np.isnan(a) & np.isnan(b))).all()


CASES = [
    # g, n, nA, mp, bonf, pw, nprior, invalid
    (8, 30, 15, 3, True, 0.5, 0, 0.0),
    (12, 40, 18, 2, False, 0.5, 6, 0.0),
    (20, 120, 60, 3, True, 0.0, 0, 0.0),
    (30, 80, 33, 4, False, 0.5, 10, 0.0),
    (50, 40, 20, 3, False, 0.5, 0, 0.0),
    (16, 60, 30, 3, False, 0.5, 4, 0.05),
    (40, 400, 150, 3, True, 0.5, 30, 0.0),
    (24, 200, 100, 1, False, 0.5, 0, 0.0),
]


def _prior(rng, g, k):
    pr = np.zeros((g, g), np.uint8)
    for _ in range(k):
        i, j = rng.choice(g, 2, replace=False)
        pr[i, j] = pr[j, i] = 1
    return pr


@pytest.mark.parametrize("case", CASES, ids=[f"g{c[0]}n{c[1]}mp{c[3]}" for c in CASES])
def test_edges_units_vs_oracle(case, eddy_lib, oracle_lib):
    g, n, nA, mp, bonf, pw, npr, inv = case
    rng = np.random.default_rng(g * 1000 + n)
    data = planted(rng, g, n, nA=nA, invalid=inv)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    pr = _prior(rng, g, npr) if npr else None
    O = oracle_lib
    prm = O.params(mp=mp, bonferroni=bonf, pw=pw)
    ctx = eddy_lib.Context(max_parents=mp, bonferroni=bonf, prior_weight=pw, permutations=3,
                           rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g), pr)
    for trial in range(3):
        lab = labels0 if trial == 0 else make_labels(rng, n, nA)
        # edge decisions of all S networks
        e_gpu = ctx.debug_edges(sid, lab)
        dA = data[:, lab == 0]
        dB = data[:, lab == 1]
        e_or, _, _ = O.k1_edges(dA, dB, pr, prm)
        assert e_gpu.shape == e_or.shape
        bad = np.argwhere(e_gpu != e_or)
        assert bad.size == 0, f"{len(bad)} edge decisions differ, first {bad[:5]}"
        # full unit
        mpk = min(mp, g - 1)
        du = ctx.debug_unit(sid, lab, mpk)
        ou = O.unit(data, lab, pr, prm)
        assert du["U"] == ou["U"]
        assert np.array_equal(du["ids"], ou["unique_ids"])
        # capped parent lists of every unique network
        for u in range(ou["U"]):
            nodes = ou["uni_nodes"][u]
            ecount = ou["uni_epn"][u + 1] - ou["uni_epn"][u]
            cnt = np.diff(np.append(nodes, ecount))
            assert np.array_equal(du["counts"][u], cnt), u
            ed = ou["uni_edges"][ou["uni_epn"][u]:ou["uni_epn"][u + 1]]
            got = np.concatenate([du["parents"][u, t, :cnt[t]] for t in range(g)])
            assert np.array_equal(got, ed), u
        dist_or = ou["out5"].sum(axis=2)
        np.testing.assert_allclose(du["dist"], dist_or, rtol=1e-9, atol=1e-7)
        if not np.isnan(ou["js"]):
            np.testing.assert_allclose(du["lval"], ou["lval"], rtol=1e-6, atol=1e-12)
        assert js_close(du["js"], ou["js"]), (du["js"], ou["js"])


def test_run_labellings_many(eddy_lib, oracle_lib):
    rng = np.random.default_rng(5)
    g, n, nA = 20, 200, 100
    data = planted(rng, g, n, nA=nA)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    lab = oracle_lib.counter_labels(11, 0, labels0, 64)
    ctx = eddy_lib.Context(max_parents=3, permutations=64, rng=eddy_lib.RNG_EXTERNAL,
                           prior_weight=0.0)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    js, U = ctx.run_labellings(sid, lab)
    ojs, oU = oracle_lib.units(data, lab, None, oracle_lib.params(mp=3, pw=0.0))
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)


def test_counter_stream_matches_oracle(eddy_lib, oracle_lib):
    """Device-generated counter labellings == oracle's Philox labellings."""
    rng = np.random.default_rng(9)
    g, n, nA = 14, 150, 70
    data = planted(rng, g, n, nA=nA)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    R = 40
    ctx = eddy_lib.Context(max_parents=3, permutations=R, rng=eddy_lib.RNG_COUNTER, seed=1234)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    ctx.run()
    js, U = ctx.js(sid)
    lab = oracle_lib.counter_labels(1234, sid, labels0, R)
    ojs, oU = oracle_lib.units(data, lab, None, oracle_lib.params(mp=3))
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)
    s = ctx.summary(sid)
    rc, a, b, p = oracle_lib.pddn(ojs)
    if rc == 0:
        assert s["betafit_ok"] == 1
        np.testing.assert_allclose([s["alpha"], s["beta"]], [a, b], rtol=1e-4)
        np.testing.assert_allclose(s["pddn"], p, rtol=1e-4, atol=1e-9)


def test_graph_replays_match_oracle(eddy_lib, oracle_lib, monkeypatch):
    """Repeated batches of one set run as a captured CUDA graph: the first
    batch of a shape launches directly, the second is captured, later ones
    replay it with new permutation indices; a switch to another set and back
    (direct, then re-capture) all match the oracle."""
    monkeypatch.setenv("EDDY_MMA_VARIANT", "2")  # a known tile shape: no tuning batch
    rng = np.random.default_rng(21)
    g, n, nA = 24, 180, 80
    data = planted(rng, g, n, nA=nA)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    seed = 77
    ctx = eddy_lib.Context(max_parents=3, permutations=64, rng=eddy_lib.RNG_COUNTER, seed=seed)
    ctx.load_matrix(data, labels0)
    sa = ctx.add_set(np.arange(g))
    sb = ctx.add_set(np.arange(0, g, 2))
    B = 48
    prm = oracle_lib.params(mp=3)
    for sid, first in [(sa, 1), (sa, 1 + B), (sa, 1 + 2 * B), (sb, 1), (sb, 1 + B), (sb, 1 + 2 * B),
                       (sa, 1 + 3 * B), (sa, 1 + 4 * B), (sa, 1 + 5 * B)]:
        js, U = ctx.run_permutations(sid, first, B)
        genes = np.arange(g) if sid == sa else np.arange(0, g, 2)
        lab = oracle_lib.counter_labels(seed, sid, labels0, first + B)[first:first + B]
        ojs, oU = oracle_lib.units(data[genes], lab, None, prm)
        assert np.array_equal(U, oU), (sid, first)
        assert js_close(js, ojs), (sid, first)


def test_glibc_stream_matches_reference_sampler(eddy_lib, oracle_lib):
    """GLIBC mode: the permutation stream of main.cu:538-573 across two sets."""
    rng = np.random.default_rng(3)
    g, n, nA = 10, 60, 25
    data = planted(rng, 2 * g, n, nA=nA)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    R = 12
    ctx = eddy_lib.Context(max_parents=3, permutations=R, rng=eddy_lib.RNG_GLIBC,
                           bonferroni=False)
    ctx.load_matrix(data, labels0)
    s0 = ctx.add_set(np.arange(g))
    s1 = ctx.add_set(np.arange(g, 2 * g))
    ctx.run()
    prm = oracle_lib.params(mp=3, bonferroni=False)
    sets = [np.arange(g), np.arange(g, 2 * g)]
    streams = oracle_lib.reference_stream(
        n, nA, labels0, R, lambda i, l0: oracle_lib.unit(data[sets[i]], l0, None, prm,
                                                          outputs=False)["js"], 2)
    for sid, rows, genes in ((s0, streams[0], sets[0]), (s1, streams[1], sets[1])):
        js, U = ctx.js(sid)
        ojs, oU = oracle_lib.units(data[genes], rows, None, prm)
        assert len(js) == len(ojs)
        assert np.array_equal(U, oU)
        assert js_close(js, ojs)


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4],
                         ids=["n128e16", "n128e8", "n192e12", "n256e8", "n256e16"])
@pytest.mark.parametrize("case", [CASES[2], CASES[4], CASES[5], CASES[6]],
                         ids=["g20", "g50", "invalid", "g40prior"])
def test_tensor_core_and_popcount_paths_agree(case, variant, eddy_lib, monkeypatch):
    """Every tile shape of the tcgen05 contingency GEMM and the popcount
    kernel give the same edge decisions for every network (bit for bit)."""
    monkeypatch.setenv("EDDY_MMA_VARIANT", str(variant))
    g, n, nA, mp, bonf, pw, npr, inv = case
    rng = np.random.default_rng(g + 7 * n)
    data = planted(rng, g, n, nA=nA, invalid=inv)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    pr = _prior(rng, g, npr) if npr else None
    ctx = eddy_lib.Context(max_parents=mp, bonferroni=bonf, prior_weight=pw,
                           rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g), pr)
    for t in range(2):
        lab = labels0 if t == 0 else make_labels(rng, n, nA)
        monkeypatch.delenv("EDDY_PAIRS_KERNEL", raising=False)
        a = ctx.debug_edges(sid, lab)
        monkeypatch.setenv("EDDY_PAIRS_KERNEL", "popc")
        b = ctx.debug_edges(sid, lab)
        assert np.array_equal(a, b)
    labs = np.stack([make_labels(rng, n, nA) for _ in range(300)])
    monkeypatch.delenv("EDDY_PAIRS_KERNEL", raising=False)
    js1, U1 = ctx.run_labellings(sid, labs)
    monkeypatch.setenv("EDDY_PAIRS_KERNEL", "popc")
    js2, U2 = ctx.run_labellings(sid, labs)
    assert np.array_equal(U1, U2)
    assert np.array_equal(js1, js2) or js_close(js1, js2)
