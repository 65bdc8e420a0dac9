"""The two operand layouts of the tensor-core contingency GEMM on the same
units.  For a set with no missing value the GEMM counts four cells of each
class-1 table and the epilogue derives the other five from the two genes'
class counts; EDDY_PAIR_LAYOUT=full keeps the nine-cell layout.  Both must
give identical edge decisions, JS and unique-network counts, and the
all-zero filter must settle exactly the same number of tables: the bound is
the same arithmetic on the same exact values (kernel1.cu:121-203 decides
every table either way)."""
import numpy as np
import pytest

from test_gpu_parity import js_close, make_labels, planted

pytestmark = pytest.mark.gpu


def _run(eddy_lib, monkeypatch, layout, data, labels0, genes, units, variant, mp=3):
    if layout == "full":
        monkeypatch.setenv("EDDY_PAIR_LAYOUT", "full")
    else:
        monkeypatch.delenv("EDDY_PAIR_LAYOUT", raising=False)
    monkeypatch.setenv("EDDY_MMA_VARIANT", str(variant))
    ctx = eddy_lib.Context(max_parents=mp, permutations=units, rng=eddy_lib.RNG_COUNTER,
                           seed=11, keep_networks=False)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.asarray(genes))
    js, U = ctx.run_permutations(sid, 1, units)
    st = ctx.stats()
    rng = np.random.default_rng(3)
    nA = int((labels0 == 0).sum())
    edges = [ctx.debug_edges(sid, make_labels(rng, len(labels0), nA)) for _ in range(2)]
    return js, U, st, edges


@pytest.mark.parametrize("variant", [1, 2, 3])
@pytest.mark.parametrize("g", [2, 3, 9, 41, 130])
def test_layouts_agree(g, variant, eddy_lib, monkeypatch):
    rng = np.random.default_rng(100 + g)
    n, nA = 300, 130
    data = planted(rng, g, n, nA=nA, planted=min(6, g // 2), w=0.9, noise=0.4)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    units = 700  # several unit blocks, the last one partial
    a = _run(eddy_lib, monkeypatch, "core", data, labels0, np.arange(g), units, variant)
    b = _run(eddy_lib, monkeypatch, "full", data, labels0, np.arange(g), units, variant)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[0], b[0], equal_nan=True)
    assert a[2]["tables"] == b[2]["tables"] == 2 * units * g * (g - 1) // 2
    assert a[2]["filtered"] == b[2]["filtered"]
    for ea, eb in zip(a[3], b[3]):
        assert np.array_equal(ea, eb)


def test_layouts_agree_near_threshold(eddy_lib, monkeypatch):
    """The 200-gene, 1000-sample workload whose dependencies sit near the
    Bonferroni edge threshold: many tables reach the general path."""
    from eddy_gpu import synth
    w = synth.make(4, seed=0)
    genes = w.sets[0][1]
    a = _run(eddy_lib, monkeypatch, "core", w.data, w.labels, genes, 1024, 3, mp=4)
    b = _run(eddy_lib, monkeypatch, "full", w.data, w.labels, genes, 1024, 3, mp=4)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[0], b[0], equal_nan=True)
    assert a[2]["filtered"] == b[2]["filtered"] and a[2]["tables"] == b[2]["tables"]
    assert a[2]["filtered"] < a[2]["tables"]  # some tables took the general path
    for ea, eb in zip(a[3], b[3]):
        assert np.array_equal(ea, eb)


def test_missing_values_keep_the_full_layout(eddy_lib, oracle_lib, monkeypatch):
    """A set with a missing value anywhere runs the nine-cell layout; a set of
    the same matrix without one runs the four-cell layout; both match the
    oracle."""
    rng = np.random.default_rng(7)
    g, n, nA = 12, 200, 90
    data = planted(rng, g, n, nA=nA, planted=4, w=0.9, noise=0.4)
    data[5, 17] = 2  # one missing value in gene 5
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    monkeypatch.delenv("EDDY_PAIR_LAYOUT", raising=False)
    ctx = eddy_lib.Context(max_parents=3, rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(data, labels0)
    labs = np.stack([make_labels(rng, n, nA) for _ in range(40)])
    for genes in (np.arange(g), np.array([0, 1, 2, 3, 4, 6, 7, 8, 9, 10, 11])):
        sid = ctx.add_set(genes)
        js, U = ctx.run_labellings(sid, labs)
        ojs, oU = oracle_lib.units(data[genes], labs, None, None)
        assert np.array_equal(U, oU)
        assert js_close(js, ojs)


@pytest.mark.parametrize("g", [30, 150])
def test_tuner_chooses_between_layouts(g, eddy_lib, monkeypatch):
    """Unpinned, the first batch of >= 512 units times every tile shape in
    both layouts (choices 0-9); whichever wins, the results equal the pinned
    9-cell ones, on the tuning batch and on the batches after it."""
    rng = np.random.default_rng(500 + g)
    n, nA = 400, 180
    data = planted(rng, g, n, nA=nA, planted=min(6, g // 2), w=0.9, noise=0.4)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    ref = _run(eddy_lib, monkeypatch, "full", data, labels0, np.arange(g), 600, 3)
    monkeypatch.delenv("EDDY_MMA_VARIANT", raising=False)
    monkeypatch.delenv("EDDY_PAIR_LAYOUT", raising=False)
    ctx = eddy_lib.Context(max_parents=3, permutations=600, rng=eddy_lib.RNG_COUNTER,
                           seed=11, keep_networks=False)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g))
    for _ in range(3):  # tuning batch, direct launch, graph replay
        js, U = ctx.run_permutations(sid, 1, 600)
        assert 0 <= ctx.stats()["variant"] < 10
        assert np.array_equal(U, ref[1])
        assert np.array_equal(js, ref[0], equal_nan=True)


def test_tuned_choice_not_shared_with_missing_values(eddy_lib, monkeypatch):
    """Two sets of the same size class in one context, the second with a
    missing value: whatever the first set tuned, the second runs the 9-cell
    layout and matches its pinned 9-cell result."""
    rng = np.random.default_rng(77)
    G, n, nA, g = 320, 300, 140, 150
    data = planted(rng, G, n, nA=nA, planted=8, w=0.9, noise=0.4)
    data[300, 5] = 2  # gene 300 has a missing value
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    genes_a = np.arange(g)
    genes_b = np.concatenate([np.arange(1, g), [300]])

    def run(pinned):
        if pinned:
            monkeypatch.setenv("EDDY_PAIR_LAYOUT", "full")
            monkeypatch.setenv("EDDY_MMA_VARIANT", "3")
        else:
            monkeypatch.delenv("EDDY_MMA_VARIANT", raising=False)
            monkeypatch.delenv("EDDY_PAIR_LAYOUT", raising=False)
        ctx = eddy_lib.Context(max_parents=3, permutations=600, rng=eddy_lib.RNG_COUNTER,
                               seed=11, keep_networks=False)
        ctx.load_matrix(data, labels0)
        sa = ctx.add_set(genes_a)  # set 0 (the counter stream is keyed by set)
        ctx.run_permutations(sa, 1, 600)
        sb = ctx.add_set(genes_b)
        js, U = ctx.run_permutations(sb, 1, 600)
        return js, U, ctx.stats()["variant"]

    ref = run(True)
    js, U, variant = run(False)
    assert variant < 5
    assert np.array_equal(U, ref[1])
    assert np.array_equal(js, ref[0], equal_nan=True)
