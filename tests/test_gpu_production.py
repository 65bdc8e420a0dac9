"""Parity of the production paths against the oracle.

- The batched path at the benchmark's shape (config 4, precision stress:
  200 genes x 1000 samples, -mp 4) in batches of 1024 units: the tuning
  batch, a batch of the tuned shape launched directly, and batches replayed
  from a CUDA graph.
- Samples of the many-set workloads (config 3: sets of 10-150 genes at 600
  samples, some with prior pairs; config 5: sets of 5-300 genes at 1000
  samples, above the reference's 200-gene cap, definitions.cuh:19) run by
  eddy_run in one context: JS and U of every iteration, the NaN break of
  main.cu:1431-1435 and pDDN (main.cu:1488-1502).  In these workloads most
  labellings give a single unique network (the planted dependencies are
  strong enough to fall past the AS 147 underflow cut-off, kernel1.cu:17, 38,
  which makes their p = 1), so most sets fail at a NaN JS as the
  reference's would; those failures are checked as such.
- The uncapped parent lists of iteration 0's two full-data networks that
  the _EdgeList file is written from (main.cu:1530-1641, parent limit
  INT_MAX at main.cu:1564).

Bars: edge decisions, U and parent lists bit-exact; JS within 1e-5
relative (+1e-9 absolute); pDDN within 1e-4 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JS_RTOL, JS_ATOL, PDDN_RTOL = 1e-5, 1e-9, 1e-4


def _close(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return bool((np.isclose(a, b, rtol=JS_RTOL, atol=JS_ATOL) | (np.isnan(a) & np.isnan(b))).all())


def test_config4_tuned_direct_and_graph_batches(eddy_lib, oracle_lib):
    from eddy_gpu import synth
    O = oracle_lib
    w = synth.make(4, seed=0)
    genes = w.sets[0][1]
    mp, pw = w.flags["mp"], w.flags["pw"]
    seed, B, calls = 31, 1024, 4
    ctx = eddy_lib.Context(max_parents=mp, prior_weight=pw, permutations=B * calls + 1,
                           rng=eddy_lib.RNG_COUNTER, seed=seed, keep_networks=False)
    ctx.load_matrix(w.data, w.labels)
    sid = ctx.add_set(genes)
    js, U = [], []
    # call 0 tunes the tile shape on its batch; call 1 launches the tuned
    # shape directly; calls 2 and 3 repeat its shape and buffers and are
    # replayed from a captured graph
    for k in range(calls):
        j, u = ctx.run_permutations(sid, 1 + k * B, B)
        js.append(j)
        U.append(u)
        # the per-kernel split of the device time adds up to the stage times
        t = ctx.timing()
        assert min(t["ms_gemm"], t["ms_decide"], t["ms_networks"], t["ms_js"]) >= 0
        assert abs(t["ms_gemm"] + t["ms_decide"] - t["ms_pairs"]) <= 0.01 + 1e-3 * t["ms_pairs"]
        assert abs(t["ms_networks"] + t["ms_js"] - t["ms_units"]) <= 0.01 + 1e-3 * t["ms_units"]
    js, U = np.concatenate(js), np.concatenate(U)
    labs = O.counter_labels(seed, sid, w.labels, B * calls + 1)
    pick = np.array([0, 1, 700, 1023, 1024, 1500, 2047, 2048, 2600, 3071, 3072, 3500, 3900,
                     4000, 4094, 4095])
    prm = O.params(mp=mp, pw=pw)
    data = w.data[genes]
    ojs, oU = O.units(data, labs[1 + pick], None, prm)
    assert np.array_equal(U[pick], oU), (U[pick], oU)
    assert _close(js[pick], ojs), (js[pick], ojs)
    # every edge decision of every network of two of those labellings
    for r in (pick[1], pick[-1]):
        lab = labs[1 + r]
        e = ctx.debug_edges(sid, lab)
        oe, _, _ = O.k1_edges(data[:, lab == 0], data[:, lab == 1], None, prm)
        assert np.array_equal(e, oe)
    ctx.close()


def _many_sets(eddy_lib, O, w, picks, R, seed):
    mp, pw = w.flags["mp"], w.flags["pw"]
    prm = O.params(mp=mp, pw=pw)
    ctx = eddy_lib.Context(max_parents=mp, prior_weight=pw, permutations=R,
                           rng=eddy_lib.RNG_COUNTER, seed=seed, keep_networks=True)
    ctx.load_matrix(w.data, w.labels)
    sids = [ctx.add_set(genes, prior) for genes, prior in picks]
    ctx.run()
    fitted = 0
    for sid, (genes, prior) in zip(sids, picks):
        labs = O.counter_labels(seed, sid, w.labels, R)
        ojs, oU = O.units(w.data[genes], labs, prior, prm)
        s = ctx.summary(sid)
        gjs, gU = ctx.js(sid)
        assert s["genes"] == len(genes)
        if np.isnan(ojs[0]):
            # main.cu:1431-1435: the set stops after iteration 0
            assert s["failed"] == 1 and s["iterations"] == 1 and np.isnan(gjs[0])
            assert gU[0] == oU[0]
            continue
        assert s["iterations"] == R
        assert np.array_equal(gU, oU), (sid, gU, oU)
        assert _close(gjs, ojs), (sid, gjs, ojs)
        assert bool(s["failed"]) == bool(np.isnan(ojs).any())
        if not s["failed"]:
            rc, oa, ob, op = O.pddn(ojs)
            assert rc == 0 and s["betafit_ok"] == 1
            assert abs(s["pddn"] - op) <= PDDN_RTOL * abs(op) + 1e-300, (s["pddn"], op)
            fitted += 1
    ctx.close()
    return fitted


def test_config3_sample_in_one_context(eddy_lib, oracle_lib):
    """Config 3's shapes: sets of uneven size from 10 to 150 genes of a
    5000 x 600 matrix (2% of genes planted), a fifth of them with 5-20 prior
    pairs at -pw 0.5; the smallest and largest sets, every prior-bearing one
    and two more."""
    from eddy_gpu import synth
    w = synth.make(3, seed=0, n_sets=30)
    sizes = [len(g) for _, g, _ in w.sets]
    idx = {int(np.argmin(sizes)), int(np.argmax(sizes)), 3, 7}
    idx |= {i for i, (_, _, p) in enumerate(w.sets) if p is not None}
    picks = [(w.sets[i][1], w.sets[i][2]) for i in sorted(idx)]
    assert any(p is not None for _, p in picks)
    _many_sets(eddy_lib, oracle_lib, w, picks, R=6, seed=3)


def test_config5_sample_in_one_context(eddy_lib, oracle_lib):
    """Config 5's shapes: a 20000 x 1000 matrix (log-normal, then log), sets
    of 5 to 300 genes (a 300-gene set, above the reference's 200-gene cap,
    the smallest set, and prior-bearing sets of the workload)."""
    from eddy_gpu import synth
    w = synth.make(5, seed=0, n_sets=40)
    sizes = [len(g) for _, g, _ in w.sets]
    rng = np.random.default_rng(5)
    big = np.sort(rng.choice(w.data.shape[0], 300, replace=False))
    picks = [(big, None), (w.sets[int(np.argmin(sizes))][1], w.sets[int(np.argmin(sizes))][2])]
    picks += [(g, p) for _, g, p in w.sets if p is not None][:2]
    _many_sets(eddy_lib, oracle_lib, w, picks, R=4, seed=5)


@pytest.mark.parametrize("cfg", [2, 4])
def test_edge_list_matches_oracle(cfg, eddy_lib, oracle_lib):
    """eddy_get_edge_list: the uncapped parents of networks 0 and S-1 of the
    unpermuted labelling equal the oracle's."""
    from eddy_gpu import synth
    O = oracle_lib
    w = synth.make(cfg, seed=0)
    _, genes, prior = w.sets[0]
    mp, pw = w.flags["mp"], w.flags["pw"]
    ctx = eddy_lib.Context(max_parents=mp, prior_weight=pw, permutations=2,
                           rng=eddy_lib.RNG_COUNTER, seed=1, keep_networks=True)
    ctx.load_matrix(w.data, w.labels)
    sid = ctx.add_set(genes, prior)
    ctx.run()
    el = ctx.edge_list(sid)
    data = w.data[genes]
    lab = w.labels
    e, _, _ = O.k1_edges(data[:, lab == 0], data[:, lab == 1], prior, O.params(mp=mp, pw=pw))
    S = e.shape[0]
    pn, epn, pe = O.parents(e[[0, S - 1]], len(genes), 1 << 30)
    assert np.array_equal(el["nodes"], pn)
    assert np.array_equal(el["epn"], epn)
    assert np.array_equal(el["edges"], pe)
    ctx.close()


def test_key_table_paths_agree(eddy_lib, oracle_lib, monkeypatch):
    """The unit kernel's table of distinct changed-node keys, built from the
    memo lists the records mark and the merged-row keys they log, and built
    by walking every unique network's records (EDDY_KEY_WALK=1, the path
    taken when the log overflows), give the same JS and U at the
    precision-stress shape, and agree with the oracle."""
    from eddy_gpu import synth
    O = oracle_lib
    w = synth.make(4, seed=1)
    genes = w.sets[0][1]
    mp, pw = w.flags["mp"], w.flags["pw"]
    out = []
    for walk in (False, True):
        if walk:
            monkeypatch.setenv("EDDY_KEY_WALK", "1")
        ctx = eddy_lib.Context(max_parents=mp, prior_weight=pw, permutations=65,
                               rng=eddy_lib.RNG_COUNTER, seed=9, keep_networks=False)
        ctx.load_matrix(w.data, w.labels)
        sid = ctx.add_set(genes)
        out.append(ctx.run_permutations(sid, 1, 64))
        ctx.close()
    monkeypatch.delenv("EDDY_KEY_WALK")
    (js0, U0), (js1, U1) = out
    assert np.array_equal(U0, U1)
    assert np.array_equal(js0, js1, equal_nan=True)
    labs = O.counter_labels(9, sid, w.labels, 65)
    ojs, oU = O.units(w.data[genes], labs[[1, 64]], None, O.params(mp=mp, pw=pw))
    assert np.array_equal(U0[[0, 63]], oU)
    assert _close(js0[[0, 63]], ojs)
