"""The exact FP64 decision path against the oracle.  With
EDDY_DECISIONS=fp64 every table of every pair is decided by the
reference's FP64 formula (kernel1.cu:121-203, 10-74, 419-431: Yates,
chi-square, the AS 147 series, Bonferroni), with no FP32 fast path and no
leave-one-out filter, so the quotient and series arithmetic of that path
decides every edge of every network: the edge decisions must be identical
to the oracle's, and the units' unique counts and JS as in the parity
tests."""
import numpy as np
import pytest

from test_gpu_parity import _prior, js_close, make_labels, planted

pytestmark = pytest.mark.gpu

CASES = [
    # g, n, nA, mp, bonf, pw, nprior, strength: weak and strong planted
    # dependencies put chi-square values near the thresholds and past the
    # AS 147 underflow cliff
    (12, 60, 30, 3, True, 0.5, 4, 0.8),
    (16, 150, 70, 3, False, 0.5, 0, 0.5),
    (20, 400, 180, 4, True, 0.0, 0, 2.0),
]


@pytest.mark.parametrize("case", CASES)
def test_fp64_form_edges_and_units(case, eddy_lib, oracle_lib, monkeypatch):
    monkeypatch.setenv("EDDY_DECISIONS", "fp64")
    g, n, nA, mp, bonf, pw, npr, w = case
    rng = np.random.default_rng(7000 + g)
    data = planted(rng, g, n, nA=nA, planted=g // 3, w=w, noise=0.4)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    pr = _prior(rng, g, npr) if npr else None
    O = oracle_lib
    prm = O.params(mp=mp, bonferroni=bonf, pw=pw)
    ctx = eddy_lib.Context(max_parents=mp, bonferroni=bonf, prior_weight=pw,
                           rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g), pr)
    labs = np.stack([labels0] + [make_labels(rng, n, nA) for _ in range(5)])
    for lab in labs[:2]:
        e_gpu = ctx.debug_edges(sid, lab)
        e_or, _, _ = O.k1_edges(data[:, lab == 0], data[:, lab == 1], pr, prm)
        bad = np.argwhere(e_gpu != e_or)
        assert bad.size == 0, f"{len(bad)} edge decisions differ, first {bad[:5]}"
    js, U = ctx.run_labellings(sid, labs)
    ojs, oU = O.units(data, labs, pr, prm)
    assert np.array_equal(U, oU)
    assert js_close(js, ojs)
