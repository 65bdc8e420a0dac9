"""eddy_unit_noalloc, the entry point for callers that may not allocate GPU
memory (a host application owning all device memory through its own pool,
or a pipeline that must avoid cudaFree's device-wide synchronisation): it
runs one labelling with every intermediate in a fixed array compiled into
the library.  Its results must equal the allocating entry point's
(eddy_run_labellings) and the oracle's on the same inputs, on two calls in
a row, up to its limit shape (64 genes x 2048 samples); sizes past that
limit are refused.  This file is collected last so a stop-at-first-failure
run has run everything else first."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

JS_RTOL, JS_ATOL = 1e-5, 1e-9


def _data(rng, g, n, nA):
    from eddy_gpu import synth
    x = rng.standard_normal((g, n))
    for k in range(4):
        x[g - 1 - k, :nA] = 0.8 * x[k, :nA] + 0.5 * rng.standard_normal(nA)
    return synth.tertiles(x)


@pytest.mark.parametrize("g,n,nA,mp,bonf,npr", [(20, 200, 100, 3, False, 4),
                                                 (48, 300, 120, 4, True, 0),
                                                 (64, 2048, 900, 3, True, 6)])
def test_noalloc_matches_allocating_entry_point(g, n, nA, mp, bonf, npr, eddy_lib,
                                                oracle_lib):
    rng = np.random.default_rng(g * 31 + n)
    data = _data(rng, g, n, nA)
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    pr = None
    if npr:
        pr = np.zeros((g, g), np.uint8)
        for _ in range(npr):
            i, j = rng.choice(g, 2, replace=False)
            pr[i, j] = pr[j, i] = 1
    ctx = eddy_lib.Context(max_parents=mp, bonferroni=bonf, rng=eddy_lib.RNG_EXTERNAL,
                           prior_weight=0.5)
    ctx.load_matrix(data, labels0)
    sid = ctx.add_set(np.arange(g), pr)
    labs = []
    for t in range(2):
        lab = np.ones(n, np.uint8)
        lab[rng.choice(n, nA, replace=False)] = 0
        labs.append(lab)
    ref_js, ref_U = ctx.run_labellings(sid, np.stack(labs))
    prm = oracle_lib.params(mp=mp, pw=0.5, bonferroni=bonf)
    o_js, o_U = oracle_lib.units(data, np.stack(labs), pr, prm)

    def close(a, b):
        return (np.isnan(a) and np.isnan(b)) or abs(a - b) <= JS_RTOL * abs(b) + JS_ATOL

    for t in range(2):  # two calls in a row share the fixed array
        js, U = eddy_lib.unit_noalloc(ctx.opts, data, labs[t], pr)
        assert U == ref_U[t] == o_U[t], (U, ref_U[t], o_U[t])
        assert close(js, ref_js[t]), (js, ref_js[t])
        assert close(js, o_js[t]), (js, o_js[t])
    ctx.close()


def test_noalloc_refuses_sizes_past_its_limit(eddy_lib):
    rng = np.random.default_rng(1)
    opts = eddy_lib.Opts(3, 0.05, 0.33, 1, 1, eddy_lib.RNG_EXTERNAL, 0, 0, 0)
    lab = np.concatenate([np.zeros(10, np.uint8), np.ones(10, np.uint8)])
    with pytest.raises(eddy_lib.EddyError, match="CAPACITY"):
        eddy_lib.unit_noalloc(opts, _data(rng, 65, 20, 10), lab)
    lab = np.concatenate([np.zeros(1100, np.uint8), np.ones(1000, np.uint8)])
    with pytest.raises(eddy_lib.EddyError, match="CAPACITY"):
        eddy_lib.unit_noalloc(opts, _data(rng, 8, 2100, 1100), lab)
