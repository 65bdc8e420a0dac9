"""Parity at the benchmark's full sizes (200 genes x 1000 samples, -mp 4,
config 2: 40 x 400 with priors), the oracle running on all host cores.
Edge decisions of all 1002 leave-one-out networks and unique-network
counts must be identical; JS within 1e-5 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return (np.isclose(a, b, rtol=1e-5, atol=1e-9) | (np.isnan(a) & np.isnan(b))).all()


@pytest.mark.parametrize("cfg", [2, 4])
def test_full_size_units(cfg, eddy_lib, oracle_lib):
    from eddy_gpu import synth
    O = oracle_lib
    w = synth.make(cfg, seed=0)
    name, genes, prior = w.sets[0]
    mp, pw = w.flags["mp"], w.flags["pw"]
    prm = O.params(mp=mp, pw=pw)
    lab = O.counter_labels(99, 0, w.labels, 3)
    ctx = eddy_lib.Context(max_parents=mp, prior_weight=pw, permutations=3,
                           rng=eddy_lib.RNG_EXTERNAL)
    ctx.load_matrix(w.data, w.labels)
    sid = ctx.add_set(genes, prior)
    data = w.data[genes]
    # every edge decision of every network of one permuted labelling
    e_gpu = ctx.debug_edges(sid, lab[1])
    e_or, _, _ = O.k1_edges(data[:, lab[1] == 0], data[:, lab[1] == 1], prior, prm)
    assert np.array_equal(e_gpu, e_or)
    js, U = ctx.run_labellings(sid, lab)
    ojs, oU = O.units(data, lab, prior, prm)
    assert np.array_equal(U, oU), (U, oU)
    assert _close(js, ojs), (js, ojs)
