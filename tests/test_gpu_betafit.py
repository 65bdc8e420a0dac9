"""The beta fit and pDDN of every set of one eddy_run call (main.cu:
1488-1502, routines.cu:494-508), from the JS values the GPU computed.
alpha and beta must equal, bit for bit, the reference's sequential moment
loop run here in Python on the same JS values; pDDN agrees with the
oracle's continued fraction (and scipy's betaincc) to 1e-10 relative.  A
set whose JS is NaN (no fit) between fitted sets leaves the others intact,
and sets added after an earlier run are fitted in their own run."""
import numpy as np
import pytest

from test_gpu_parity import planted

pytestmark = pytest.mark.gpu

PDDN_RTOL = 1e-10


def _moments(js):
    """routines.cu:494-508 / main.cu:1491-1495 in the reference's order."""
    s = 0.0
    for x in js:
        s += float(x)
    mu = s / len(js)
    v = 0.0
    for x in js:
        d = float(x) - mu
        v += d * d
    var = v / len(js)
    a = (((1 - mu) / var) - (1 / mu)) * (mu * mu)
    return a, a * (1 / mu - 1)


def _check(ctx, sid, oracle_lib):
    s = ctx.summary(sid)
    js, _ = ctx.js(sid)
    assert bool(s["failed"]) == bool(np.isnan(js).any())
    if s["failed"]:
        assert s["betafit_ok"] == 0
        return False
    a, b = _moments(js)
    assert s["alpha"] == a and s["beta"] == b
    rc, oa, ob, op = oracle_lib.pddn(np.asarray(js, np.float64))
    assert rc == 0 and s["betafit_ok"] == 1
    assert oa == a and ob == b
    assert abs(s["pddn"] - op) <= PDDN_RTOL * abs(op) + 1e-300
    try:
        from scipy.special import betaincc
    except ImportError:
        return True
    ref = betaincc(a, b, js[0])
    assert abs(s["pddn"] - ref) <= 1e-8 * abs(ref) + 1e-300
    return True


def _data(rng, G, n, nA):
    # planted class-0 dependencies: gene G-1-k on gene k, k < 12; genes 20
    # and 21 constant (a set of them has one network: JS NaN)
    data = planted(rng, G, n, nA=nA, planted=12, w=0.9, noise=0.3)
    data[20:22, :] = 0
    labels0 = np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])
    return data, labels0


def _set(rng, G, pairs, extra):
    genes = [g for k in pairs for g in (k, G - 1 - k)]
    pool = [g for g in range(12, G - 12) if g not in (20, 21)]
    return np.array(genes + list(rng.choice(pool, extra, replace=False)))


@pytest.mark.parametrize("rng_mode", ["counter", "glibc"])
def test_many_sets_in_one_run(eddy_lib, oracle_lib, rng_mode):
    rng = np.random.default_rng(41)
    G, n, nA = 60, 160, 70
    data, labels0 = _data(rng, G, n, nA)
    R = 48
    mode = eddy_lib.RNG_COUNTER if rng_mode == "counter" else eddy_lib.RNG_GLIBC
    ctx = eddy_lib.Context(max_parents=3, permutations=R, rng=mode, seed=5)
    ctx.load_matrix(data, labels0)
    sids = [ctx.add_set(_set(rng, G, [0, 1, 2], 0)),
            ctx.add_set(_set(rng, G, [3, 4], 8)),
            ctx.add_set(_set(rng, G, [5, 6, 7], 14)),
            ctx.add_set(np.array([20, 21])),  # NaN JS: no fit
            ctx.add_set(_set(rng, G, [8, 9, 10, 11], 22)),
            ctx.add_set(_set(rng, G, [0, 5], 5))]
    ctx.run()
    fitted = [_check(ctx, sid, oracle_lib) for sid in sids]
    assert fitted[3] is False
    # (a set with one identical-network permutation has a NaN JS: no fit)
    assert sum(fitted) >= (2 if rng_mode == "counter" else 1)


def test_fit_after_earlier_runs(eddy_lib, oracle_lib):
    """Sets added after an earlier eddy_run are fitted in their own run."""
    rng = np.random.default_rng(42)
    G, n, nA = 40, 120, 60
    data, labels0 = _data(rng, G, n, nA)
    # (seed 10: no permutation of either set has a single unique network,
    # so both sets are fitted)
    ctx = eddy_lib.Context(max_parents=3, permutations=32, rng=eddy_lib.RNG_COUNTER, seed=10)
    ctx.load_matrix(data, labels0)
    a = ctx.add_set(_set(rng, G, [0, 1, 2], 4))
    ctx.run()
    first = ctx.summary(a)
    b = ctx.add_set(_set(rng, G, [3, 4, 5], 6))
    ctx.run()
    again = ctx.summary(a)
    assert again.keys() == first.keys()
    for k in first:
        assert again[k] == first[k] or (np.isnan(again[k]) and np.isnan(first[k])), k
    assert _check(ctx, a, oracle_lib) and _check(ctx, b, oracle_lib)
