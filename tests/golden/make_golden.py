"""Generates the golden fixtures of this directory from the reference itself.

Runs the reference's own kernel sources (kernel1.cu .. kernel5.cu) and host
routines (routines.cu), compiled for the CPU by oracle/Makefile's `ref`
target (a CUDA-thread emulator drives the unchanged kernel bodies), on small
seeded inputs that cover the edge cases of the hot path:
  run2 (c < 1024) and run2Scalable (c >= 1024) launch shapes, Bonferroni on
  and off, priors with -pw 0.5 and -pw 0 (alphaEdgePrior = 1), -mp 1..4
  (the BDeu 3-parent cap), values outside {-1,0,1}, tiny tables (Yates,
  dof 0), and a set whose networks are all identical (U = 1, NaN JS).
Writes units.npz (inputs and every intermediate the kernels produce),
gammds.npz (the host AS 147 twin on a grid) and writers.json (output files
of the reference's writers).  Only runnable where the reference sources
exist; the fixtures it writes are committed.

    EDDY_REFERENCE_ROOT=<reference root> python tests/golden/make_golden.py
"""
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def tern(rng, g, n, planted=3, w=0.8, noise=0.5, nA=None, invalid=0.0):
    x = rng.standard_normal((g, n))
    nA = n // 2 if nA is None else nA
    for k in range(min(planted, g // 2)):
        x[g - 1 - k, :nA] = w * x[k, :nA] + noise * rng.standard_normal(nA)
    s = np.sort(x, axis=1)
    t1 = s[:, int(np.ceil(n / 3)) - 1][:, None]
    t2 = s[:, int(np.ceil(2 * n / 3)) - 1][:, None]
    d = np.where(x <= t1, -1, np.where(x <= t2, 0, 1)).astype(np.int8)
    if invalid:
        d[rng.random(d.shape) < invalid] = 7
    return d


def prior_pairs(rng, g, k):
    pr = np.zeros((g, g), np.uint8)
    for _ in range(k):
        i, j = rng.choice(g, 2, replace=False)
        pr[i, j] = pr[j, i] = 1
    return pr


# name, g, n, nA, mp, bonferroni, pw, prior pairs, invalid fraction, planted,
# alpha_edge, planted weight, noise
CASES = [
    ("A_bonferroni", 8, 60, 30, 3, True, 0.5, 0, 0.0, 3, 0.3, 0.8, 0.4),
    ("B_prior_rawp", 12, 40, 18, 2, False, 0.5, 6, 0.0, 3, 0.2, 0.8, 0.4),
    ("C_pw0_prior", 20, 60, 30, 3, True, 0.0, 8, 0.0, 4, 0.05, 0.8, 0.4),
    ("D_scalable", 50, 24, 12, 4, False, 0.5, 0, 0.0, 6, 0.1, 0.8, 0.4),
    ("E_invalid", 16, 50, 25, 3, False, 0.5, 4, 0.06, 4, 0.2, 0.5, 1.0),
    ("F_mp4_dense", 10, 40, 20, 4, False, 0.5, 0, 0.0, 5, 0.3, 0.5, 1.0),
    ("G_no_edges", 6, 20, 10, 3, True, 0.5, 0, 0.0, 0, 0.05, 0.8, 0.4),
    ("H_tiny", 6, 16, 8, 3, False, 0.5, 2, 0.0, 2, 0.3, 0.8, 0.4),
    ("I_mp1", 14, 36, 20, 1, False, 0.5, 0, 0.0, 4, 0.2, 0.5, 1.0),
]


def main():
    if not O.ref_available():
        O.build(ref=True)
    rng = np.random.default_rng(20241203)
    store = {}
    meta = []
    for ci, (name, g, n, nA, mp, bonf, pw, npr, inv, planted, alpha, w, noise) in \
            enumerate(CASES):
        data = tern(rng, g, n, planted=planted, w=w, noise=noise, nA=nA, invalid=inv)
        pr = prior_pairs(rng, g, npr) if npr else np.zeros((g, g), np.uint8)
        prm = O.params(mp=mp, bonferroni=bonf, pw=pw, alpha_edge=alpha)
        labs = [np.concatenate([np.zeros(nA, np.uint8), np.ones(n - nA, np.uint8)])]
        perm = np.ones(n, np.uint8)
        perm[rng.choice(n, nA, replace=False)] = 0
        labs.append(perm)
        for li, lab in enumerate(labs):
            r = O.ref_unit(data, lab, pr, prm)
            key = f"{name}_{li}"
            store[key + "_data"] = data
            store[key + "_labels"] = lab
            store[key + "_prior"] = pr
            store[key + "_params"] = np.array([mp, prm.alpha_edge, prm.alpha_edge_prior,
                                               prm.bonferroni], np.float64)
            store[key + "_edges"] = np.packbits(r["edges"], axis=None)
            store[key + "_edges_shape"] = np.array(r["edges"].shape, np.int64)
            for k in ("ppn", "stf", "edges_pn", "pnodes", "pedges", "unique_ids", "uni_nodes",
                      "uni_edges", "uni_epn", "out5", "lval"):
                store[key + "_" + k] = r[k]
            store[key + "_scal"] = np.array([r["U"], r["total_edges"], r["S"]], np.int64)
            store[key + "_js"] = np.array([r["js"]], np.float64)
            meta.append(key)
    store["cases"] = np.array(meta)
    np.savez_compressed(os.path.join(HERE, "units.npz"), **store)

    # host AS 147 twin (routines.cu:117-184) on a grid
    xs = np.concatenate([np.geomspace(1e-6, 120, 60), [0.0, -1.0, 85.0, 88.0, 90.0, 95.0]])
    ps = np.array([0.0, 0.5, 1.0, 2.0, 1.5, 3.0])
    vals = np.array([[O.ref().ref_gammds(float(x), float(p)) for p in ps] for x in xs])
    np.savez_compressed(os.path.join(HERE, "gammds.npz"), x=xs, p=ps, value=vals)

    # the reference's writers on the networks of case C (iteration 0)
    name = "B_prior_rawp_0"
    data, lab, pr = store[name + "_data"], store[name + "_labels"], store[name + "_prior"]
    g = data.shape[0]
    genes = [f"GENE{i:03d}" for i in range(g)]
    names = np.zeros((g, 50), np.uint8)
    for i, s in enumerate(genes):
        names[i, :len(s)] = np.frombuffer(s.encode(), np.uint8)
    nb = names.tobytes()
    U = int(store[name + "_scal"][0])
    e = np.unpackbits(store[name + "_edges"])[:int(np.prod(store[name + "_edges_shape"]))]
    e = e.reshape(store[name + "_edges_shape"]).astype(np.int32)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        p1, p2, p3 = (os.path.join(td, f) for f in ("net.txt", "bdeu.txt", "el.txt"))
        uepn = store[name + "_uni_epn"].astype(np.int32)
        O.ref().ref_write_networks(p1.encode(), b"expr.txt", b"class.txt", b"SETC", U,
                                   np.ascontiguousarray(uepn[:U]), nb, g,
                                   np.ascontiguousarray(store[name + "_uni_nodes"].ravel()),
                                   np.ascontiguousarray(store[name + "_uni_edges"]),
                                   int(uepn[U]),
                                   np.ascontiguousarray(store[name + "_unique_ids"]))
        O.ref().ref_write_bdeu(p2.encode(), b"expr.txt", b"class.txt", b"SETC", b"CLASS_A",
                               b"CLASS_B", U, np.ascontiguousarray(store[name + "_lval"].ravel()))
        nodes, epn, edges = O.ref_uncapped(g, e[0], e[-1])
        O.ref().ref_write_edge_list(p3.encode(), b"expr.txt", b"class.txt", b"SETC", nb, g,
                                    np.ascontiguousarray(nodes.ravel()), edges, epn,
                                    np.ascontiguousarray(pr.astype(np.int32)), b"CLASS_A",
                                    b"CLASS_B")
        for k, p in (("networks", p1), ("bdeu", p2), ("edgelist", p3)):
            with open(p) as f:
                out[k] = f.read()
    out["case"] = name
    out["genes"] = genes
    out["uncapped"] = dict(nodes=nodes.tolist(), epn=epn.tolist(), edges=edges.tolist())
    with open(os.path.join(HERE, "writers.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(meta), "units,", os.path.getsize(os.path.join(HERE, "units.npz")), "bytes")


if __name__ == "__main__":
    main()
