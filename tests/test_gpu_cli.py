"""The eddy CLI as a drop-in for the reference's ./eddy on a GB300: config 1
and config 2 inputs written in the reference's file formats, the reference's
glibc permutation stream, printed lines and output files (_Networks,
_BDEU_SCORES and _EdgeList) checked against the oracle driven by the same
stream."""
import os
import re
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CLI = os.path.join(ROOT, "eddy-gpu_gb300", "bin", "eddy")


def _run_cli(tmp, files, extra):
    cmd = [CLI, "-d", files["d"], "-c", files["c"], "-g", files["g"]] + extra
    r = subprocess.run(cmd, cwd=tmp, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("cfg,R", [(1, 40), (2, 30)])
def test_cli_matches_oracle(cfg, R, eddy_lib, oracle_lib, tmp_path):
    from eddy_gpu import synth
    O = oracle_lib
    w = synth.make(cfg, seed=0)
    files = synth.write_files(w, str(tmp_path))
    mp, pw = w.flags["mp"], w.flags["pw"]
    out = _run_cli(str(tmp_path), files, ["-mp", str(mp), "-r", str(R), "-pw", str(pw),
                                          "-pD", "1.0"])
    name, genes, prior = w.sets[0]
    prm = O.params(mp=mp, pw=pw)
    data = w.data[genes]
    streams = O.reference_stream(data.shape[1], int((w.labels == 0).sum()), w.labels, R,
                                 lambda i, l0: O.unit(data, l0, prior, prm, outputs=False)["js"],
                                 1)
    ojs, oU = O.units(data, streams[0], prior, prm)
    u0 = int(re.search(r"Original Number of unique Networks : (\d+)", out).group(1))
    assert u0 == oU[0]
    res = open(os.path.join(str(tmp_path), "results.txt")).read().split("\n")
    assert res[0] == "Pathway\tJS\tPval\tnGenes"
    if np.isnan(ojs).any():
        # a NaN JS in any iteration fails the set (main.cu:1465-1479)
        assert "nan value- quiting!" in out
        assert res[1] == f"{name} failed with {len(genes)} genes- one of the js scores was nan"
        return
    js0 = float(re.search(r"Original JS : ([0-9.eE+-]+)", out).group(1))
    assert abs(js0 - ojs[0]) <= 2e-6
    rc, a, b, p = O.pddn(ojs)
    pd = float(re.search(r"pDDN = ([0-9.eE+nan-]+)", out).group(1))
    assert abs(pd - p) <= 2e-6, (pd, p)
    f = res[1].split("\t")
    assert f[0] == name and int(f[3]) == len(genes)
    # -pD 1.0: every set is significant -> the three files exist and the
    # networks file carries the oracle's iteration-0 unique networks
    u = O.unit(data, w.labels, prior, prm)
    gn = [files["genes"][i] for i in genes]
    net = dict(U=u["U"], ids=u["unique_ids"], nodes=u["uni_nodes"], epn=u["uni_epn"],
               edges=u["uni_edges"])
    ref_path = os.path.join(str(tmp_path), "expected_networks.txt")
    eddy_lib.write_networks(ref_path, files["d"], files["c"], name, net, gn)
    got = open(os.path.join(str(tmp_path), name + "_Networks.txt")).read()
    assert got == open(ref_path).read()
    b = open(os.path.join(str(tmp_path), name + "_BDEU_SCORES.txt")).read().split("\n")
    vals = np.array([[float(x) for x in ln.split("\t")[1:3]] for ln in b if ln.startswith("Network ")
                     and ln[8].isdigit()])
    assert np.allclose(vals, u["lval"].T, atol=2e-6)
    # _EdgeList.txt: the oracle's uncapped parent lists of iteration 0's two
    # full-data networks (main.cu:1530-1641) through the reference-format
    # writer, byte for byte
    e = u["edges"]
    S = e.shape[0]
    pn, epn, pe = O.parents(e[[0, S - 1]], len(genes), 1 << 30)
    exp_el = os.path.join(str(tmp_path), "expected_edgelist.txt")
    eddy_lib.write_edge_list(exp_el, gn, dict(nodes=pn, edges=pe, epn=epn), prior, "CLASS_A",
                             "CLASS_B")
    got_el = open(os.path.join(str(tmp_path), name + "_EdgeList.txt")).read()
    assert got_el == open(exp_el).read()
