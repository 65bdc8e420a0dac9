"""Output files and host-side pieces of the drop-in boundary (no GPU).

The library's writers are compared byte for byte with the output of the
reference's own writers (routines.cu:217-492, compiled and run by
tests/golden/make_golden.py) on the same networks."""
import json
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden")


def _case():
    w = json.load(open(os.path.join(GOLD, "writers.json")))
    z = np.load(os.path.join(GOLD, "units.npz"))
    return w, z, w["case"]


def test_writers_match_reference_bytes(eddy_lib, tmp_path):
    w, z, key = _case()
    U = int(z[key + "_scal"][0])
    epn = z[key + "_uni_epn"].astype(np.int32)
    net = dict(U=U, ids=z[key + "_unique_ids"], nodes=z[key + "_uni_nodes"], epn=epn,
               edges=z[key + "_uni_edges"])
    genes = w["genes"]
    p1, p2, p3 = (str(tmp_path / f) for f in ("n.txt", "b.txt", "e.txt"))
    eddy_lib.write_networks(p1, "expr.txt", "class.txt", "SETC", net, genes)
    assert open(p1).read() == w["networks"]
    eddy_lib.write_bdeu(p2, "expr.txt", "class.txt", "SETC", "CLASS_A", "CLASS_B",
                        z[key + "_lval"])
    assert open(p2).read() == w["bdeu"]
    el = w["uncapped"]
    eddy_lib.write_edge_list(p3, genes, dict(nodes=np.array(el["nodes"]), epn=np.array(el["epn"]),
                                             edges=np.array(el["edges"])),
                             z[key + "_prior"], "CLASS_A", "CLASS_B")
    assert open(p3).read() == w["edgelist"]


def test_library_exports_every_declared_symbol(eddy_lib):
    """libeddy_gpu.so loads without a GPU and exports each entry point of
    include/eddy_gpu.h (no compute call is made)."""
    hdr = open(os.path.join(ROOT, "include", "eddy_gpu.h")).read()
    declared = set(re.findall(r"^\s*(?:int|const char \*)\s*(eddy_\w+)\(", hdr, re.M))
    L = eddy_lib.library()
    for name in sorted(declared):
        assert hasattr(L, name), name
    assert declared == set(eddy_lib.EXPORTS), declared ^ set(eddy_lib.EXPORTS)


def test_ctx_without_device_fails_cleanly(eddy_lib):
    """No CUDA device (this container): creation reports EDDY_ERR_CUDA, no crash."""
    from conftest import has_gpu
    if has_gpu():
        return
    try:
        eddy_lib.Context()
    except eddy_lib.EddyError as e:
        assert "EDDY_ERR_CUDA" in str(e)
    else:
        raise AssertionError("context created without a GPU")


def test_synth_tertiles_and_files(tmp_path):
    from eddy_gpu import synth
    x = np.random.default_rng(0).standard_normal((5, 300))
    d = synth.tertiles(x)
    for row in d:
        counts = np.bincount(row + 1, minlength=3)
        assert counts.tolist() == [100, 100, 100]
    w = synth.make(2, seed=0)
    f = synth.write_files(w, str(tmp_path))
    lines = open(f["d"]).read().split("\n")
    assert lines[0].startswith("gene_id\tS00000\t")
    assert lines[-2] == "" and lines[-1] == ""  # trailing blank line (main.cu:276-283)
    assert len(lines) == 1 + w.data.shape[0] + 2
    cls = open(f["c"]).read().rstrip("\n").split("\t")
    assert cls.count("CLASS_A") == 150 and cls.count("CLASS_B") == 250
    gmt = open(f["g"]).read().split("\n")[0].split("\t")
    assert gmt[0] == "SET2" and len(gmt) == 2 + 40
    prior = open(os.path.join(str(tmp_path), "PRIORS", "SET2.prior")).read().strip().split("\n")
    assert len(prior) == 30 and prior[0].split("\t")[1] == "pp"
