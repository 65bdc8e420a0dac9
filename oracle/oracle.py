"""ctypes bindings for the oracle (liboracle.so) and, where it was built, the
CPU build of the reference's own kernel/host-routine sources (_ref/).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libeddy_ref.so")

_i8p = np.ctypeslib.ndpointer(np.int8, flags="C")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C")


class Params(C.Structure):
    _fields_ = [("max_parents", C.c_int), ("alpha_edge", C.c_double),
                ("alpha_edge_prior", C.c_double), ("bonferroni", C.c_int)]


class UnitResult(C.Structure):
    _fields_ = [("js", C.c_double), ("U", C.c_int), ("S", C.c_int),
                ("total_edges", C.c_int), ("uni_edges_total", C.c_int)]


def build(ref: bool | None = None, ref_root: str | None = None) -> None:
    """Compile liboracle.so, and _ref/ from the reference sources under
    ref_root (or $EDDY_REFERENCE_ROOT) when that directory holds them."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    refroot = ref_root or os.environ.get("EDDY_REFERENCE_ROOT")
    have = bool(refroot) and os.path.isfile(os.path.join(refroot, "kernel1.cu"))
    if ref is None:
        ref = have
    if ref:
        if not have:
            raise FileNotFoundError("the reference sources were not found: pass ref_root "
                                    "or set EDDY_REFERENCE_ROOT")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={refroot}"],
                       check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(ref=False)
        L = C.CDLL(LIB)
        L.or_gammds.restype = C.c_double
        L.or_gammds.argtypes = [C.c_double, C.c_double]
        L.or_chisq.restype = C.c_double
        L.or_chisq.argtypes = [_i32p, C.POINTER(C.c_int)]
        L.or_edge_decision.restype = C.c_int
        L.or_edge_decision.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(Params)]
        L.or_k1_edges.restype = None
        L.or_k1_edges.argtypes = [C.c_int, C.c_int, C.c_int, _i8p, _i8p,
                                  C.c_void_p, C.POINTER(Params), _u8p,
                                  C.c_void_p, C.c_void_p]
        L.or_parents.restype = C.c_int
        L.or_parents.argtypes = [C.c_int, C.c_int, _u8p, C.c_int, _i32p,
                                 _i32p, C.c_void_p]
        L.or_unique.restype = C.c_int
        L.or_unique.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _i32p, _u8p]
        L.or_bdeu_node.restype = C.c_double
        L.or_bdeu_node.argtypes = [C.c_int, C.c_int, _i8p, _i32p, _i32p,
                                   C.c_int, C.c_int, _i32p]
        L.or_normalise.restype = None
        L.or_normalise.argtypes = [C.c_int, _f64p, _f64p]
        L.or_js.restype = C.c_double
        L.or_js.argtypes = [C.c_int, _f64p, _f64p]
        L.or_unit.restype = None
        L.or_unit.argtypes = [C.c_int, C.c_int, _i8p, _u8p, C.c_void_p,
                              C.POINTER(Params), C.POINTER(UnitResult)] + \
            [C.c_void_p] * 7
        L.or_units.restype = C.c_int
        L.or_units.argtypes = [C.c_int, C.c_int, _i8p, C.c_int, _u8p,
                               C.c_void_p, C.POINTER(Params), _f64p, _i32p,
                               C.c_int]
        L.or_glibc_labels.restype = None
        L.or_glibc_labels.argtypes = [C.c_int, C.c_int, _u8p, C.c_int, _u8p,
                                      C.c_int, C.c_int]
        L.or_glibc_rand_calls.restype = C.c_longlong
        L.or_counter_labels.restype = None
        L.or_counter_labels.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int,
                                        _u8p, C.c_int, _u8p]
        L.or_philox4x32_10.restype = None
        L.or_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.or_ibetac.restype = C.c_double
        L.or_ibetac.argtypes = [C.c_double, C.c_double, C.c_double]
        L.or_pddn.restype = C.c_int
        L.or_pddn.argtypes = [C.c_int, _f64p, C.POINTER(C.c_double),
                              C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib = L
    return _lib


def params(mp=3, alpha_edge=0.05, alpha_edge_prior=None, bonferroni=True,
           pw=0.5, lam=2.0) -> Params:
    if alpha_edge_prior is None:
        alpha_edge_prior = 1 - (1 - alpha_edge) * pw ** (1 / lam)
    return Params(int(mp), float(alpha_edge), float(alpha_edge_prior),
                  1 if bonferroni else 0)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def gammds(x, p):
    return lib().or_gammds(float(x), float(p))


def chisq(tally):
    t = np.ascontiguousarray(np.asarray(tally, np.int32).reshape(9))
    d = C.c_int()
    chi = lib().or_chisq(t, C.byref(d))
    return chi, d.value


def unit(data, labels, prior=None, prm=None, outputs=True):
    """One labelling of one gene set (data g x n int8, labels n 0/1)."""
    prm = prm or params()
    data = np.ascontiguousarray(data, np.int8)
    labels = np.ascontiguousarray(labels, np.uint8)
    g, n = data.shape
    S = n + 2
    c = g * (g - 1) // 2
    pr = None if prior is None else np.ascontiguousarray(prior, np.uint8)
    res = UnitResult()
    out = {}
    if outputs:
        mpc = min(prm.max_parents, max(g - 1, 1))
        out = dict(edges=np.zeros((S, c), np.uint8),
                   unique_ids=np.zeros(S, np.int32),
                   uni_nodes=np.zeros((S, g), np.int32),
                   uni_edges=np.zeros(S * g * mpc + 1, np.int32),
                   uni_epn=np.zeros(S + 1, np.int32),
                   out5=np.zeros(2 * S * g, np.float64),
                   lval=np.zeros(2 * S, np.float64))
    lib().or_unit(g, n, data, labels, _ptr(pr), C.byref(prm), C.byref(res),
                  *[_ptr(out.get(k)) for k in ("edges", "unique_ids",
                                              "uni_nodes", "uni_edges",
                                              "uni_epn", "out5", "lval")])
    r = dict(js=res.js, U=res.U, S=res.S, total_edges=res.total_edges)
    if outputs:
        U = res.U
        r.update(edges=out["edges"], unique_ids=out["unique_ids"][:U],
                 uni_nodes=out["uni_nodes"][:U],
                 uni_edges=out["uni_edges"][:res.uni_edges_total],
                 uni_epn=out["uni_epn"][:U + 1],
                 out5=out["out5"][:2 * U * g].reshape(2, U, g),
                 lval=out["lval"][:2 * U].reshape(2, U))
    return r


def units(data, labels, prior=None, prm=None, threads=0):
    prm = prm or params()
    data = np.ascontiguousarray(data, np.int8)
    labels = np.ascontiguousarray(labels, np.uint8)
    g, n = data.shape
    R = labels.shape[0]
    js = np.zeros(R, np.float64)
    U = np.zeros(R, np.int32)
    pr = None if prior is None else np.ascontiguousarray(prior, np.uint8)
    lib().or_units(g, n, data, R, labels, _ptr(pr), C.byref(prm), js, U,
                   int(threads))
    return js, U


def k1_edges(dA, dB, prior=None, prm=None):
    prm = prm or params()
    dA = np.ascontiguousarray(dA, np.int8)
    dB = np.ascontiguousarray(dB, np.int8)
    g, nA = dA.shape
    nB = dB.shape[1]
    S = nA + nB + 2
    c = g * (g - 1) // 2
    e = np.zeros((S, c), np.uint8)
    ppn = np.zeros(2 * g, np.int32)
    stf = np.zeros(6 * g, np.int32)
    pr = None if prior is None else np.ascontiguousarray(prior, np.uint8)
    lib().or_k1_edges(g, nA, nB, dA, dB, _ptr(pr), C.byref(prm), e,
                      _ptr(ppn), _ptr(stf))
    return e, ppn, stf


def parents(edges, g, max_parents):
    edges = np.ascontiguousarray(edges, np.uint8)
    nets = edges.shape[0]
    pn = np.zeros((nets, g), np.int32)
    epn = np.zeros(nets + 1, np.int32)
    tot = lib().or_parents(nets, g, edges, int(max_parents), pn, epn, None)
    pe = np.zeros(max(tot, 1), np.int32)
    lib().or_parents(nets, g, edges, int(max_parents), pn, epn, _ptr(pe))
    return pn, epn, pe[:tot]


def glibc_labels(n, n_class1, labels0, R, reset=True, first=0):
    """Iterations first .. first+R-1 of the reference's label stream."""
    out = np.zeros((R, n), np.uint8)
    lib().or_glibc_labels(int(n), int(n_class1),
                          np.ascontiguousarray(labels0, np.uint8), int(R), out,
                          1 if reset else 0, int(first))
    return out


def reference_stream(n, n_class1, labels0, R, js0_of_set, nsets):
    """Labellings of nsets consecutive gene sets as main.cu:359-573 draws
    them: one libc rand() stream, iteration 0 always consumes its draws, a
    NaN JS of iteration 0 stops the set (main.cu:1431-1435).
    js0_of_set(i, labels0) -> JS of iteration 0 of set i."""
    out = []
    for i in range(nsets):
        first = glibc_labels(n, n_class1, labels0, 1, reset=(i == 0), first=0)
        if np.isnan(js0_of_set(i, first[0])):
            out.append(first)
            continue
        rest = glibc_labels(n, n_class1, labels0, R - 1, reset=False, first=1) if R > 1 \
            else np.zeros((0, n), np.uint8)
        out.append(np.concatenate([first, rest]))
    return out


def counter_labels(seed, set_id, labels0, R):
    labels0 = np.ascontiguousarray(labels0, np.uint8)
    n = labels0.size
    nA = int((labels0 == 0).sum())
    out = np.zeros((R, n), np.uint8)
    lib().or_counter_labels(int(seed), int(set_id), n, nA, labels0, int(R), out)
    return out


def philox(ctr, key):
    o = np.zeros(4, np.uint32)
    lib().or_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), o)
    return o


def ibetac(a, b, x):
    return lib().or_ibetac(float(a), float(b), float(x))


def pddn(js):
    js = np.ascontiguousarray(js, np.float64)
    a, b, p = C.c_double(), C.c_double(), C.c_double()
    rc = lib().or_pddn(js.size, js, C.byref(a), C.byref(b), C.byref(p))
    return rc, a.value, b.value, p.value


# ------------------------------------------------------------------ _ref
def ref_available() -> bool:
    return os.path.exists(REFLIB)


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(REFLIB)
        L.ref_unit.restype = C.c_int
        L.ref_unit.argtypes = [C.c_int] * 3 + [_i32p, _i32p, _i32p,
                                               C.c_double, C.c_double,
                                               C.c_int, C.c_int] + \
            [C.c_void_p] * 6 + [C.c_int] + [C.c_void_p] * 8
        L.ref_uncapped.restype = C.c_int
        L.ref_uncapped.argtypes = [C.c_int, _i32p, _i32p, _i32p, _i32p, _i32p,
                                   C.c_int]
        L.ref_gammds.restype = C.c_double
        L.ref_gammds.argtypes = [C.c_double, C.c_double]
        L.ref_kool.restype = C.c_double
        L.ref_kool.argtypes = [_f64p, _f64p, C.c_int, C.c_int]
        L.ref_mean.restype = C.c_double
        L.ref_mean.argtypes = [_f64p, C.c_int]
        L.ref_variance.restype = C.c_double
        L.ref_variance.argtypes = [C.c_double, _f64p, C.c_int]
        L.ref_write_networks.restype = None
        L.ref_write_networks.argtypes = [C.c_char_p] * 4 + [C.c_int, _i32p,
                                                            C.c_char_p, C.c_int,
                                                            _i32p, _i32p,
                                                            C.c_int, _i32p]
        L.ref_write_bdeu.restype = None
        L.ref_write_bdeu.argtypes = [C.c_char_p] * 6 + [C.c_int, _f64p]
        L.ref_write_edge_list.restype = None
        L.ref_write_edge_list.argtypes = [C.c_char_p] * 5 + [C.c_int, _i32p,
                                                             _i32p, _i32p,
                                                             _i32p,
                                                             C.c_char_p,
                                                             C.c_char_p]
        _ref = L
    return _ref


def ref_unit(data, labels, prior=None, prm=None):
    """The reference's own kernels + host routines for one labelling."""
    prm = prm or params()
    data = np.ascontiguousarray(data, np.int32)
    labels = np.asarray(labels, np.uint8)
    g, n = data.shape
    tA = np.ascontiguousarray(data[:, labels == 0])
    tB = np.ascontiguousarray(data[:, labels == 1])
    nA, nB = tA.shape[1], tB.shape[1]
    S = nA + nB + 2
    c = g * (g - 1) // 2
    pr = np.zeros((g, g), np.int32) if prior is None else \
        np.ascontiguousarray(prior, np.int32)
    cap = S * g * max(1, min(prm.max_parents, g)) + 1
    o = dict(out23=np.zeros(S * c, np.int32), ppn=np.zeros(2 * g, np.int32),
             stf=np.zeros(6 * g, np.int32), edges_pn=np.zeros(S + 1, np.int32),
             pnodes=np.zeros(S * g, np.int32), pedges=np.zeros(cap, np.int32),
             unique_ids=np.zeros(S, np.int32),
             uni_nodes=np.zeros(S * g, np.int32),
             uni_edges=np.zeros(cap, np.int32),
             uni_epn=np.zeros(S + 1, np.int32),
             out5=np.zeros(2 * S * g, np.float64),
             lval=np.zeros(2 * S, np.float64), scal=np.zeros(4, np.int32),
             js=np.zeros(1, np.float64))
    rc = ref().ref_unit(g, nA, nB, tA, tB, pr, prm.alpha_edge,
                        prm.alpha_edge_prior, prm.bonferroni, prm.max_parents,
                        _ptr(o["out23"]), _ptr(o["ppn"]), _ptr(o["stf"]),
                        _ptr(o["edges_pn"]), _ptr(o["pnodes"]),
                        _ptr(o["pedges"]), cap, _ptr(o["unique_ids"]),
                        _ptr(o["uni_nodes"]), _ptr(o["uni_edges"]),
                        _ptr(o["uni_epn"]), _ptr(o["out5"]), _ptr(o["lval"]),
                        _ptr(o["scal"]), _ptr(o["js"]))
    if rc != 0:
        raise ValueError("ref_unit rejected the sizes")
    U, E, ue, S_ = (int(v) for v in o["scal"])
    return dict(js=float(o["js"][0]), U=U, S=S_, total_edges=E,
                edges=o["out23"].reshape(S, c).astype(np.uint8),
                ppn=o["ppn"], stf=o["stf"], edges_pn=o["edges_pn"],
                pnodes=o["pnodes"].reshape(S, g), pedges=o["pedges"][:E],
                unique_ids=o["unique_ids"][:U],
                uni_nodes=o["uni_nodes"][:U * g].reshape(U, g),
                uni_edges=o["uni_edges"][:ue], uni_epn=o["uni_epn"][:U + 1],
                out5=o["out5"][:2 * U * g].reshape(2, U, g),
                lval=o["lval"][:2 * U].reshape(2, U))


def ref_uncapped(g, net0, net1):
    nodes = np.zeros(2 * g, np.int32)
    epn = np.zeros(3, np.int32)
    cap = g * g + 1
    edges = np.zeros(cap, np.int32)
    tot = ref().ref_uncapped(g, np.ascontiguousarray(net0, np.int32),
                             np.ascontiguousarray(net1, np.int32), nodes, epn,
                             edges, cap)
    return nodes.reshape(2, g), epn, edges[:tot]
