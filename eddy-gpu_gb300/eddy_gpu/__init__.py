"""Python host binding of libeddy_gpu (the C ABI declared in include/eddy_gpu.h).

Mirrors the reference's process-level interface (main.cu:27-1711) as calls:
load the ternary matrix and labels, add gene sets with their prior matrices,
run the permutation test, read JS / pDDN / unique-network counts and the
iteration-0 networks.  Every call goes to the CUDA library; there is no
Python or CPU implementation of the hot path here, and loading fails loudly
when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libeddy_gpu.so")

RNG_GLIBC, RNG_COUNTER, RNG_EXTERNAL = 0, 1, 2
ERRORS = {1: "EDDY_ERR_ARG", 2: "EDDY_ERR_CUDA", 3: "EDDY_ERR_STATE",
          4: "EDDY_ERR_CAPACITY", 5: "EDDY_ERR_BETAFIT", 6: "EDDY_ERR_INTERNAL"}

# every symbol include/eddy_gpu.h declares
EXPORTS = ["eddy_ctx_create", "eddy_ctx_destroy", "eddy_last_error", "eddy_load_matrix",
           "eddy_add_set", "eddy_set_labellings", "eddy_run", "eddy_get_set_summary",
           "eddy_get_js", "eddy_get_networks", "eddy_get_edge_list", "eddy_run_labellings",
           "eddy_debug_edges", "eddy_debug_unit", "eddy_run_permutations",
           "eddy_set_stream", "eddy_clear_sets", "eddy_write_networks", "eddy_write_bdeu",
           "eddy_write_edge_list", "eddy_unit_noalloc", "eddy_last_stats", "eddy_device_info",
           "eddy_last_timing", "eddy_last_stage_timing"]


class Opts(C.Structure):
    _fields_ = [("max_parents", C.c_int), ("alpha_edge", C.c_double),
                ("alpha_edge_prior", C.c_double), ("bonferroni", C.c_int),
                ("permutations", C.c_int), ("rng", C.c_int), ("seed", C.c_uint64),
                ("device", C.c_int), ("keep_networks", C.c_int)]


class Summary(C.Structure):
    _fields_ = [("genes", C.c_int), ("iterations", C.c_int), ("failed", C.c_int),
                ("betafit_ok", C.c_int), ("unique0", C.c_int), ("js0", C.c_double),
                ("alpha", C.c_double), ("beta", C.c_double), ("pddn", C.c_double),
                ("exact_rechecks", C.c_uint64), ("tables", C.c_uint64)]


class EddyError(RuntimeError):
    pass


_lib = None


def library(path: str | None = None):
    """Loads libeddy_gpu.so; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise EddyError(f"libeddy_gpu.so not built ({p}); run eddy-gpu_gb300/build.py")
    L = C.CDLL(p)
    vp = C.c_void_p
    L.eddy_ctx_create.argtypes = [C.POINTER(Opts), C.POINTER(vp)]
    L.eddy_ctx_destroy.argtypes = [vp]
    L.eddy_last_error.restype = C.c_char_p
    L.eddy_last_error.argtypes = [vp]
    L.eddy_load_matrix.argtypes = [vp, vp, C.c_int, C.c_int, vp]
    L.eddy_add_set.argtypes = [vp, vp, C.c_int, vp, C.POINTER(C.c_int)]
    L.eddy_set_labellings.argtypes = [vp, C.c_int, vp, C.c_int]
    L.eddy_run.argtypes = [vp]
    L.eddy_get_set_summary.argtypes = [vp, C.c_int, C.POINTER(Summary)]
    L.eddy_get_js.argtypes = [vp, C.c_int, vp, vp]
    L.eddy_get_networks.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    vp, vp, vp, vp, vp]
    L.eddy_get_edge_list.argtypes = [vp, C.c_int, C.POINTER(C.c_int), vp, vp, vp]
    L.eddy_run_labellings.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp]
    L.eddy_debug_edges.argtypes = [vp, C.c_int, vp, vp]
    L.eddy_debug_unit.argtypes = [vp, C.c_int, vp, C.c_int, C.POINTER(C.c_int),
                                  C.POINTER(C.c_double), vp, vp, vp, vp, vp]
    L.eddy_run_permutations.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp]
    L.eddy_set_stream.argtypes = [vp, vp]
    L.eddy_clear_sets.argtypes = [vp]
    L.eddy_unit_noalloc.argtypes = [C.POINTER(Opts), vp, C.c_int, C.c_int, vp, vp, vp,
                                     C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    cp = C.c_char_p
    L.eddy_write_networks.argtypes = [cp, cp, cp, cp, C.c_int, vp, vp, C.c_int, vp, vp, C.c_int,
                                      vp]
    L.eddy_write_bdeu.argtypes = [cp, cp, cp, cp, cp, cp, C.c_int, vp]
    L.eddy_write_edge_list.argtypes = [cp, vp, C.c_int, vp, vp, vp, vp, cp, cp]
    L.eddy_last_stats.argtypes = [vp, vp, C.POINTER(C.c_int)]
    L.eddy_last_timing.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    L.eddy_last_stage_timing.argtypes = [vp, C.POINTER(C.c_double)]
    _lib = L
    return L


def write_networks(path, input_name, class_name, set_name, net: dict, genes):
    """<set>_Networks.txt from eddy_get_networks() output (routines.cu:240-306)."""
    L = library()
    g = len(genes)
    names = (C.c_char_p * g)(*[s.encode() for s in genes])
    epn = np.ascontiguousarray(net["epn"], np.int32)
    nodes = np.ascontiguousarray(net["nodes"], np.int32).ravel()
    edges = np.ascontiguousarray(net["edges"], np.int32)
    ids = np.ascontiguousarray(net["ids"], np.int32)
    U = int(net["U"])
    rc = L.eddy_write_networks(path.encode(), input_name.encode(), class_name.encode(),
                               set_name.encode(), U, _p(epn), names, g, _p(nodes), _p(edges),
                               int(epn[U]), _p(ids))
    if rc:
        raise EddyError(f"eddy_write_networks failed ({rc})")


def write_bdeu(path, input_name, class_name, set_name, class1, class2, lval):
    L = library()
    lv = np.ascontiguousarray(lval, np.float64).ravel()
    rc = L.eddy_write_bdeu(path.encode(), input_name.encode(), class_name.encode(),
                           set_name.encode(), class1.encode(), class2.encode(), lv.size // 2,
                           _p(lv))
    if rc:
        raise EddyError(f"eddy_write_bdeu failed ({rc})")


def write_edge_list(path, genes, el: dict, prior, class1, class2):
    L = library()
    g = len(genes)
    names = (C.c_char_p * g)(*[s.encode() for s in genes])
    nodes = np.ascontiguousarray(el["nodes"], np.int32).ravel()
    edges = np.ascontiguousarray(el["edges"], np.int32)
    epn = np.ascontiguousarray(el["epn"], np.int32)
    pr = None if prior is None else np.ascontiguousarray(prior, np.uint8)
    rc = L.eddy_write_edge_list(path.encode(), names, g, _p(nodes), _p(edges), _p(epn), _p(pr),
                                class1.encode(), class2.encode())
    if rc:
        raise EddyError(f"eddy_write_edge_list failed ({rc})")


def unit_noalloc(opts: "Opts", data, labels, prior=None, stream=None):
    """eddy_unit_noalloc: one labelling with no device allocation (host in,
    host out).  Returns (js, U); raises on a non-zero status."""
    L = library()
    data = np.ascontiguousarray(data, np.int8)
    labels = np.ascontiguousarray(labels, np.uint8)
    pr = None if prior is None else np.ascontiguousarray(prior, np.uint8)
    g, n = data.shape
    js = C.c_double()
    U = C.c_int32()
    rc = L.eddy_unit_noalloc(C.byref(opts), _p(data), g, n, _p(labels), _p(pr),
                             C.c_void_p(stream or 0), C.byref(js), C.byref(U))
    if rc:
        raise EddyError(f"eddy_unit_noalloc failed ({ERRORS.get(rc, rc)})")
    return js.value, U.value


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    """One eddy_ctx (one device, one stream)."""

    def __init__(self, max_parents=3, alpha_edge=0.05, alpha_edge_prior=None,
                 bonferroni=True, permutations=100, rng=RNG_GLIBC, seed=0, device=0,
                 keep_networks=True, prior_weight=0.5, lam=2.0):
        if alpha_edge_prior is None:
            alpha_edge_prior = 1 - (1 - alpha_edge) * prior_weight ** (1 / lam)
        self.L = library()
        self.opts = Opts(int(max_parents), float(alpha_edge), float(alpha_edge_prior),
                         1 if bonferroni else 0, int(permutations), int(rng), int(seed),
                         int(device), 1 if keep_networks else 0)
        h = C.c_void_p()
        rc = self.L.eddy_ctx_create(C.byref(self.opts), C.byref(h))
        if rc != 0:
            raise EddyError(f"eddy_ctx_create failed ({ERRORS.get(rc, rc)})")
        self.h = h
        self.n = 0
        self.g = {}

    def close(self):
        if self.h:
            self.L.eddy_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc != 0:
            msg = self.L.eddy_last_error(self.h)
            raise EddyError(f"{ERRORS.get(rc, rc)}: {msg.decode() if msg else ''}")

    def load_matrix(self, data, labels):
        data = np.ascontiguousarray(data, np.int8)
        labels = np.ascontiguousarray(labels, np.uint8)
        G, n = data.shape
        self._ck(self.L.eddy_load_matrix(self.h, _p(data), G, n, _p(labels)))
        self.n = n

    def add_set(self, genes, prior=None) -> int:
        genes = np.ascontiguousarray(genes, np.int32)
        pr = None if prior is None else np.ascontiguousarray(prior, np.uint8)
        sid = C.c_int()
        self._ck(self.L.eddy_add_set(self.h, _p(genes), genes.size, _p(pr), C.byref(sid)))
        self.g[sid.value] = genes.size
        return sid.value

    def set_labellings(self, set_id, labels):
        labels = np.ascontiguousarray(labels, np.uint8)
        self._ck(self.L.eddy_set_labellings(self.h, set_id, _p(labels), labels.shape[0]))

    def run(self):
        self._ck(self.L.eddy_run(self.h))

    def summary(self, set_id) -> dict:
        s = Summary()
        self._ck(self.L.eddy_get_set_summary(self.h, set_id, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Summary._fields_}

    def js(self, set_id):
        it = self.summary(set_id)["iterations"]
        js = np.zeros(it, np.float64)
        U = np.zeros(it, np.int32)
        self._ck(self.L.eddy_get_js(self.h, set_id, _p(js), _p(U)))
        return js, U

    def networks(self, set_id) -> dict:
        U, E = C.c_int(), C.c_int()
        self._ck(self.L.eddy_get_networks(self.h, set_id, C.byref(U), C.byref(E),
                                          None, None, None, None, None))
        g = self.g[set_id]
        ids = np.zeros(U.value, np.int32)
        nodes = np.zeros(U.value * g, np.int32)
        epn = np.zeros(U.value + 1, np.int32)
        edges = np.zeros(max(E.value, 1), np.int32)
        lval = np.zeros(2 * U.value, np.float64)
        self._ck(self.L.eddy_get_networks(self.h, set_id, C.byref(U), C.byref(E), _p(ids),
                                          _p(nodes), _p(epn), _p(edges), _p(lval)))
        return dict(U=U.value, ids=ids, nodes=nodes.reshape(U.value, g), epn=epn,
                    edges=edges[:E.value], lval=lval.reshape(2, U.value))

    def edge_list(self, set_id) -> dict:
        E = C.c_int()
        self._ck(self.L.eddy_get_edge_list(self.h, set_id, C.byref(E), None, None, None))
        g = self.g[set_id]
        nodes = np.zeros(2 * g, np.int32)
        epn = np.zeros(3, np.int32)
        edges = np.zeros(max(E.value, 1), np.int32)
        self._ck(self.L.eddy_get_edge_list(self.h, set_id, C.byref(E), _p(nodes), _p(epn),
                                           _p(edges)))
        return dict(nodes=nodes.reshape(2, g), epn=epn, edges=edges[:E.value])

    def run_labellings(self, set_id, labels):
        labels = np.ascontiguousarray(labels, np.uint8)
        R = labels.shape[0]
        js = np.zeros(R, np.float64)
        U = np.zeros(R, np.int32)
        self._ck(self.L.eddy_run_labellings(self.h, set_id, _p(labels), R, _p(js), _p(U)))
        return js, U

    def debug_edges(self, set_id, labels):
        labels = np.ascontiguousarray(labels, np.uint8)
        g = self.g[set_id]
        S = labels.size + 2
        c = g * (g - 1) // 2
        out = np.zeros((S, c), np.uint8)
        self._ck(self.L.eddy_debug_edges(self.h, set_id, _p(labels), _p(out)))
        return out

    def debug_unit(self, set_id, labels, mpk):
        labels = np.ascontiguousarray(labels, np.uint8)
        g = self.g[set_id]
        S = labels.size + 2
        ids = np.zeros(S, np.int32)
        cnt = np.zeros((S, g), np.int32)
        par = np.full((S, g, mpk), -1, np.int32)
        dist = np.zeros((2, S), np.float64)
        lval = np.zeros((2, S), np.float64)
        U = C.c_int()
        js = C.c_double()
        self._ck(self.L.eddy_debug_unit(self.h, set_id, _p(labels), int(mpk), C.byref(U),
                                        C.byref(js), _p(ids), _p(cnt), _p(par), _p(dist),
                                        _p(lval)))
        u = U.value
        return dict(U=u, js=js.value, ids=ids[:u], counts=cnt[:u], parents=par[:u],
                    dist=dist[:, :u], lval=lval[:, :u])

    def run_permutations(self, set_id, first, count):
        js = np.zeros(count, np.float64)
        U = np.zeros(count, np.int32)
        self._ck(self.L.eddy_run_permutations(self.h, set_id, int(first), int(count), _p(js),
                                              _p(U)))
        return js, U

    def set_stream(self, stream_handle: int | None):
        self._ck(self.L.eddy_set_stream(self.h, C.c_void_p(stream_handle or 0)))

    def clear_sets(self):
        self._ck(self.L.eddy_clear_sets(self.h))
        self.g = {}

    def stats(self) -> dict:
        st = np.zeros(4, np.uint64)
        v = C.c_int()
        self._ck(self.L.eddy_last_stats(self.h, _p(st), C.byref(v)))
        return dict(exact_rechecks=int(st[0]), tables=int(st[1]), filtered=int(st[2]),
                    duplicates=int(st[3]), variant=v.value)

    def timing(self) -> dict:
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        n = C.c_longlong()
        self._ck(self.L.eddy_last_timing(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(n)))
        st = (C.c_double * 4)()
        self._ck(self.L.eddy_last_stage_timing(self.h, st))
        return dict(ms_kernels=a.value, ms_pairs=b.value, ms_units=c.value, launches=n.value,
                    ms_gemm=st[0], ms_decide=st[1], ms_networks=st[2], ms_js=st[3])
