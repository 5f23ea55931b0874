"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure: used by the tests, by __graft_entry__.smoke() as the
checker and by bench.py for the timed CPU baseline.  It is never on the
engine's path.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def read_bin(path, weighted=False):
    """Read a .bin in the reference layout (src/graph/graph.cpp:177-219) and
    return (n, offs[n+1] with leading 0, nbr, w or None)."""
    with open(path, "rb") as f:
        raw = f.read()
    n = int(np.frombuffer(raw, dtype=np.int32, count=1)[0])
    incl = np.frombuffer(raw, dtype=np.int64, count=n, offset=4)
    e = int(incl[-1]) if n else 0
    nbr = np.frombuffer(raw, dtype=np.int32, count=e, offset=4 + 8 * n).copy()
    w = None
    if weighted:
        w = np.frombuffer(raw, dtype=np.int32, count=e, offset=4 + 8 * n + 4 * e).copy()
    offs = np.zeros(n + 1, dtype=np.int64)
    offs[1:] = incl
    return n, offs, nbr, w


class Oracle:
    def __init__(self, build=True):
        if build and not os.path.exists(LIB):
            subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
        self.lib = ctypes.CDLL(LIB)
        L = self.lib
        L.orc_q_from_sums.restype = ctypes.c_double
        L.orc_q_from_sums.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
        L.orc_phase1.restype = ctypes.c_int32
        L.orc_phase1.argtypes = [ctypes.c_int32, _i64p, _i32p, _i32p, ctypes.c_int64, ctypes.c_double,
                                 _i32p, _f64p, _f64p, ctypes.c_int32, _i32p, ctypes.c_int32]
        L.orc_contract.restype = ctypes.c_int32
        L.orc_contract.argtypes = [ctypes.c_int32, _i64p, _i32p, _i32p, _i32p, _i32p, _i64p, _i32p, _i32p,
                                   _i64p]
        L.orc_louvain.restype = ctypes.c_int32
        L.orc_louvain.argtypes = [ctypes.c_int32, _i64p, _i32p, _i32p, ctypes.c_double, ctypes.c_int32,
                                  _i32p, _f64p, _i32p, _i32p, ctypes.c_int32, _f64p, ctypes.c_int32, _i32p,
                                  ctypes.c_int32]
        L.orc_louvain_refine.restype = ctypes.c_int32
        L.orc_louvain_refine.argtypes = L.orc_louvain.argtypes
        L.orc_refine.restype = None
        L.orc_refine.argtypes = [ctypes.c_int32, _i64p, _i32p, _i32p, _i32p, _i32p]
        L.orc_modularity.restype = ctypes.c_double
        L.orc_modularity.argtypes = [ctypes.c_int32, _i64p, _i32p, _i32p, _i32p]
        _f32p = ctypes.POINTER(ctypes.c_float)
        L.orc_fixed_shift.restype = ctypes.c_int32
        L.orc_fixed_shift.argtypes = [_f32p, ctypes.c_int64]
        L.orc_fixed_weights.restype = None
        L.orc_fixed_weights.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int32, _i64p]
        L.orc_louvain_fixed.restype = ctypes.c_int32
        L.orc_louvain_fixed.argtypes = [ctypes.c_int32, _i64p, _i32p, _i64p, ctypes.c_double, ctypes.c_int32,
                                        _i32p, _f64p, _i32p, _i32p, ctypes.c_int32, _f64p, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_int32), ctypes.c_int32]
        L.orc_louvain_fixed_refine.restype = ctypes.c_int32
        L.orc_louvain_fixed_refine.argtypes = L.orc_louvain_fixed.argtypes
        L.orc_modularity_f32.restype = ctypes.c_double
        L.orc_modularity_f32.argtypes = [ctypes.c_int32, _i64p, _i32p, _f32p, _i32p]
        L.orc_generate_rmat.restype = ctypes.c_int32
        L.orc_generate_rmat.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_uint64,
                                        ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(_i64p), ctypes.POINTER(_i32p)]
        L.orc_free.restype = None
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_seq_louvain.restype = ctypes.c_int32
        L.orc_seq_louvain.argtypes = [ctypes.c_int32, _i64p, _i32p, _i32p, ctypes.c_double, ctypes.c_int32,
                                      _i32p, _f64p, _i32p, ctypes.c_int32, _i64p]

    @staticmethod
    def _arrs(offs, nbr, w):
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        w = None if w is None else np.ascontiguousarray(w, dtype=np.int32)
        return offs, nbr, w

    def phase1(self, offs, nbr, w=None, min_mod=1e-6, nthreads=1, iter_cap=4096):
        offs, nbr, w = self._arrs(offs, nbr, w)
        n = offs.shape[0] - 1
        m2 = int(w.sum(dtype=np.int64)) if w is not None else int(offs[-1])
        lab = np.zeros(n, dtype=np.int32)
        q = ctypes.c_double()
        iq = np.zeros(iter_cap, dtype=np.float64)
        nq = ctypes.c_int32()
        it = self.lib.orc_phase1(n, _p(offs, _i64p), _p(nbr, _i32p), _p(w, _i32p), m2, min_mod,
                                 _p(lab, _i32p), ctypes.byref(q), _p(iq, _f64p), iter_cap, ctypes.byref(nq),
                                 nthreads)
        return {"labels": lab, "q": q.value, "iterations": it, "iter_q": iq[:min(nq.value, iter_cap)].tolist()}

    def contract(self, offs, nbr, w, labels):
        offs, nbr, w = self._arrs(offs, nbr, w)
        n = offs.shape[0] - 1
        labels = np.ascontiguousarray(labels, dtype=np.int32)
        rl = np.zeros(n, dtype=np.int32)
        no = np.zeros(n + 1, dtype=np.int64)
        cap = max(int(offs[-1]), 1)
        nn = np.zeros(cap, dtype=np.int32)
        nw = np.zeros(cap, dtype=np.int32)
        ne = ctypes.c_int64()
        C = self.lib.orc_contract(n, _p(offs, _i64p), _p(nbr, _i32p), _p(w, _i32p), _p(labels, _i32p),
                                  _p(rl, _i32p), _p(no, _i64p), _p(nn, _i32p), _p(nw, _i32p), ctypes.byref(ne))
        e = ne.value
        return {"C": C, "relabel": rl, "offs": no[:C + 1].copy(), "nbr": nn[:e].copy(), "w": nw[:e].copy()}

    def refine(self, offs, nbr, w, P):
        """Sub-community labels of the refinement of partition P."""
        offs, nbr, w = self._arrs(offs, nbr, w)
        P = np.ascontiguousarray(P, dtype=np.int32)
        R = np.zeros(P.shape[0], dtype=np.int32)
        self.lib.orc_refine(P.shape[0], _p(offs, _i64p), _p(nbr, _i32p), _p(w, _i32p), _p(P, _i32p),
                            _p(R, _i32p))
        return R

    def louvain(self, offs, nbr, w=None, min_mod=1e-6, max_levels=0, nthreads=1, iter_cap=65536, refine=False):
        offs, nbr, w = self._arrs(offs, nbr, w)
        n = offs.shape[0] - 1
        comm = np.zeros(n, dtype=np.int32)
        lq = np.zeros(64, dtype=np.float64)
        lc = np.zeros(64, dtype=np.int32)
        li = np.zeros(64, dtype=np.int32)
        iq = np.zeros(iter_cap, dtype=np.float64)
        nq = ctypes.c_int32()
        fn = self.lib.orc_louvain_refine if refine else self.lib.orc_louvain
        r = fn(n, _p(offs, _i64p), _p(nbr, _i32p), _p(w, _i32p), min_mod, max_levels,
                                 _p(comm, _i32p), _p(lq, _f64p), _p(lc, _i32p), _p(li, _i32p), 64,
                                 _p(iq, _f64p), iter_cap, ctypes.byref(nq), nthreads)
        return {"rounds": r, "labels": comm, "level_q": lq[:r].tolist(), "level_c": lc[:r].tolist(),
                "level_iters": li[:r].tolist(), "iter_q": iq[:min(nq.value, iter_cap)].tolist(),
                "modularity": float(lq[r - 1]) if r > 0 else float("nan")}

    def modularity(self, offs, nbr, w, labels):
        offs, nbr, w = self._arrs(offs, nbr, w)
        labels = np.ascontiguousarray(labels, dtype=np.int32)
        return self.lib.orc_modularity(offs.shape[0] - 1, _p(offs, _i64p), _p(nbr, _i32p), _p(w, _i32p),
                                       _p(labels, _i32p))

    def fixed_weights(self, wf):
        """(shift, int64 fixed-point weights) of float weights, as the engine
        holds them."""
        wf = np.ascontiguousarray(wf, dtype=np.float32)
        f32 = ctypes.POINTER(ctypes.c_float)
        shift = self.lib.orc_fixed_shift(_p(wf, f32), wf.shape[0])
        out = np.zeros(wf.shape[0], dtype=np.int64)
        self.lib.orc_fixed_weights(_p(wf, f32), wf.shape[0], shift, _p(out, _i64p))
        return shift, out

    def louvain_f32(self, offs, nbr, wf, min_mod=1e-6, max_levels=0, nthreads=1, iter_cap=65536, refine=False):
        """Multi-round run of a float-weight graph on its fixed-point weights."""
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        shift, w64 = self.fixed_weights(wf)
        assert shift >= 0
        n = offs.shape[0] - 1
        comm = np.zeros(n, dtype=np.int32)
        lq = np.zeros(64, dtype=np.float64)
        lc = np.zeros(64, dtype=np.int32)
        li = np.zeros(64, dtype=np.int32)
        iq = np.zeros(iter_cap, dtype=np.float64)
        nq = ctypes.c_int32()
        fn = self.lib.orc_louvain_fixed_refine if refine else self.lib.orc_louvain_fixed
        r = fn(n, _p(offs, _i64p), _p(nbr, _i32p), _p(w64, _i64p), min_mod, max_levels, _p(comm, _i32p),
               _p(lq, _f64p), _p(lc, _i32p), _p(li, _i32p), 64, _p(iq, _f64p), iter_cap, ctypes.byref(nq), nthreads)
        return {"rounds": r, "labels": comm, "level_q": lq[:r].tolist(), "level_c": lc[:r].tolist(),
                "level_iters": li[:r].tolist(), "iter_q": iq[:min(nq.value, iter_cap)].tolist(),
                "modularity": float(lq[r - 1]) if r > 0 else float("nan"), "shift": shift}

    def modularity_f32(self, offs, nbr, wf, labels):
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        wf = np.ascontiguousarray(wf, dtype=np.float32)
        labels = np.ascontiguousarray(labels, dtype=np.int32)
        return self.lib.orc_modularity_f32(offs.shape[0] - 1, _p(offs, _i64p), _p(nbr, _i32p),
                                           _p(wf, ctypes.POINTER(ctypes.c_float)), _p(labels, _i32p))

    def q_from_sums(self, sum_in, sum_tot2, m2):
        return self.lib.orc_q_from_sums(sum_in, sum_tot2, m2)

    def generate_rmat(self, scale, nedges, a=0.57, b=0.19, c=0.19, noise=0.0, keep_isolated=True, seed=1,
                      nthreads=0):
        """Seeded R-MAT graph built on the CPU (oracle/generators.c), identical
        to the engine library's generator: (offs[n+1] with leading 0, nbr)."""
        n = ctypes.c_int32()
        po = _i64p()
        pn = _i32p()
        rc = self.lib.orc_generate_rmat(scale, nedges, a, b, c, noise, int(keep_isolated), seed, nthreads,
                                        ctypes.byref(n), ctypes.byref(po), ctypes.byref(pn))
        if rc != 0:
            raise ValueError("orc_generate_rmat: bad arguments or out of memory")
        try:
            offs = np.ctypeslib.as_array(po, shape=(n.value + 1,)).copy()
            e = int(offs[-1])
            nbr = np.ctypeslib.as_array(pn, shape=(max(e, 1),))[:e].copy()
        finally:
            self.lib.orc_free(ctypes.cast(po, ctypes.c_void_p))
            self.lib.orc_free(ctypes.cast(pn, ctypes.c_void_p))
        return offs, nbr

    def seq_louvain(self, offs, nbr, w=None, min_mod=1e-6, max_levels=0):
        """The sequential (Blondel et al.) Louvain method on one thread."""
        offs, nbr, w = self._arrs(offs, nbr, w)
        n = offs.shape[0] - 1
        comm = np.zeros(n, dtype=np.int32)
        lq = np.zeros(64, dtype=np.float64)
        lc = np.zeros(64, dtype=np.int32)
        mv = ctypes.c_int64()
        r = self.lib.orc_seq_louvain(n, _p(offs, _i64p), _p(nbr, _i32p), _p(w, _i32p), min_mod, max_levels,
                                     _p(comm, _i32p), _p(lq, _f64p), _p(lc, _i32p), 64, ctypes.byref(mv))
        if r < 0:
            raise ValueError("orc_seq_louvain: bad input or out of memory")
        k = min(r, 64)
        return {"levels": r, "labels": comm, "level_q": lq[:k].tolist(), "level_c": lc[:k].tolist(),
                "modularity": float(lq[k - 1]), "moves": mv.value}
