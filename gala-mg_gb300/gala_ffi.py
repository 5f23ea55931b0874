"""ctypes binding of libgala.so (the C ABI in include/gala.h).

This is the Python face of the engine used by the tests and bench.py; it
mirrors the reference's entry points (louvain_gpu, louvain_main_process,
build_compressed_graph) through the C ABI.  There is no Python or CPU
fallback: if libgala.so is missing, loading fails with an error.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libgala.so")

GALA_MAX_LEVELS = 64
STATUS = {0: "GALA_OK", 1: "GALA_ERR_INVALID", 2: "GALA_ERR_IO", 3: "GALA_ERR_FORMAT", 4: "GALA_ERR_CUDA",
          5: "GALA_ERR_NO_DEVICE", 6: "GALA_ERR_OOM", 7: "GALA_ERR_OVERFLOW", 8: "GALA_ERR_CAPACITY"}

# every symbol include/gala.h declares
EXPORTS = ["gala_last_error", "gala_status_string", "gala_kernel_launch_count", "gala_default_options",
           "gala_graph_load_bin", "gala_graph_store_bin", "gala_graph_from_text", "gala_graph_from_csr",
           "gala_graph_info", "gala_graph_arrays", "gala_graph_destroy", "gala_generate_sbm",
           "gala_generate_rmat", "gala_context_create", "gala_context_destroy", "gala_context_set_stream",
           "gala_graph_pin", "gala_louvain", "gala_louvain_device", "gala_phase1_device", "gala_contract_device",
           "gala_modularity_host", "gala_modularity_device_static", "gala_proposal_create",
           "gala_proposal_destroy", "gala_proposal_get_params", "gala_proposal_set_params", "gala_proposal_samples",
           "gala_proposal_clear_samples", "gala_proposal_read_samples", "gala_proposal_gradient",
           "gala_proposal_logits", "gala_proposal_train", "gala_louvain_batch", "gala_generate_sbm_batch",
           "gala_graph_from_csr_f32", "gala_graph_weights_f32", "gala_generate_lfr", "gala_autotune",
           "gala_context_set_hub_table_cap", "gala_context_set_update_mode", "gala_context_set_copy_overlap",
           "gala_context_set_long_rows"]

PROPOSAL_OFF, PROPOSAL_TRACE, PROPOSAL_SKIP = 0, 1, 2
PROPOSAL_PARAMS = 32 * 8 + 32 + 32 * 32 + 32 + 32 + 1

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class GalaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Options(ctypes.Structure):
    _fields_ = [("min_modularity", ctypes.c_double), ("max_levels", ctypes.c_int32),
                ("verbose", ctypes.c_int32), ("use_graphs", ctypes.c_int32), ("fp64_gains", ctypes.c_int32),
                ("proposal_mode", ctypes.c_int32), ("proposal_threshold", ctypes.c_float),
                ("trace_sample_shift", ctypes.c_int32), ("sorted_levels", ctypes.c_int32), ("proposal", ctypes.c_void_p),
                ("distinct_rows", ctypes.c_int32), ("bin5_block", ctypes.c_int32),
                ("bin_max", ctypes.c_int32 * 3), ("refine", ctypes.c_int32), ("level_dir", ctypes.c_char_p),
                ("proposal_from", ctypes.c_int32), ("batch_mode", ctypes.c_int32)]


class Tuning(ctypes.Structure):
    _fields_ = [("bin_max", ctypes.c_int32 * 3), ("bin5_block", ctypes.c_int32), ("ms", ctypes.c_double),
                ("default_ms", ctypes.c_double), ("candidates", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def to_dict(self):
        return {"bin_max": list(self.bin_max), "bin5_block": self.bin5_block, "ms": self.ms,
                "default_ms": self.default_ms, "candidates": self.candidates}


class Result(ctypes.Structure):
    _fields_ = [("modularity", ctypes.c_double), ("num_vertices", ctypes.c_int32),
                ("num_communities", ctypes.c_int32), ("num_levels", ctypes.c_int32),
                ("total_iterations", ctypes.c_int32),
                ("level_modularity", ctypes.c_double * GALA_MAX_LEVELS),
                ("level_communities", ctypes.c_int32 * GALA_MAX_LEVELS),
                ("level_iterations", ctypes.c_int32 * GALA_MAX_LEVELS),
                ("iter_modularity", _f64p), ("iter_capacity", ctypes.c_int32), ("iter_count", ctypes.c_int32),
                ("time_total_ms", ctypes.c_double), ("time_phase1_ms", ctypes.c_double),
                ("time_decide_ms", ctypes.c_double), ("time_update_ms", ctypes.c_double),
                ("time_contract_ms", ctypes.c_double), ("time_h2d_ms", ctypes.c_double),
                ("time_d2h_ms", ctypes.c_double), ("decide_sweeps", ctypes.c_int64),
                ("decide_bytes", ctypes.c_int64), ("update_bytes", ctypes.c_int64),
                ("kernel_launches", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64),
                ("d2h_bytes", ctypes.c_int64), ("fp64_decisions", ctypes.c_int64),
                ("decisions", ctypes.c_int64), ("skipped", ctypes.c_int64), ("verify_sweeps", ctypes.c_int32),
                ("incremental_sweeps", ctypes.c_int32), ("samples", ctypes.c_int64),
                ("level_vertices", ctypes.c_int32 * GALA_MAX_LEVELS),
                ("level_entries", ctypes.c_int64 * GALA_MAX_LEVELS),
                ("level_phase1_ms", ctypes.c_double * GALA_MAX_LEVELS),
                ("level_decide_ms", ctypes.c_double * GALA_MAX_LEVELS),
                ("level_update_ms", ctypes.c_double * GALA_MAX_LEVELS),
                ("level_contract_ms", ctypes.c_double * GALA_MAX_LEVELS),
                ("level_movers", ctypes.c_int64 * GALA_MAX_LEVELS),
                ("level_active_entries", ctypes.c_int64 * GALA_MAX_LEVELS),
                ("host_total_ms", ctypes.c_double), ("host_h2d_ms", ctypes.c_double),
                ("host_run_ms", ctypes.c_double), ("host_d2h_ms", ctypes.c_double)]

    def to_dict(self, trace=None):
        L = self.num_levels
        d = {"modularity": self.modularity, "num_vertices": self.num_vertices,
             "num_communities": self.num_communities, "rounds": L, "total_iterations": self.total_iterations,
             "level_q": list(self.level_modularity[:L]), "level_c": list(self.level_communities[:L]),
             "level_iters": list(self.level_iterations[:L]),
             "time_total_ms": self.time_total_ms, "time_phase1_ms": self.time_phase1_ms,
             "time_decide_ms": self.time_decide_ms, "time_update_ms": self.time_update_ms,
             "time_contract_ms": self.time_contract_ms, "time_h2d_ms": self.time_h2d_ms,
             "time_d2h_ms": self.time_d2h_ms, "decide_sweeps": self.decide_sweeps,
             "decide_bytes": self.decide_bytes, "update_bytes": self.update_bytes,
             "kernel_launches": self.kernel_launches, "h2d_bytes": self.h2d_bytes, "d2h_bytes": self.d2h_bytes,
             "fp64_decisions": self.fp64_decisions, "decisions": self.decisions, "skipped": self.skipped,
             "verify_sweeps": self.verify_sweeps, "incremental_sweeps": self.incremental_sweeps,
             "samples": self.samples,
             "host_ms": {"total": self.host_total_ms, "h2d": self.host_h2d_ms, "run": self.host_run_ms,
                         "d2h": self.host_d2h_ms},
             "levels": [{"vertices": self.level_vertices[i], "entries": self.level_entries[i],
                         "phase1_ms": self.level_phase1_ms[i], "decide_ms": self.level_decide_ms[i],
                         "update_ms": self.level_update_ms[i], "contract_ms": self.level_contract_ms[i],
                         "movers": self.level_movers[i], "active_entries": self.level_active_entries[i]}
                        for i in range(min(L, GALA_MAX_LEVELS))]}
        if trace is not None:
            d["iter_q"] = trace[:min(self.iter_count, len(trace))].tolist()
        return d


class BatchResult(ctypes.Structure):
    _fields_ = [("num_graphs", ctypes.c_int32), ("num_levels", ctypes.c_int32),
                ("total_iterations", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("vertices", ctypes.c_int64), ("entries", ctypes.c_int64),
                ("time_total_ms", ctypes.c_double), ("time_phase1_ms", ctypes.c_double),
                ("time_contract_ms", ctypes.c_double), ("time_h2d_ms", ctypes.c_double),
                ("time_d2h_ms", ctypes.c_double), ("kernel_launches", ctypes.c_int64),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]


_lib = None


def load(path=LIB_PATH):
    """Load libgala.so (raises OSError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"libgala.so not built at {path}; run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    L.gala_last_error.restype = ctypes.c_char_p
    L.gala_status_string.restype = ctypes.c_char_p
    L.gala_status_string.argtypes = [ctypes.c_int]
    L.gala_kernel_launch_count.restype = ctypes.c_int64
    L.gala_default_options.argtypes = [ctypes.POINTER(Options)]
    L.gala_graph_load_bin.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(_vp)]
    L.gala_graph_store_bin.argtypes = [_vp, ctypes.c_char_p]
    L.gala_graph_from_text.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_vp)]
    L.gala_graph_from_csr.argtypes = [ctypes.c_int32, _i64p, _i32p, _i32p, ctypes.POINTER(_vp)]
    L.gala_graph_info.argtypes = [_vp, _i32p, _i64p, _i32p]
    L.gala_graph_arrays.argtypes = [_vp, ctypes.POINTER(_i64p), ctypes.POINTER(_i32p), ctypes.POINTER(_i32p)]
    L.gala_graph_destroy.argtypes = [_vp]
    L.gala_graph_destroy.restype = None
    L.gala_generate_sbm.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_uint64, ctypes.POINTER(_vp)]
    L.gala_generate_rmat.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_uint64,
                                     ctypes.c_int32, ctypes.POINTER(_vp)]
    L.gala_context_create.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(_vp)]
    L.gala_context_destroy.argtypes = [_vp]
    L.gala_context_destroy.restype = None
    L.gala_context_set_stream.argtypes = [_vp, _vp]
    L.gala_context_set_hub_table_cap.argtypes = [_vp, ctypes.c_int64]
    L.gala_context_set_hub_table_cap.restype = ctypes.c_int
    L.gala_context_set_update_mode.argtypes = [_vp, ctypes.c_int32]
    L.gala_context_set_update_mode.restype = ctypes.c_int
    L.gala_context_set_long_rows.argtypes = [_vp, ctypes.c_int32]
    L.gala_context_set_long_rows.restype = ctypes.c_int
    L.gala_context_set_copy_overlap.argtypes = [_vp, ctypes.c_int32]
    L.gala_context_set_copy_overlap.restype = ctypes.c_int
    L.gala_graph_pin.argtypes = [_vp]
    L.gala_louvain.argtypes = [_vp, _vp, ctypes.POINTER(Options), _i32p, ctypes.POINTER(Result)]
    L.gala_louvain_device.argtypes = [_vp, ctypes.c_int32, _vp, _vp, _vp, ctypes.POINTER(Options), _vp,
                                      ctypes.POINTER(Result)]
    L.gala_phase1_device.argtypes = [_vp, ctypes.c_int32, _vp, _vp, _vp, ctypes.c_double, _vp, _f64p, _f64p,
                                     ctypes.c_int32, _i32p]
    L.gala_contract_device.argtypes = [_vp, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32p, _i64p]
    L.gala_modularity_host.argtypes = [_vp, _i32p, _f64p]
    L.gala_modularity_device_static.argtypes = [ctypes.c_int32, _vp, _vp, _vp, _vp, _f64p]
    L.gala_modularity_device_static.restype = ctypes.c_int
    _f32p = ctypes.POINTER(ctypes.c_float)
    L.gala_proposal_create.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(_vp)]
    L.gala_proposal_destroy.argtypes = [_vp]
    L.gala_proposal_destroy.restype = None
    L.gala_proposal_get_params.argtypes = [_vp, _f32p, ctypes.c_int32, _i32p]
    L.gala_proposal_set_params.argtypes = [_vp, _f32p, ctypes.c_int32]
    L.gala_proposal_samples.argtypes = [_vp, _i64p, _i64p]
    L.gala_proposal_clear_samples.argtypes = [_vp]
    L.gala_proposal_read_samples.argtypes = [_vp, ctypes.c_int64, ctypes.c_int64, _f32p, _f32p]
    L.gala_proposal_gradient.argtypes = [_vp, _f32p, _f32p, ctypes.c_int32, ctypes.c_float, _f32p, _f32p]
    L.gala_proposal_logits.argtypes = [_vp, _f32p, ctypes.c_int32, _f32p]
    L.gala_proposal_train.argtypes = [_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_uint64, _f32p]
    L.gala_louvain_batch.argtypes = [_vp, ctypes.POINTER(_vp), ctypes.c_int32, ctypes.POINTER(Options), _i32p,
                                     _f64p, _i32p, ctypes.POINTER(BatchResult)]
    L.gala_generate_sbm_batch.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_uint64, ctypes.c_int32, ctypes.POINTER(_vp)]
    L.gala_louvain_batch.restype = ctypes.c_int
    L.gala_graph_from_csr_f32.argtypes = [ctypes.c_int32, _i64p, _i32p, _f32p, ctypes.POINTER(_vp)]
    L.gala_graph_from_csr_f32.restype = ctypes.c_int
    L.gala_graph_weights_f32.argtypes = [_vp, ctypes.POINTER(_f32p)]
    L.gala_graph_weights_f32.restype = ctypes.c_int
    L.gala_generate_lfr.argtypes = [ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.c_uint64,
                                    ctypes.c_int32, ctypes.POINTER(_vp)]
    L.gala_generate_lfr.restype = ctypes.c_int
    L.gala_autotune.argtypes = [_vp, ctypes.POINTER(_vp), ctypes.c_int32, ctypes.POINTER(Options), ctypes.c_int32,
                                ctypes.POINTER(Tuning)]
    L.gala_autotune.restype = ctypes.c_int
    L.gala_generate_sbm_batch.restype = ctypes.c_int
    for name in ["gala_proposal_create", "gala_proposal_get_params", "gala_proposal_set_params",
                 "gala_proposal_samples", "gala_proposal_clear_samples", "gala_proposal_read_samples",
                 "gala_proposal_gradient", "gala_proposal_logits", "gala_proposal_train"]:
        getattr(L, name).restype = ctypes.c_int
    for name in ["gala_graph_load_bin", "gala_graph_store_bin", "gala_graph_from_text", "gala_graph_from_csr",
                 "gala_graph_info", "gala_graph_arrays", "gala_generate_sbm", "gala_generate_rmat",
                 "gala_context_create", "gala_context_set_stream", "gala_graph_pin", "gala_louvain",
                 "gala_louvain_device", "gala_phase1_device", "gala_contract_device", "gala_modularity_host"]:
        getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def _check(status):
    if status != 0:
        raise GalaError(status, load().gala_last_error().decode(errors="replace"))


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


def launch_count():
    return int(load().gala_kernel_launch_count())


def modularity_device_static(n, d_offs, d_nbr, d_w, d_comm):
    """gala_modularity_device_static on raw device pointers (no device
    allocation inside the call)."""
    q = ctypes.c_double()
    _check(load().gala_modularity_device_static(n, d_offs, d_nbr, d_w or None, d_comm, ctypes.byref(q)))
    return q.value


def default_options(**kw):
    o = Options()
    load().gala_default_options(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Graph:
    """Host graph owned by libgala (reference layout: inclusive offsets)."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None):
            load().gala_graph_destroy(self.h)
            self.h = None

    @staticmethod
    def load_bin(path, weighted=False):
        h = _vp()
        _check(load().gala_graph_load_bin(path.encode(), int(weighted), ctypes.byref(h)))
        return Graph(h)

    @staticmethod
    def from_text(path, weighted=False, nthreads=0):
        h = _vp()
        _check(load().gala_graph_from_text(path.encode(), int(weighted), nthreads, ctypes.byref(h)))
        return Graph(h)

    @staticmethod
    def from_csr(offs, nbr, w=None):
        """offs: n+1 offsets with a leading 0 (converted to the reference's
        inclusive layout)."""
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        incl = np.ascontiguousarray(offs[1:])
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        w = None if w is None else np.ascontiguousarray(w, dtype=np.int32)
        h = _vp()
        _check(load().gala_graph_from_csr(incl.shape[0], _ptr(incl, _i64p), _ptr(nbr, _i32p), _ptr(w, _i32p),
                                          ctypes.byref(h)))
        return Graph(h)

    @staticmethod
    def sbm(n, k, p_in, p_out, seed):
        h = _vp()
        _check(load().gala_generate_sbm(n, k, p_in, p_out, seed, ctypes.byref(h)))
        return Graph(h)

    @staticmethod
    def from_csr_f32(offs, nbr, wf):
        """Float-weight graph; offs with a leading 0."""
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        incl = np.ascontiguousarray(offs[1:])
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        wf = np.ascontiguousarray(wf, dtype=np.float32)
        h = _vp()
        _check(load().gala_graph_from_csr_f32(len(incl), _ptr(incl, _i64p), _ptr(nbr, _i32p),
                                              _ptr(wf, ctypes.POINTER(ctypes.c_float)), ctypes.byref(h)))
        return Graph(h)

    @staticmethod
    def lfr(n, tau1=2.5, dmin=4, dmax=20000, tau2=1.5, cmin=20, cmax=50000, mu=0.3, float_weights=True, seed=0,
            nthreads=0):
        """gala_generate_lfr: LFR-style planted graph (lognormal float weights)."""
        h = _vp()
        _check(load().gala_generate_lfr(n, tau1, dmin, dmax, tau2, cmin, cmax, mu, int(float_weights), seed, nthreads,
                                        ctypes.byref(h)))
        return Graph(h)

    @staticmethod
    def sbm_batch(count, n_min=200, n_max=200000, k_min=8, k_max=64, deg_min=12.0, deg_max=40.0, mix_min=0.1,
                  mix_max=0.4, seed=0, nthreads=0):
        """gala_generate_sbm_batch: `count` planted-partition graphs."""
        hs = (_vp * count)()
        _check(load().gala_generate_sbm_batch(count, n_min, n_max, k_min, k_max, deg_min, deg_max, mix_min, mix_max,
                                              seed, nthreads, hs))
        return [Graph(_vp(h)) for h in hs]

    @staticmethod
    def rmat(scale, edges, a=0.57, b=0.19, c=0.19, seed=1, nthreads=0, noise=0.0, keep_isolated=False):
        h = _vp()
        _check(load().gala_generate_rmat(scale, edges, a, b, c, noise, int(keep_isolated), seed, nthreads,
                                         ctypes.byref(h)))
        return Graph(h)

    def store_bin(self, path):
        _check(load().gala_graph_store_bin(self.h, path.encode()))

    def pin(self):
        _check(load().gala_graph_pin(self.h))

    def info(self):
        """(vertices, CSR entries, weight kind: 0 none, 1 int32, 2 float32);
        a graph never changes, so the answer is kept after the first call."""
        if getattr(self, "_info", None) is None:
            n, e, w = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int32()
            _check(load().gala_graph_info(self.h, ctypes.byref(n), ctypes.byref(e), ctypes.byref(w)))
            self._info = (n.value, e.value, w.value)
        return self._info

    def arrays(self):
        """(offs[n+1] with leading 0, nbr, w or None) as numpy copies."""
        n, e, weighted = self.info()
        po, pn, pw = _i64p(), _i32p(), _i32p()
        _check(load().gala_graph_arrays(self.h, ctypes.byref(po), ctypes.byref(pn), ctypes.byref(pw)))
        offs = np.zeros(n + 1, dtype=np.int64)
        offs[1:] = np.ctypeslib.as_array(po, shape=(n,))
        nbr = np.ctypeslib.as_array(pn, shape=(e,)).copy() if e else np.zeros(0, np.int32)
        w = np.ctypeslib.as_array(pw, shape=(e,)).copy() if (weighted == 1 and e) else None
        return offs, nbr, w

    def weights_f32(self):
        """Float weights (numpy copy) of a float-weight graph, else None."""
        n, e, weighted = self.info()
        if weighted != 2:
            return None
        p = ctypes.POINTER(ctypes.c_float)()
        _check(load().gala_graph_weights_f32(self.h, ctypes.byref(p)))
        return np.ctypeslib.as_array(p, shape=(e,)).copy() if e else np.zeros(0, np.float32)

    def modularity(self, labels):
        labels = np.ascontiguousarray(labels, dtype=np.int32)
        q = ctypes.c_double()
        _check(load().gala_modularity_host(self.h, _ptr(labels, _i32p), ctypes.byref(q)))
        return q.value


class Context:
    """Device context (one CUDA stream + workspace)."""

    def __init__(self, max_vertices, max_entries, device=0):
        self.h = _vp()
        _check(load().gala_context_create(device, int(max_vertices), int(max_entries), ctypes.byref(self.h)))

    def close(self):
        if getattr(self, "h", None):
            load().gala_context_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_hub_table_cap(self, slots):
        """Cap every hub's global hash table at `slots` (0 = by degree); for
        tests of the overflow status."""
        _check(load().gala_context_set_hub_table_cap(self.h, slots))

    def set_update_mode(self, mode):
        """Weight update of the sweeps: 0 = incremental when few rows moved
        (default), 1 = always full, 2 = incremental whenever allowed."""
        _check(load().gala_context_set_update_mode(self.h, mode))

    def set_long_rows(self, mode):
        """Contraction rows of more than 8192 entries: 0 = by key range
        (default), 1 = global hash tables only."""
        _check(load().gala_context_set_long_rows(self.h, mode))

    def set_copy_overlap(self, chunks):
        """gala_louvain of a pinned unweighted graph: copy the neighbours in
        `chunks` row chunks overlapped with the first sweep (8, the default;
        True = 8, False or 0 = one copy up front)."""
        if chunks is True:
            chunks = 8
        _check(load().gala_context_set_copy_overlap(self.h, int(chunks)))

    def set_stream(self, stream_handle):
        """Order the context's work on a caller CUDA stream (an int handle,
        e.g. torch.cuda.Stream().cuda_stream); None = own stream."""
        _check(load().gala_context_set_stream(self.h, stream_handle))

    def louvain(self, graph, min_mod=1e-6, max_levels=0, verbose=False, iter_capacity=4096, fp64_gains=False,
                proposal=None, mode=PROPOSAL_OFF, threshold=0.5, sample_shift=0, sorted_levels=False,
                use_graphs=False, tuning=None, level_dir=None, refine=False, proposal_from=0):
        """gala_louvain: host graph in, host labels out.  `proposal` (a
        Proposal) with mode PROPOSAL_TRACE records training samples, with
        PROPOSAL_SKIP decides only the vertices it proposes; `refine` turns
        on the Leiden-style refinement."""
        n, _, _ = graph.info()
        labels = np.zeros(n, dtype=np.int32)
        trace = np.zeros(iter_capacity, dtype=np.float64)
        r = Result()
        r.iter_modularity = _ptr(trace, _f64p)
        r.iter_capacity = iter_capacity
        o = default_options(min_modularity=min_mod, max_levels=max_levels, verbose=int(verbose),
                            fp64_gains=int(fp64_gains), proposal_mode=int(mode),
                            proposal_threshold=float(threshold), trace_sample_shift=int(sample_shift),
                            sorted_levels=int(sorted_levels), use_graphs=int(use_graphs),
                            proposal=proposal.h if proposal is not None else None, refine=int(refine),
                            proposal_from=int(proposal_from))
        if tuning:
            o.bin_max = (ctypes.c_int32 * 3)(*tuning["bin_max"])
            o.bin5_block = tuning["bin5_block"]
        if level_dir:
            o.level_dir = level_dir.encode()
        _check(load().gala_louvain(self.h, graph.h, ctypes.byref(o), _ptr(labels, _i32p), ctypes.byref(r)))
        d = r.to_dict(trace)
        d["labels"] = labels
        return d

    def autotune(self, graphs, repeats=2, **opts):
        """gala_autotune over one graph or a batch; returns the tuning dict
        (pass its bin_max / bin5_block as options)."""
        if isinstance(graphs, Graph):
            graphs = [graphs]
        hs = (_vp * len(graphs))(*[g.h for g in graphs])
        t = Tuning()
        o = default_options(**opts)
        _check(load().gala_autotune(self.h, hs, len(graphs), ctypes.byref(o), repeats, ctypes.byref(t)))
        return t.to_dict()

    def louvain_batch(self, graphs, min_mod=1e-6, max_levels=0, use_graphs=False, tuning=None, batch_mode=0):
        """gala_louvain_batch: many host graphs in one union run.  Returns the
        per-graph labels (local community ids), modularity and community
        counts plus the batch timings."""
        G = len(graphs)
        sizes = [g.info()[0] for g in graphs]
        labels = np.zeros(sum(sizes), dtype=np.int32)
        q = np.zeros(G, dtype=np.float64)
        c = np.zeros(G, dtype=np.int32)
        hs = (_vp * G)(*[g.h for g in graphs])
        r = BatchResult()
        o = default_options(min_modularity=min_mod, max_levels=max_levels, use_graphs=int(use_graphs),
                            batch_mode=int(batch_mode))
        if tuning:
            o.bin_max = (ctypes.c_int32 * 3)(*tuning["bin_max"])
            o.bin5_block = tuning["bin5_block"]
        _check(load().gala_louvain_batch(self.h, hs, G, ctypes.byref(o), _ptr(labels, _i32p), _ptr(q, _f64p),
                                         _ptr(c, _i32p), ctypes.byref(r)))
        starts = np.concatenate([[0], np.cumsum(sizes)])
        d = {f: getattr(r, f) for f, _ in BatchResult._fields_ if f != "reserved"}
        d.update({"labels": [labels[starts[i]:starts[i + 1]] for i in range(G)], "modularity": q,
                  "communities": c})
        return d

    def louvain_device(self, n, d_offs, d_nbr, d_w, d_out, min_mod=1e-6, max_levels=0, iter_capacity=4096,
                       fp64_gains=False, distinct_rows=False):
        """gala_louvain_device on raw device pointers (ints)."""
        trace = np.zeros(iter_capacity, dtype=np.float64)
        r = Result()
        r.iter_modularity = _ptr(trace, _f64p)
        r.iter_capacity = iter_capacity
        o = default_options(min_modularity=min_mod, max_levels=max_levels, fp64_gains=int(fp64_gains),
                            distinct_rows=int(distinct_rows))
        _check(load().gala_louvain_device(self.h, n, d_offs, d_nbr, d_w or None, ctypes.byref(o), d_out,
                                          ctypes.byref(r)))
        return r.to_dict(trace)

    def phase1_device(self, n, d_offs, d_nbr, d_w, d_out, min_mod=1e-6, iter_capacity=4096):
        q = ctypes.c_double()
        it = ctypes.c_int32()
        trace = np.zeros(iter_capacity, dtype=np.float64)
        _check(load().gala_phase1_device(self.h, n, d_offs, d_nbr, d_w or None, min_mod, d_out, ctypes.byref(q),
                                         _ptr(trace, _f64p), iter_capacity, ctypes.byref(it)))
        return {"q": q.value, "iterations": it.value, "iter_q": trace[:it.value + 1].tolist()}

    def contract_device(self, n, d_offs, d_nbr, d_w, d_comm, d_new_offs, d_new_nbr, d_new_w):
        C = ctypes.c_int32()
        E = ctypes.c_int64()
        _check(load().gala_contract_device(self.h, n, d_offs, d_nbr, d_w or None, d_comm, d_new_offs, d_new_nbr,
                                           d_new_w, ctypes.byref(C), ctypes.byref(E)))
        return C.value, E.value


class Proposal:
    """The learned move-proposal network (gala_proposal_*): an 8 -> 32 -> 32
    -> 1 MLP with its training-sample buffer on one device."""

    def __init__(self, max_samples=1 << 20, seed=0, device=0):
        self.h = _vp()
        _check(load().gala_proposal_create(device, int(max_samples), int(seed), ctypes.byref(self.h)))

    def close(self):
        if getattr(self, "h", None):
            load().gala_proposal_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def params(self):
        p = np.zeros(PROPOSAL_PARAMS, dtype=np.float32)
        cnt = ctypes.c_int32()
        _check(load().gala_proposal_get_params(self.h, _ptr(p, ctypes.POINTER(ctypes.c_float)), p.size,
                                               ctypes.byref(cnt)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(load().gala_proposal_set_params(self.h, _ptr(p, ctypes.POINTER(ctypes.c_float)), p.size))

    def samples(self):
        c = ctypes.c_int64()
        pos = ctypes.c_int64()
        _check(load().gala_proposal_samples(self.h, ctypes.byref(c), ctypes.byref(pos)))
        return c.value, pos.value

    def clear_samples(self):
        _check(load().gala_proposal_clear_samples(self.h))

    def read_samples(self, first=0, n=None):
        if n is None:
            n = self.samples()[0] - first
        X = np.zeros((n, 8), dtype=np.float32)
        Y = np.zeros(n, dtype=np.float32)
        f = ctypes.POINTER(ctypes.c_float)
        _check(load().gala_proposal_read_samples(self.h, first, n, _ptr(X, f), _ptr(Y, f)))
        return X, Y

    def gradient(self, X, Y, pos_weight=1.0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        g = np.zeros(PROPOSAL_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        f = ctypes.POINTER(ctypes.c_float)
        _check(load().gala_proposal_gradient(self.h, _ptr(X, f), _ptr(Y, f), len(Y), pos_weight, _ptr(g, f),
                                             ctypes.byref(loss)))
        return g, loss.value

    def logits(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros(len(X), dtype=np.float32)
        f = ctypes.POINTER(ctypes.c_float)
        _check(load().gala_proposal_logits(self.h, _ptr(X, f), len(X), _ptr(out, f)))
        return out

    def train(self, epochs=4, batch_size=4096, lr=3e-3, pos_weight=1.0, seed=0):
        loss = ctypes.c_float()
        _check(load().gala_proposal_train(self.h, epochs, batch_size, lr, pos_weight, seed, ctypes.byref(loss)))
        return loss.value
