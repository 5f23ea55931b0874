"""Float-weight graphs (no counterpart in the reference, whose weights are
int32).

The engine holds float weights as exact 64-bit fixed-point integers
round(w * 2^S) and evaluates every gain and pruning bound with the FP64
expressions.  Parity:
  * against the oracle's restatement on the same fixed-point weights:
    bit-exact labels and per-iteration modularity;
  * against the int32 path: a graph whose float weights are integers gives
    the same partition and the same modularity (scaling all weights by 2^S
    scales every FP64 gain exactly);
  * the returned modularity matches a host FP64 recomputation on the float
    weights within 1e-9.
"""
import os

import numpy as np
import pytest

from test_gpu_parity import _sym_graph

Q_TOL = 1e-9


def test_lfr_generator_deterministic_and_thread_independent(ffi):
    a = ffi.Graph.lfr(20000, dmin=4, dmax=400, cmin=20, cmax=2000, seed=3, nthreads=1)
    b = ffi.Graph.lfr(20000, dmin=4, dmax=400, cmin=20, cmax=2000, seed=3, nthreads=4)
    oa, na, _ = a.arrays()
    ob, nb, _ = b.arrays()
    assert np.array_equal(oa, ob) and np.array_equal(na, nb)
    wa, wb = a.weights_f32(), b.weights_f32()
    assert np.array_equal(wa, wb) and np.all(wa > 0)
    n, e, weighted = a.info()
    assert weighted == 2 and n == 20000
    deg = np.diff(oa)
    assert 6 <= deg.mean() <= 20 and deg.max() <= 400
    # lognormal(0, 1): median weight about 1 (parallel edges sum, so slightly above)
    assert 0.8 < np.median(wa) < 1.5


def test_float_bin_roundtrip(ffi, tmp_path):
    g = ffi.Graph.lfr(3000, dmin=4, dmax=100, cmin=20, cmax=500, seed=5)
    p = str(tmp_path / "f.bin")
    g.store_bin(p)
    h = ffi.Graph.load_bin(p, weighted=2)
    o1, n1, _ = g.arrays()
    o2, n2, _ = h.arrays()
    assert np.array_equal(o1, o2) and np.array_equal(n1, n2)
    assert np.array_equal(g.weights_f32(), h.weights_f32())
    n, e, _ = g.info()
    assert os.path.getsize(p) == 4 + 8 * n + 8 * e


def test_oracle_fixed_point_matches_int_path(oracle):
    rng = np.random.default_rng(8)
    offs, nbr, w = _sym_graph(rng, 3000, 15000, True)
    ri = oracle.louvain(offs, nbr, w)
    rf = oracle.louvain_f32(offs, nbr, w.astype(np.float32))
    assert rf["shift"] >= 6
    assert np.array_equal(ri["labels"], rf["labels"])
    assert ri["iter_q"] == rf["iter_q"]


def test_oracle_float_modularity_matches_fp64_host(oracle, ffi):
    g = ffi.Graph.lfr(8000, dmin=4, dmax=200, cmin=20, cmax=1000, seed=9)
    offs, nbr, _ = g.arrays()
    wf = g.weights_f32()
    r = oracle.louvain_f32(offs, nbr, wf)
    q = oracle.modularity_f32(offs, nbr, wf, r["labels"])
    assert abs(q - r["modularity"]) <= Q_TOL
    assert r["modularity"] > 0.3


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["small", "hubs"])
def test_gpu_float_equals_int_path(ffi, torch_cuda, case):
    rng = np.random.default_rng(31)
    hubs = [(3, 12000), (77, 9000)] if case == "hubs" else ()
    offs, nbr, w = _sym_graph(rng, 30000, 150000, True, hubs=hubs)
    gi = ffi.Graph.from_csr(offs, nbr, w)
    gf = ffi.Graph.from_csr_f32(offs, nbr, w.astype(np.float32))
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    ri = ctx.louvain(gi)
    rf = ctx.louvain(gf)
    ctx.close()
    assert np.array_equal(ri["labels"], rf["labels"])
    assert ri["iter_q"] == rf["iter_q"]
    assert ri["level_c"] == rf["level_c"]


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2])
def test_gpu_lfr_float_matches_oracle(ffi, oracle, torch_cuda, seed):
    g = ffi.Graph.lfr(40000, dmin=4, dmax=2000, cmin=20, cmax=5000, seed=seed)
    offs, nbr, _ = g.arrays()
    wf = g.weights_f32()
    n, e, _ = g.info()
    ctx = ffi.Context(n, e)
    r = ctx.louvain(g)
    r2 = ctx.louvain(g)
    ctx.close()
    o = oracle.louvain_f32(offs, nbr, wf, nthreads=4)
    assert np.array_equal(r["labels"], o["labels"])
    assert r["iter_q"] == o["iter_q"]
    assert np.array_equal(r["labels"], r2["labels"]) and r["iter_q"] == r2["iter_q"]
    q = oracle.modularity_f32(offs, nbr, wf, r["labels"])
    assert abs(q - r["modularity"]) <= Q_TOL
    assert abs(g.modularity(r["labels"]) - r["modularity"]) <= Q_TOL
