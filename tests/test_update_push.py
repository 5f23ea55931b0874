"""Incremental weight update of the phase-1 sweeps against the full update
and the oracle.

The full update (compute_In, kernel_functions.cu:890-1034 of the reference)
sums In over every row after every sweep.  The incremental one sums In of
every mover again, pushes +-w from the movers to their neighbours that did
not move and then evaluates the pruning bound of every vertex.  Update mode 1
forces the full update, mode 2 the incremental one from a level's second
sweep on, mode 0 (the default) picks per sweep.  Every mode must give the
oracle's run bit for bit: labels, per-level communities and Q, and every
iteration's Q.
"""
import numpy as np
import pytest

from test_gpu_parity import _sym_graph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch


def _same(a, b):
    assert a["rounds"] == b["rounds"]
    assert a["level_c"] == b["level_c"]
    assert a["level_q"] == b["level_q"]
    assert a["iter_q"] == b["iter_q"]
    assert np.array_equal(a["labels"], b["labels"])


def _modes(ffi, g, n, e, **kw):
    ctx = ffi.Context(n, e)
    out = {}
    for mode in (1, 2, 0):
        ctx.set_update_mode(mode)
        out[mode] = ctx.louvain(g, **kw)
    ctx.close()
    return out


@pytest.mark.parametrize("case", ["sparse", "hubs_weighted", "dense_weighted"])
def test_incremental_matches_full_and_oracle(ffi, oracle, torch_cuda, case):
    rng = np.random.default_rng({"sparse": 3, "hubs_weighted": 4, "dense_weighted": 5}[case])
    if case == "sparse":
        offs, nbr, w = _sym_graph(rng, 8000, 20000, False)
    elif case == "hubs_weighted":  # hub rows > 8192 entries move and receive pushes
        hubs = [(5, 9500), (77, 12000), (1234, 3000), (9, 5000)]
        offs, nbr, w = _sym_graph(rng, 30000, 60000, True, hubs=hubs)
    else:
        offs, nbr, w = _sym_graph(rng, 1500, 200000, True)
    g = ffi.Graph.from_csr(offs, nbr, w)
    r = _modes(ffi, g, offs.shape[0] - 1, offs[-1])
    o = oracle.louvain(offs, nbr, w)
    for mode in (1, 2, 0):
        _same(r[mode], o)
    assert r[1]["incremental_sweeps"] == 0
    assert r[2]["incremental_sweeps"] > 0
    assert r[2]["incremental_sweeps"] >= r[0]["incremental_sweeps"]


@pytest.mark.parametrize("use_graphs", [False, True])
def test_incremental_rmat_matches_oracle(ffi, oracle, torch_cuda, use_graphs):
    """R-MAT rows of every degree bin; with use_graphs the sweeps after the
    first are replayed from CUDA graphs, the update path chosen inside them."""
    g = ffi.Graph.rmat(15, 300000, seed=7)
    offs, nbr, _ = g.arrays()
    r = _modes(ffi, g, offs.shape[0] - 1, offs[-1], use_graphs=use_graphs)
    o = oracle.louvain(offs, nbr, None, nthreads=0)
    for mode in (1, 2, 0):
        _same(r[mode], o)
    assert r[2]["incremental_sweeps"] > 0 and r[1]["incremental_sweeps"] == 0
    assert r[0]["incremental_sweeps"] <= r[2]["incremental_sweeps"]


def test_incremental_auto_on_a_large_level(ffi, oracle, torch_cuda):
    """Over 2^23 entries the default mode enqueues the incremental update
    (after a sweep that moved under a third of the rows) and lets the device
    pick it per sweep."""
    g = ffi.Graph.rmat(19, 5_000_000, seed=3)
    offs, nbr, _ = g.arrays()
    assert offs[-1] >= (1 << 23)
    r = _modes(ffi, g, offs.shape[0] - 1, offs[-1])
    _same(r[0], r[1])
    _same(r[2], r[1])
    o = oracle.louvain(offs, nbr, None, nthreads=0)
    _same(r[0], o)


def test_incremental_float_weights(ffi, oracle, torch_cuda):
    """64-bit fixed-point weights: the pushes subtract in two's complement."""
    g = ffi.Graph.lfr(30000, dmin=4, dmax=2000, cmin=20, cmax=5000, seed=3)
    offs, nbr, _ = g.arrays()
    n, e, _ = g.info()
    r = _modes(ffi, g, n, e)
    for mode in (2, 0):
        _same(r[mode], r[1])
    assert r[2]["incremental_sweeps"] > 0
    o = oracle.louvain_f32(offs, nbr, g.weights_f32(), nthreads=4)
    assert np.array_equal(r[2]["labels"], o["labels"]) and r[2]["iter_q"] == o["iter_q"]


def test_asymmetric_graph_keeps_full_update(ffi, oracle, torch_cuda):
    """A graph with entries that have no mirror fails the symmetry check:
    every sweep takes the full update, even when forced."""
    rng = np.random.default_rng(11)
    offs, nbr, w = _sym_graph(rng, 6000, 30000, True)
    # drop one entry from every 50th row that has more than one
    keep = np.ones(nbr.shape[0], dtype=bool)
    deg = np.diff(offs)
    for v in range(0, offs.shape[0] - 1, 50):
        if deg[v] > 1:
            keep[offs[v]] = False
    rows = np.repeat(np.arange(offs.shape[0] - 1), deg)[keep]
    nbr2, w2 = nbr[keep], w[keep]
    offs2 = np.zeros_like(offs)
    np.add.at(offs2, rows + 1, 1)
    offs2 = np.cumsum(offs2)
    g = ffi.Graph.from_csr(offs2, nbr2, w2)
    r = _modes(ffi, g, offs2.shape[0] - 1, offs2[-1])
    assert r[2]["incremental_sweeps"] == 0 and r[0]["incremental_sweeps"] == 0
    _same(r[2], r[1])
    _same(r[0], r[1])
    o = oracle.louvain(offs2, nbr2, w2)
    _same(r[1], o)


def test_update_mode_rejects_bad_values(ffi, torch_cuda):
    ctx = ffi.Context(16, 64)
    for bad in (-1, 3):
        with pytest.raises(ffi.GalaError):
            ctx.set_update_mode(bad)
    ctx.set_update_mode(0)
    ctx.close()
