"""Contraction rows of more than 8192 entries inside a Louvain run.

Long-rows mode 0 (the default) sums every 4096-entry chunk of a row per
neighbour community in shared memory, partitions the chunk's distinct
communities by id range (8192 ids per bucket) and sums every (row, bucket)
in one shared-memory table: a dense table for a bucket of more than 2048
pairs (split by chunk range over several CTAs above 32768 pairs), a hash
table for a run of smaller buckets.  Mode 1 adds every chunk's sums into a
global hash table of the row.  The reference builds each row with one hash
table per community (build_compressed_graph.cu:5-173, kernel_functions.cu:
1083-1694).  Both modes must give the oracle's run bit for bit: labels,
per-level communities and Q, every iteration's Q.

R-MAT scale 19 with 5M edges (seed 9) has, in its second contraction, 110
long rows with 177 buckets of more than 2048 pairs and 4 of more than 32768
(counted on the oracle's levels), so every item kind runs.
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
    for mode in (1, 0):
        ctx.set_long_rows(mode)
        out[mode] = ctx.louvain(g, **kw)
    ctx.close()
    return out


@pytest.mark.parametrize("use_graphs", [False, True])
def test_rmat_split_buckets_match_oracle(ffi, oracle, torch_cuda, use_graphs):
    g = ffi.Graph.rmat(19, 5_000_000, seed=9)
    offs, nbr, _ = g.arrays()
    r = _modes(ffi, g, offs.shape[0] - 1, offs[-1], use_graphs=use_graphs)
    _same(r[0], r[1])
    _same(r[0], oracle.louvain(offs, nbr, None, nthreads=0))


def test_weighted_hubs_match_oracle(ffi, oracle, torch_cuda):
    """Integer weights; hub rows of up to 40000 entries in level 0."""
    rng = np.random.default_rng(21)
    hubs = [(3, 40000), (17, 25000), (911, 12000), (4040, 9000)]
    offs, nbr, w = _sym_graph(rng, 60000, 150000, True, hubs=hubs)
    g = ffi.Graph.from_csr(offs, nbr, w)
    r = _modes(ffi, g, offs.shape[0] - 1, offs[-1])
    _same(r[0], r[1])
    _same(r[0], oracle.louvain(offs, nbr, w))


def test_wide_weights_match(ffi, oracle, torch_cuda):
    """64-bit fixed-point weights (LFR with float weights)."""
    g = ffi.Graph.lfr(60000, dmin=8, dmax=4000, cmin=50, cmax=20000, seed=5)
    offs, nbr, _ = g.arrays()
    n, e, _ = g.info()
    r = _modes(ffi, g, n, e)
    _same(r[0], r[1])
    o = oracle.louvain_f32(offs, nbr, g.weights_f32(), nthreads=4)
    assert np.array_equal(r[0]["labels"], o["labels"]) and r[0]["iter_q"] == o["iter_q"]


def test_sorted_levels_keep_global_tables(ffi, torch_cuda):
    """Sorted contracted levels take the global tables in both modes."""
    g = ffi.Graph.rmat(17, 1_500_000, seed=4)
    offs, _, _ = g.arrays()
    r = _modes(ffi, g, offs.shape[0] - 1, offs[-1], sorted_levels=True)
    _same(r[0], r[1])


def test_long_rows_rejects_bad_values(ffi, torch_cuda):
    ctx = ffi.Context(16, 64)
    for bad in (-1, 2):
        with pytest.raises(ffi.GalaError):
            ctx.set_long_rows(bad)
    ctx.set_long_rows(0)
    ctx.close()
