"""gala_louvain with the neighbour copy overlapped with level 0.

A page-locked unweighted graph of at least 2^22 entries has its neighbours
copied in row-range chunks while the first sweep initialises and decides the
vertices of every chunk that has arrived.  The run must equal the run with one
copy up front and the oracle bit for bit: labels, per-level communities and
Q, every iteration's Q (including the singleton partition's, which comes from
the chunked row kernels).
"""
import numpy as np
import pytest

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


@pytest.mark.parametrize("keep_isolated", [False, True])
def test_chunked_copy_matches_single_copy_and_oracle(ffi, oracle, torch_cuda, keep_isolated):
    g = ffi.Graph.rmat(19, 5_000_000, seed=9, keep_isolated=keep_isolated)
    offs, nbr, _ = g.arrays()
    assert offs[-1] >= (1 << 22)
    g.pin()
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    ctx.set_copy_overlap(True)
    r1 = ctx.louvain(g)
    r1b = ctx.louvain(g)  # the context reused: the copy waits for the previous run's buffers
    ctx.set_copy_overlap(False)
    r0 = ctx.louvain(g)
    ctx.close()
    _same(r1, r0)
    _same(r1b, r0)
    assert r1["h2d_bytes"] == r0["h2d_bytes"] and r1["time_h2d_ms"] > 0
    _same(r0, oracle.louvain(offs, nbr, None, nthreads=0))


def test_chunked_copy_with_graphs_and_refine(ffi, torch_cuda):
    """CUDA graphs for the later sweeps and the refinement keep working on a
    level 0 whose rows arrived in chunks."""
    g = ffi.Graph.rmat(19, 5_000_000, seed=4)
    offs, _, _ = g.arrays()
    g.pin()
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    out = {}
    for on in (True, False):
        ctx.set_copy_overlap(on)
        out[on] = (ctx.louvain(g, use_graphs=True), ctx.louvain(g, refine=True))
    ctx.close()
    for k in range(2):
        _same(out[True][k], out[False][k])


@pytest.mark.parametrize("mode", ["trace", "skip"])
def test_chunked_copy_with_proposals(ffi, torch_cuda, mode):
    """Proposal runs take level 0 after the whole copy (the chunked first
    sweep is for plain runs): the same partitions with and without chunks."""
    g = ffi.Graph.rmat(19, 5_000_000, seed=6)
    offs, _, _ = g.arrays()
    g.pin()
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    out = {}
    for on in (8, 0):
        ctx.set_copy_overlap(on)
        prop = ffi.Proposal(max_samples=1 << 16, seed=1)
        kw = {"mode": ffi.PROPOSAL_TRACE} if mode == "trace" else {"mode": ffi.PROPOSAL_SKIP, "threshold": 0.5}
        out[on] = ctx.louvain(g, proposal=prop, **kw)
        prop.close()
    ctx.close()
    _same(out[8], out[0])


@pytest.mark.parametrize("chunks", [2, 16])
def test_chunk_counts(ffi, torch_cuda, chunks):
    g = ffi.Graph.rmat(19, 5_000_000, seed=2)
    offs, _, _ = g.arrays()
    g.pin()
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    ctx.set_copy_overlap(chunks)
    r1 = ctx.louvain(g)
    ctx.set_copy_overlap(0)
    r0 = ctx.louvain(g)
    ctx.close()
    _same(r1, r0)


def test_copy_overlap_rejects_bad_values(ffi, torch_cuda):
    ctx = ffi.Context(16, 64)
    for bad in (-1, 1, 17):
        with pytest.raises(ffi.GalaError):
            ctx.set_copy_overlap(bad)
    ctx.close()
