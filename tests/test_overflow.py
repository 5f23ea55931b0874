"""The device overflow status, driven on purpose.

Every hash-table probe in the engine is bounded: an insert that finds no
slot in its table sets an error bit instead of dropping weight (the
reference drops it silently, src/louvain_gpu/kernel_functions.cu:217), and
the host turns the bit into GALA_ERR_OVERFLOW after the sweep.  Tables are
sized so that this cannot happen; gala_context_set_hub_table_cap caps the
hub tables below a hub's distinct neighbour communities so that the bounded
probes run out.  The run must stop with the status, no fault or hang, and the
same context must give the oracle's partition on the next run.
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


def _graph_with_hub(rng, n=20000, m=40000, hub_deg=12000):
    """A sparse random graph plus vertex 0 joined to hub_deg random vertices:
    the hub's row (degree > 8192) goes to the multi-CTA hub tables."""
    u = np.concatenate([rng.integers(0, n, m), np.zeros(hub_deg, dtype=np.int64)])
    v = np.concatenate([rng.integers(0, n, m), rng.choice(np.arange(1, n), hub_deg, replace=False)])
    keep = u != v
    a = np.concatenate([u[keep], v[keep]])
    b = np.concatenate([v[keep], u[keep]])
    key = np.unique(a.astype(np.int64) * n + b)
    rows, cols = key // n, (key % n).astype(np.int32)
    offs = np.zeros(n + 1, dtype=np.int64)
    np.add.at(offs, rows + 1, 1)
    return np.cumsum(offs), cols


def test_hub_table_overflow_reports_status_and_context_recovers(ffi, oracle, torch_cuda):
    offs, nbr = _graph_with_hub(np.random.default_rng(5))
    assert np.diff(offs)[0] > 8192
    g = ffi.Graph.from_csr(offs, nbr, None)
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    try:
        # in the first sweep every vertex is its own community: the hub's
        # 12,000 distinct keys cannot fit 1,024 slots
        ctx.set_hub_table_cap(1024)
        with pytest.raises(ffi.GalaError) as e:
            ctx.louvain(g)
        assert e.value.status == 7  # GALA_ERR_OVERFLOW
        assert "error bits" in str(e.value)
        # back to tables sized by degree: the same context gives the oracle's
        # partition and every iteration's Q
        ctx.set_hub_table_cap(0)
        r = ctx.louvain(g)
        o = oracle.louvain(offs, nbr, None)
        assert np.array_equal(r["labels"], o["labels"])
        assert r["iter_q"] == o["iter_q"] and r["level_c"] == o["level_c"]
        # a cap above the sized tables changes nothing
        ctx.set_hub_table_cap(1 << 16)
        r2 = ctx.louvain(g)
        assert np.array_equal(r2["labels"], r["labels"]) and r2["iter_q"] == r["iter_q"]
    finally:
        ctx.close()


def test_hub_table_cap_rejects_bad_sizes(ffi, torch_cuda):
    ctx = ffi.Context(100, 1000)
    try:
        for bad in (-1, 16, 1000, 3 << 10):
            with pytest.raises(ffi.GalaError) as e:
                ctx.set_hub_table_cap(bad)
            assert e.value.status == 1
        ctx.set_hub_table_cap(32)
        ctx.set_hub_table_cap(0)
    finally:
        ctx.close()
