"""Batched graphs (gala_louvain_batch, no counterpart in the reference).

Every graph of a batch follows the single-graph rules with its own m2, min
Tot, modularity, iteration convergence and round rule, so its partition must
equal, bit for bit, the one the single-graph entry point and the CPU oracle
give for it alone; its modularity must match a host FP64 recomputation.
"""
import numpy as np
import pytest


def test_sbm_batch_generator_deterministic_and_in_range(ffi):
    a = ffi.Graph.sbm_batch(24, n_min=200, n_max=3000, seed=5)
    b = ffi.Graph.sbm_batch(24, n_min=200, n_max=3000, seed=5)
    sizes = []
    for ga, gb in zip(a, b):
        na, ea, _ = ga.info()
        nb, eb, _ = gb.info()
        assert (na, ea) == (nb, eb)
        oa, ca, _ = ga.arrays()
        ob, cb, _ = gb.arrays()
        assert np.array_equal(oa, ob) and np.array_equal(ca, cb)
        assert na <= 3000 and ea > 0
        sizes.append(na)
        deg = ea / na
        assert 4 <= deg <= 60
    assert max(sizes) > 2 * min(sizes)


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch


def _singles(ffi, graphs):
    out = []
    for g in graphs:
        n, e, _ = g.info()
        ctx = ffi.Context(n, e)
        out.append(ctx.louvain(g))
        ctx.close()
    return out


@pytest.mark.gpu
def test_batch_equals_single_runs(ffi, oracle, torch_cuda):
    graphs = ffi.Graph.sbm_batch(48, n_min=200, n_max=20000, seed=11)
    # plus graphs of the other families: a karate-sized SBM and random weighted graphs
    graphs.append(ffi.Graph.sbm(1024, 32, 0.3, 0.005, 3))
    rng = np.random.default_rng(4)
    for n in (300, 2500):
        u = rng.integers(0, n, 6 * n)
        v = rng.integers(0, n, 6 * n)
        keep = u != v
        u, v = u[keep], v[keep]
        key = np.unique(np.minimum(u, v).astype(np.int64) * n + np.maximum(u, v))
        a, b = key // n, key % n
        rows = np.concatenate([a, b])
        cols = np.concatenate([b, a]).astype(np.int32)
        wt = rng.integers(1, 7, a.shape[0])
        ww = np.concatenate([wt, wt]).astype(np.int32)
        order = np.lexsort((cols, rows))
        rows, cols, ww = rows[order], cols[order], ww[order]
        offs = np.zeros(n + 1, dtype=np.int64)
        np.add.at(offs, rows + 1, 1)
        graphs.append(ffi.Graph.from_csr(np.cumsum(offs), cols, ww))
    tot_n = sum(g.info()[0] for g in graphs)
    tot_e = sum(g.info()[1] for g in graphs)
    ctx = ffi.Context(tot_n, tot_e)
    r = ctx.louvain_batch(graphs)
    rg = ctx.louvain_batch(graphs, use_graphs=True)
    ctx.close()
    assert r["num_graphs"] == len(graphs)
    for i in range(len(graphs)):
        assert np.array_equal(r["labels"][i], rg["labels"][i]) and r["modularity"][i] == rg["modularity"][i]
    singles = _singles(ffi, graphs)
    for i, (g, s) in enumerate(zip(graphs, singles)):
        assert np.array_equal(r["labels"][i], s["labels"]), i
        assert r["modularity"][i] == s["modularity"], i
        assert r["communities"][i] == s["num_communities"], i
        assert abs(g.modularity(r["labels"][i]) - r["modularity"][i]) <= 1e-9
    # the oracle on a few of them
    for i in (0, len(graphs) - 3, len(graphs) - 1):
        offs, nbr, w = graphs[i].arrays()
        o = oracle.louvain(offs, nbr, w)
        assert np.array_equal(r["labels"][i], o["labels"])


@pytest.mark.gpu
def test_batch_max_levels_and_single_graph(ffi, torch_cuda):
    g = ffi.Graph.sbm(1024, 32, 0.3, 0.005, 9)
    n, e, _ = g.info()
    ctx = ffi.Context(n, e)
    r = ctx.louvain_batch([g])
    s = ctx.louvain(g)
    assert np.array_equal(r["labels"][0], s["labels"]) and r["modularity"][0] == s["modularity"]
    r1 = ctx.louvain_batch([g], max_levels=1)
    s1 = ctx.louvain(g, max_levels=1)
    assert np.array_equal(r1["labels"][0], s1["labels"]) and r1["num_levels"] == 1
    # the context still runs single graphs correctly after a batch
    s2 = ctx.louvain(g)
    assert np.array_equal(s2["labels"], s["labels"])
    ctx.close()


@pytest.mark.gpu
def test_batch_staged_and_page_locked_inputs_agree(ffi, torch_cuda):
    """A batch's graphs reach the device either staged (raw copies into the
    context's pinned buffer, one transfer, ids shifted on the device) or,
    when every graph is page-locked, read in place by the GPU.  Both give the
    same partitions; the per-graph state is kept between calls of different
    batch sizes."""
    rng = np.random.default_rng(21)
    big = ffi.Graph.sbm_batch(20, n_min=2000, n_max=40000, seed=23)
    small = big[:3]
    w_rows = []
    for n in (5000, 9000):  # weighted graphs beside unweighted ones
        offs, nbr, _ = ffi.Graph.sbm(n, 16, 0.02, 0.0005, int(rng.integers(1 << 30))).arrays()
        rows = np.repeat(np.arange(n), np.diff(offs))
        w_rows.append(ffi.Graph.from_csr(offs, nbr, (1 + (rows + nbr) % 5).astype(np.int32)))
    mixed = big[3:8] + w_rows
    tot_n = sum(g.info()[0] for g in big + w_rows)
    tot_e = sum(g.info()[1] for g in big + w_rows)
    ctx = ffi.Context(tot_n, tot_e)
    staged = {k: ctx.louvain_batch(gs) for k, gs in (("small", small), ("big", big), ("mixed", mixed))}
    pinned = 0
    for g in big + w_rows:
        try:
            g.pin()
            pinned += 1
        except ffi.GalaError:
            pass  # arrays sharing a page with one already registered: staged
    again = {k: ctx.louvain_batch(gs) for k, gs in (("small", small), ("mixed", mixed), ("big", big))}
    ctx.close()
    assert pinned > 0
    for k in staged:
        for a, b in zip(staged[k]["labels"], again[k]["labels"]):
            assert np.array_equal(a, b), k
        assert np.array_equal(staged[k]["modularity"], again[k]["modularity"]), k
        assert np.array_equal(staged[k]["communities"], again[k]["communities"]), k


def _random_weighted(rng, n, deg, wmax, isolated=0):
    """Random symmetric int-weighted graph; the last `isolated` vertices have
    no edges."""
    m = n * deg // 2
    live = n - isolated
    u = rng.integers(0, live, m)
    v = rng.integers(0, live, m)
    keep = u != v
    u, v = u[keep], v[keep]
    key = np.unique(np.minimum(u, v).astype(np.int64) * n + np.maximum(u, v))
    a, b = key // n, key % n
    rows = np.concatenate([a, b])
    cols = np.concatenate([b, a]).astype(np.int32)
    wt = rng.integers(1, wmax + 1, a.shape[0])
    ww = np.concatenate([wt, wt]).astype(np.int32)
    order = np.lexsort((cols, rows))
    rows, cols, ww = rows[order], cols[order], ww[order]
    offs = np.zeros(n + 1, dtype=np.int64)
    np.add.at(offs, rows + 1, 1)
    return np.cumsum(offs), cols, ww


@pytest.mark.gpu
def test_batch_one_cta_per_graph_equals_union_run_singles_and_oracle(ffi, oracle, torch_cuda):
    """Batches whose graphs all have at most 4096 vertices run in one
    persistent launch, each CTA running whole graphs (every sweep, the
    contraction, every round).  Their partitions, modularity and community
    counts must equal the union run's, the single-graph runs' and the
    oracle's, bit for bit."""
    rng = np.random.default_rng(31)
    graphs = ffi.Graph.sbm_batch(40, n_min=50, n_max=4000, seed=17)
    graphs.append(ffi.Graph.sbm(1024, 32, 0.3, 0.005, 5))
    for n, deg, wmax, iso in ((300, 8, 6, 0), (2500, 14, 9, 40), (4096, 6, 3, 0), (60, 3, 2, 7)):
        graphs.append(ffi.Graph.from_csr(*_random_weighted(rng, n, deg, wmax, iso)))
    graphs.append(ffi.Graph.from_csr(*_random_weighted(rng, 2, 1, 1)))  # one edge
    tot_n = sum(g.info()[0] for g in graphs)
    tot_e = sum(g.info()[1] for g in graphs)
    assert max(g.info()[0] for g in graphs) <= 4096
    ctx = ffi.Context(tot_n, tot_e)
    r = ctx.louvain_batch(graphs)
    r2 = ctx.louvain_batch(graphs)  # the workspace is reused
    u = ctx.louvain_batch(graphs, batch_mode=1)
    r1 = ctx.louvain_batch(graphs, max_levels=1)
    u1 = ctx.louvain_batch(graphs, max_levels=1, batch_mode=1)
    ctx.close()
    assert r["kernel_launches"] < 10 < u["kernel_launches"]
    for i in range(len(graphs)):
        for other in (r2, u):
            assert np.array_equal(r["labels"][i], other["labels"][i]), i
            assert r["modularity"][i] == other["modularity"][i], i
            assert r["communities"][i] == other["communities"][i], i
        assert np.array_equal(r1["labels"][i], u1["labels"][i]), i
        assert r1["modularity"][i] == u1["modularity"][i], i
    singles = _singles(ffi, graphs)
    for i, (g, s) in enumerate(zip(graphs, singles)):
        assert np.array_equal(r["labels"][i], s["labels"]), i
        assert r["modularity"][i] == s["modularity"], i
        assert abs(g.modularity(r["labels"][i]) - r["modularity"][i]) <= 1e-9
    for i in (0, 17, len(graphs) - 6, len(graphs) - 3, len(graphs) - 2):
        offs, nbr, w = graphs[i].arrays()
        o = oracle.louvain(offs, nbr, w)
        assert np.array_equal(r["labels"][i], o["labels"]), i
        assert r["modularity"][i] == o["modularity"], i
