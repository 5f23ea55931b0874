"""Leiden-style refinement (gala_options.refine; no counterpart in the
reference).

The engine and the oracle (refine_w64 / louvain_w64 in
oracle/louvain_oracle.c) implement the same deterministic synchronous rule,
so with refinement on the partition, the per-iteration modularity and the
per-round community counts must agree bit for bit; the oracle's refinement
must only split communities; and the final modularity must match a host FP64
recomputation.
"""
import numpy as np
import pytest

from test_gpu_parity import _sym_graph


def _graphs(ffi):
    rng = np.random.default_rng(12)
    out = [("sbm", ffi.Graph.sbm(2048, 32, 0.2, 0.01, 1))]
    offs, nbr, w = _sym_graph(rng, 6000, 30000, True)
    out.append(("weighted", ffi.Graph.from_csr(offs, nbr, w)))
    out.append(("rmat", ffi.Graph.rmat(14, 150000, seed=3)))
    return out


def test_oracle_refinement_splits_communities(ffi, oracle):
    for name, g in _graphs(ffi):
        offs, nbr, w = g.arrays()
        plain = oracle.louvain(offs, nbr, w)
        P = plain["labels"]
        R = oracle.refine(offs, nbr, w, P)
        # every sub-community lies inside one community, and is labelled by a
        # member of that community
        order = np.argsort(R, kind="stable")
        Rs, Ps = R[order], P[order]
        starts = np.r_[0, np.flatnonzero(np.diff(Rs)) + 1]
        for a, b in zip(starts, np.r_[starts[1:], Rs.shape[0]]):
            assert np.all(Ps[a:b] == Ps[a]), name
            assert P[Rs[a]] == Ps[a], name
        assert np.unique(R).shape[0] >= np.unique(P).shape[0]


def test_oracle_refined_rounds_reach_plain_quality(ffi, oracle):
    # not a theorem for this rule: on these graphs the refined rounds end
    # within 0.002 of the plain ones, and clearly higher on the LFR graph
    for name, g in _graphs(ffi) + [("lfr", ffi.Graph.lfr(20000, dmin=4, dmax=200, cmin=20, cmax=1000, seed=2))]:
        offs, nbr, w = g.arrays()
        if name == "lfr":
            w = None
        a = oracle.louvain(offs, nbr, w)
        b = oracle.louvain(offs, nbr, w, refine=True)
        assert b["modularity"] >= a["modularity"] - 0.002, name
        if name == "lfr":
            assert b["modularity"] > a["modularity"] + 0.005
        assert abs(oracle.modularity(offs, nbr, w, b["labels"]) - b["modularity"]) < 1e-9


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch


@pytest.mark.gpu
def test_gpu_refine_matches_oracle(ffi, oracle, torch_cuda):
    for name, g in _graphs(ffi):
        offs, nbr, w = g.arrays()
        n, e, _ = g.info()
        ctx = ffi.Context(n, e)
        r = ctx.louvain(g, refine=True)
        r2 = ctx.louvain(g, refine=True)
        plain = ctx.louvain(g)
        ctx.close()
        o = oracle.louvain(offs, nbr, w, refine=True)
        assert np.array_equal(r["labels"], o["labels"]), name
        assert r["iter_q"] == o["iter_q"], name
        assert r["level_c"] == o["level_c"], name
        assert np.array_equal(r["labels"], r2["labels"]) and r["iter_q"] == r2["iter_q"], name
        assert abs(g.modularity(r["labels"]) - r["modularity"]) < 1e-9, name
        # the plain rounds are untouched by the option's existence
        po = oracle.louvain(offs, nbr, w)
        assert np.array_equal(plain["labels"], po["labels"]), name


def _float_graphs(ffi):
    rng = np.random.default_rng(3)
    offs, nbr, w = _sym_graph(rng, 4000, 24000, True)
    # symmetric float weights: a function of the unordered pair
    src = np.repeat(np.arange(offs.shape[0] - 1), np.diff(offs))
    lo, hi = np.minimum(src, nbr).astype(np.int64), np.maximum(src, nbr).astype(np.int64)
    wsym = (w * (1.0 + ((lo * 7919 + hi * 104729) % 97) / 64.0)).astype(np.float32)
    out = [("random", offs, nbr, wsym, ffi.Graph.from_csr_f32(offs, nbr, wsym))]
    g = ffi.Graph.lfr(20000, dmin=4, dmax=200, cmin=20, cmax=1000, seed=5)
    lo_, ln, _ = g.arrays()
    out.append(("lfr", lo_, ln, g.weights_f32(), g))
    return out


def test_oracle_refined_float_rounds(ffi, oracle):
    for name, offs, nbr, wf, _ in _float_graphs(ffi):
        a = oracle.louvain_f32(offs, nbr, wf)
        b = oracle.louvain_f32(offs, nbr, wf, refine=True)
        assert b["modularity"] >= a["modularity"] - 0.002, name
        assert abs(oracle.modularity_f32(offs, nbr, wf, b["labels"]) - b["modularity"]) < 1e-6, name


@pytest.mark.gpu
def test_gpu_refine_float_matches_oracle(ffi, oracle, torch_cuda):
    for name, offs, nbr, wf, g in _float_graphs(ffi):
        n, e, _ = g.info()
        ctx = ffi.Context(n, e)
        r = ctx.louvain(g, refine=True)
        r2 = ctx.louvain(g, refine=True)
        ctx.close()
        o = oracle.louvain_f32(offs, nbr, wf, refine=True)
        assert np.array_equal(r["labels"], o["labels"]), name
        assert r["iter_q"] == o["iter_q"], name
        assert r["level_c"] == o["level_c"], name
        assert np.array_equal(r["labels"], r2["labels"]) and r["iter_q"] == r2["iter_q"], name


@pytest.mark.gpu
def test_gpu_refine_single_round_equals_plain(ffi, torch_cuda):
    # one round: the round is the last, so nothing is refined
    g = ffi.Graph.sbm(2048, 32, 0.2, 0.01, 4)
    n, e, _ = g.info()
    ctx = ffi.Context(n, e)
    a = ctx.louvain(g, max_levels=1)
    b = ctx.louvain(g, max_levels=1, refine=True)
    ctx.close()
    assert np.array_equal(a["labels"], b["labels"]) and a["iter_q"] == b["iter_q"]


@pytest.mark.gpu
def test_gpu_refine_rejected_with_checkpoints(ffi, torch_cuda, tmp_path):
    g = ffi.Graph.sbm(512, 16, 0.3, 0.01, 5)
    n, e, _ = g.info()
    ctx = ffi.Context(n, e)
    with pytest.raises(RuntimeError, match="refinement"):
        ctx.louvain(g, refine=True, level_dir=str(tmp_path))
    ctx.close()
