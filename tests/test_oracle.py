"""CPU tests of the oracle against the reference's own known answers.

The oracle (oracle/louvain_oracle.c) is pinned by
  * the reference's printed karate run (README.md:55-90): every iteration's
    Q, every round's community count, on the .bin written by the reference's
    own preprocess (tests/golden/karate.txt.bin);
  * the reference's host modularity formula (kernel_functions.cu:1037-1079)
    on every partition it returns.
"""
import json
import os

import numpy as np
import pytest

from oracle_ffi import read_bin


def _karate(golden):
    return read_bin(os.path.join(golden, "karate.txt.bin"))


def test_karate_trace_matches_reference_readme(oracle, golden):
    n, offs, nbr, w = _karate(golden)
    assert n == 34 and offs[-1] == 156
    tr = json.load(open(os.path.join(golden, "karate_trace.json")))
    r = oracle.louvain(offs, nbr, None, 1e-6)
    assert r["rounds"] == len(tr["rounds"])
    got = ["%f" % q for q in r["iter_q"]]
    want = [q for rd in tr["rounds"] for q in rd["iterations_q"]]
    assert got == want
    assert r["level_c"] == [rd["communities"] for rd in tr["rounds"]]
    assert ["%f" % q for q in r["level_q"]] == [rd["modularity"] for rd in tr["rounds"]]
    assert len(np.unique(r["labels"])) == tr["final"]["to"]


def test_karate_final_modularity_matches_host_recompute(oracle, golden):
    n, offs, nbr, w = _karate(golden)
    r = oracle.louvain(offs, nbr, None, 1e-6)
    q = oracle.modularity(offs, nbr, None, r["labels"])
    assert abs(q - r["modularity"]) < 1e-9


@pytest.mark.parametrize("seed", [0, 1])
def test_sbm_golden(oracle, golden, seed):
    n, offs, nbr, w = read_bin(os.path.join(golden, f"sbm_s{seed}.txt.bin"))
    exp = json.load(open(os.path.join(golden, f"sbm_s{seed}.expect.json")))
    r = oracle.louvain(offs, nbr, None, 1e-6)
    assert r["rounds"] == exp["rounds"]
    assert [repr(q) for q in r["level_q"]] == exp["level_q"]
    assert r["level_c"] == exp["level_c"]
    assert [repr(q) for q in r["iter_q"]] == exp["iter_q"]
    q = oracle.modularity(offs, nbr, None, r["labels"])
    assert abs(q - r["modularity"]) < 1e-9


def _random_graph(rng, n, m, weighted):
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    keep = u != v
    u, v = u[keep], v[keep]
    a = np.concatenate([u, v])
    b = np.concatenate([v, u])
    wt = rng.integers(1, 9, u.shape[0]) if weighted else np.ones(u.shape[0], dtype=np.int64)
    ww = np.concatenate([wt, wt])
    key = a.astype(np.int64) * n + b
    order = np.argsort(key, kind="stable")
    key, ww = key[order], ww[order]
    uk, idx = np.unique(key, return_index=True)
    wsum = np.add.reduceat(ww, idx)
    rows = (uk // n).astype(np.int64)
    cols = (uk % n).astype(np.int32)
    offs = np.zeros(n + 1, dtype=np.int64)
    np.add.at(offs, rows + 1, 1)
    offs = np.cumsum(offs)
    return offs, cols, (wsum.astype(np.int32) if weighted else None)


@pytest.mark.parametrize("weighted", [False, True])
def test_phase1_threads_agree(oracle, weighted):
    rng = np.random.default_rng(5)
    offs, nbr, w = _random_graph(rng, 3000, 12000, weighted)
    a = oracle.phase1(offs, nbr, w, nthreads=1)
    b = oracle.phase1(offs, nbr, w, nthreads=4)
    assert np.array_equal(a["labels"], b["labels"])
    assert a["iter_q"] == b["iter_q"]


def test_contract_invariants(oracle):
    rng = np.random.default_rng(2)
    offs, nbr, w = _random_graph(rng, 2000, 9000, True)
    labels = rng.integers(0, 300, offs.shape[0] - 1).astype(np.int32)
    c = oracle.contract(offs, nbr, w, labels)
    # total weight preserved, rows sorted ascending, symmetric
    assert int(c["w"].sum()) == int(w.sum())
    C = c["C"]
    assert C == len(np.unique(labels))
    dense = np.zeros((C, C), dtype=np.int64)
    for r in range(C):
        s, e = c["offs"][r], c["offs"][r + 1]
        assert np.all(np.diff(c["nbr"][s:e]) > 0)
        dense[r, c["nbr"][s:e]] = c["w"][s:e]
    assert np.array_equal(dense, dense.T)
    # the new ids keep the order of the labels
    mp = {old: i for i, old in enumerate(sorted(set(labels.tolist())))}
    assert np.array_equal(c["relabel"], np.array([mp[x] for x in labels], dtype=np.int32))


def test_modularity_of_singletons(oracle):
    rng = np.random.default_rng(3)
    offs, nbr, w = _random_graph(rng, 500, 3000, False)
    n = offs.shape[0] - 1
    q = oracle.modularity(offs, nbr, None, np.arange(n, dtype=np.int32))
    deg = np.diff(offs).astype(np.float64)
    m2 = deg.sum()
    assert abs(q - (-(deg ** 2).sum() / m2 ** 2)) < 1e-12
