"""GPU parity: the CUDA engine, called through the C ABI, against the CPU
oracle and the reference's own printed karate run.

The bar is bit-exact: labels, community counts and every iteration's
modularity (the engine and the oracle compute Q from the same exact integer
sums with the same FP64 expression; decisions use the reference's FP64
operation order without FMA contraction).  Independently, the modularity of
every returned partition must match a host FP64 recomputation within 1e-9.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle_ffi import read_bin

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch


def _sym_graph(rng, n, m, weighted, hubs=()):
    """Random symmetric CSR; hubs = [(vertex, extra random neighbours)]."""
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    for h, d in hubs:
        u = np.concatenate([u, np.full(d, h)])
        v = np.concatenate([v, rng.integers(0, n, d)])
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


def _run_both(ffi, oracle, offs, nbr, w):
    g = ffi.Graph.from_csr(offs, nbr, w)
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    r = ctx.louvain(g)
    ctx.close()
    o = oracle.louvain(offs, nbr, w)
    return g, r, o


def _assert_same(r, o):
    assert r["rounds"] == o["rounds"]
    assert r["level_c"] == o["level_c"]
    assert r["level_q"] == o["level_q"]
    assert r["iter_q"] == o["iter_q"]
    assert np.array_equal(r["labels"], o["labels"])


def test_karate_matches_reference_readme(ffi, oracle, golden, torch_cuda):
    g = ffi.Graph.load_bin(os.path.join(golden, "karate.txt.bin"))
    offs, nbr, w = g.arrays()
    ctx = ffi.Context(34, 156)
    r = ctx.louvain(g)
    tr = json.load(open(os.path.join(golden, "karate_trace.json")))
    assert ["%f" % q for q in r["iter_q"]] == [q for rd in tr["rounds"] for q in rd["iterations_q"]]
    assert r["level_c"] == [rd["communities"] for rd in tr["rounds"]]
    o = oracle.louvain(offs, nbr, None)
    _assert_same(r, o)
    assert abs(g.modularity(r["labels"]) - r["modularity"]) < 1e-9


@pytest.mark.parametrize("seed", [0, 1])
def test_sbm_golden(ffi, oracle, golden, torch_cuda, seed):
    path = os.path.join(golden, f"sbm_s{seed}.txt.bin")
    exp = json.load(open(path.replace(".txt.bin", ".expect.json")))
    g = ffi.Graph.load_bin(path)
    offs, nbr, w = g.arrays()
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    r = ctx.louvain(g)
    assert [repr(q) for q in r["iter_q"]] == exp["iter_q"]
    assert r["level_c"] == exp["level_c"]
    _assert_same(r, oracle.louvain(offs, nbr, None))


@pytest.mark.parametrize("weighted", [False, True])
@pytest.mark.parametrize("case", ["sparse", "dense", "hubs"])
def test_random_graphs_all_bins(ffi, oracle, torch_cuda, weighted, case):
    rng = np.random.default_rng(hash((case, weighted)) % 1000)
    if case == "sparse":      # degrees 1..~12: group bins
        offs, nbr, w = _sym_graph(rng, 6000, 14000, weighted)
    elif case == "dense":     # degrees ~250..450: warp and 256-thread CTA bins
        offs, nbr, w = _sym_graph(rng, 1500, 250000, weighted)
    else:                     # hubs of degree > 8192 (global tables) and 2k-8k (large smem tables)
        hubs = [(5, 9500), (77, 9500), (1234, 12000), (29000, 9000), (9, 3000), (10, 5000), (11, 7000)]
        offs, nbr, w = _sym_graph(rng, 30000, 60000, weighted, hubs=hubs)
    deg = np.diff(offs)
    g, r, o = _run_both(ffi, oracle, offs, nbr, w)
    _assert_same(r, o)
    assert abs(g.modularity(r["labels"]) - r["modularity"]) < 1e-9


def test_rmat_power_law(ffi, oracle, torch_cuda):
    g = ffi.Graph.rmat(15, 300000, seed=5)
    offs, nbr, w = g.arrays()
    assert np.diff(offs).max() > 2048
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    r = ctx.louvain(g)
    o = oracle.louvain(offs, nbr, None, nthreads=0)
    _assert_same(r, o)
    assert abs(g.modularity(r["labels"]) - r["modularity"]) < 1e-9
    # per-round diagnostics: round 0 runs on the input graph, every later round
    # on the previous round's communities; moves and decided entries add up
    lv = r["levels"]
    assert len(lv) == r["rounds"] and lv[0]["vertices"] == offs.shape[0] - 1 and lv[0]["entries"] == offs[-1]
    for k in range(1, len(lv)):
        assert lv[k]["vertices"] == r["level_c"][k - 1]
        assert lv[k]["entries"] <= lv[k - 1]["entries"]
    assert sum(x["active_entries"] for x in lv) >= sum(x["entries"] for x in lv)
    assert all(x["decide_ms"] + x["update_ms"] <= x["phase1_ms"] + 1e-3 for x in lv)
    assert abs(sum(x["contract_ms"] for x in lv) - r["time_contract_ms"]) < 1e-3


@pytest.mark.parametrize("case", ["karate", "sbm", "rmat", "weighted", "small_weights"])
def test_integer_gains_equal_fp64_gains(ffi, golden, torch_cuda, case):
    """The default exact-integer gain path and the all-FP64 path (the
    reference's expressions for every candidate) give the same partition."""
    rng = np.random.default_rng(17)
    if case == "karate":
        g = ffi.Graph.load_bin(os.path.join(golden, "karate.txt.bin"))
    elif case == "sbm":
        g = ffi.Graph.load_bin(os.path.join(golden, "sbm_s1.txt.bin"))
    elif case == "rmat":
        g = ffi.Graph.rmat(15, 250000, seed=11)
    elif case == "weighted":
        g = ffi.Graph.from_csr(*_sym_graph(rng, 20000, 150000, True, hubs=[(7, 9000), (8, 3000)]))
    else:  # many equal gains: all weights 1 or 2 on a ring of cliques
        offs, nbr, w = _sym_graph(rng, 3000, 9000, True)
        w = (w % 2 + 1).astype(np.int32)
        g = ffi.Graph.from_csr(offs, nbr, w)
    n, e, _ = g.info()
    ctx = ffi.Context(n, e)
    a = ctx.louvain(g)
    b = ctx.louvain(g, fp64_gains=True)
    assert a["iter_q"] == b["iter_q"]
    assert a["level_c"] == b["level_c"]
    assert np.array_equal(a["labels"], b["labels"])
    # level graphs with rows sorted by neighbour id give the same run
    c = ctx.louvain(g, sorted_levels=True)
    assert a["iter_q"] == c["iter_q"] and np.array_equal(a["labels"], c["labels"])
    # so do sweeps replayed from CUDA graphs
    d = ctx.louvain(g, use_graphs=True)
    assert a["iter_q"] == d["iter_q"] and np.array_equal(a["labels"], d["labels"])


def test_deterministic_replay(ffi, torch_cuda):
    g = ffi.Graph.rmat(14, 150000, seed=9)
    n, e, _ = g.info()
    ctx = ffi.Context(n, e)
    a = ctx.louvain(g)
    b = ctx.louvain(g)
    assert a["iter_q"] == b["iter_q"] and np.array_equal(a["labels"], b["labels"])


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("weighted", [False, True])
def test_phase1_and_contract_device_entry_points(ffi, oracle, torch_cuda, weighted):
    torch = torch_cuda
    rng = np.random.default_rng(21)
    offs, nbr, w = _sym_graph(rng, 5000, 40000, weighted, hubs=[(3, 2500)])
    n = offs.shape[0] - 1
    E = int(offs[-1])
    d_offs, d_nbr = _dev(torch, offs), _dev(torch, nbr)
    d_w = _dev(torch, w) if w is not None else None
    d_comm = torch.zeros(n, dtype=torch.int32, device="cuda")
    ctx = ffi.Context(n, E)
    p = ctx.phase1_device(n, d_offs.data_ptr(), d_nbr.data_ptr(), d_w.data_ptr() if d_w is not None else None,
                          d_comm.data_ptr())
    o = oracle.phase1(offs, nbr, w)
    assert p["iter_q"] == o["iter_q"] and p["q"] == o["q"]
    lab = d_comm.cpu().numpy()
    assert np.array_equal(lab, o["labels"])
    # contraction of that partition, bit-exact CSR with sorted rows
    d_no = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    d_nn = torch.zeros(max(E, 1), dtype=torch.int32, device="cuda")
    d_nw = torch.zeros(max(E, 1), dtype=torch.int32, device="cuda")
    C, newE = ctx.contract_device(n, d_offs.data_ptr(), d_nbr.data_ptr(),
                                  d_w.data_ptr() if d_w is not None else None, d_comm.data_ptr(), d_no.data_ptr(),
                                  d_nn.data_ptr(), d_nw.data_ptr())
    c = oracle.contract(offs, nbr, w, o["labels"])
    assert C == c["C"] and newE == int(c["offs"][-1])
    assert np.array_equal(d_no.cpu().numpy()[:C + 1], c["offs"])
    assert np.array_equal(d_nn.cpu().numpy()[:newE], c["nbr"])
    assert np.array_equal(d_nw.cpu().numpy()[:newE], c["w"])
    assert np.array_equal(d_comm.cpu().numpy(), c["relabel"])


def test_contract_arbitrary_partitions(ffi, oracle, torch_cuda):
    """Contraction of partitions phase 1 would not produce: a few huge
    communities (rows > 4096 entries, global tables) and many tiny ones."""
    torch = torch_cuda
    rng = np.random.default_rng(8)
    offs, nbr, w = _sym_graph(rng, 40000, 400000, True)
    n = offs.shape[0] - 1
    E = int(offs[-1])
    ctx = ffi.Context(n, E)
    for k in (3, 700, 20000):
        lab = rng.integers(0, k, n).astype(np.int32) * 2  # gaps in the label range
        d_offs, d_nbr, d_w = _dev(torch, offs), _dev(torch, nbr), _dev(torch, w)
        d_comm = _dev(torch, lab)
        d_no = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
        d_nn = torch.zeros(E, dtype=torch.int32, device="cuda")
        d_nw = torch.zeros(E, dtype=torch.int32, device="cuda")
        C, newE = ctx.contract_device(n, d_offs.data_ptr(), d_nbr.data_ptr(), d_w.data_ptr(), d_comm.data_ptr(),
                                      d_no.data_ptr(), d_nn.data_ptr(), d_nw.data_ptr())
        c = oracle.contract(offs, nbr, w, lab)
        assert C == c["C"]
        assert np.array_equal(d_no.cpu().numpy()[:C + 1], c["offs"])
        assert np.array_equal(d_nn.cpu().numpy()[:newE], c["nbr"])
        assert np.array_equal(d_nw.cpu().numpy()[:newE], c["w"])


@pytest.mark.parametrize("members", [600, 5000])
def test_contract_large_rows_hash_and_bitmap(ffi, oracle, torch_cuda, members):
    """Rows of more than 4096 entries in hash mode (the table is smaller than
    the community count): 600 members -> ~12k entries, sorted in shared
    memory; 5000 members -> ~45k distinct neighbours, ranked by the bitmap."""
    torch = torch_cuda
    rng = np.random.default_rng(members)
    n = 200000
    offs, nbr, w = _sym_graph(rng, n, 1000000, True)
    E = int(offs[-1])
    lab = np.arange(n, dtype=np.int32)
    for k in range(4):
        idx = rng.choice(n, members, replace=False)
        lab[idx] = idx[0]
    ctx = ffi.Context(n, E)
    d_offs, d_nbr, d_w, d_comm = _dev(torch, offs), _dev(torch, nbr), _dev(torch, w), _dev(torch, lab)
    d_no = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    d_nn = torch.zeros(E, dtype=torch.int32, device="cuda")
    d_nw = torch.zeros(E, dtype=torch.int32, device="cuda")
    C, newE = ctx.contract_device(n, d_offs.data_ptr(), d_nbr.data_ptr(), d_w.data_ptr(), d_comm.data_ptr(),
                                  d_no.data_ptr(), d_nn.data_ptr(), d_nw.data_ptr())
    c = oracle.contract(offs, nbr, w, lab)
    assert C == c["C"]
    assert np.array_equal(d_no.cpu().numpy()[:C + 1], c["offs"])
    assert np.array_equal(d_nn.cpu().numpy()[:newE], c["nbr"])
    assert np.array_equal(d_nw.cpu().numpy()[:newE], c["w"])


def test_louvain_device_equals_host_entry(ffi, torch_cuda):
    torch = torch_cuda
    g = ffi.Graph.rmat(13, 60000, seed=4)
    offs, nbr, w = g.arrays()
    n = offs.shape[0] - 1
    ctx = ffi.Context(n, offs[-1])
    r_host = ctx.louvain(g)
    d_offs, d_nbr = _dev(torch, offs), _dev(torch, nbr)
    d_out = torch.zeros(n, dtype=torch.int32, device="cuda")
    r_dev = ctx.louvain_device(n, d_offs.data_ptr(), d_nbr.data_ptr(), None, d_out.data_ptr())
    assert r_dev["iter_q"] == r_host["iter_q"]
    assert np.array_equal(d_out.cpu().numpy(), r_host["labels"])
    # the caller's distinct-rows guarantee (first sweep without aggregation)
    r_dd = ctx.louvain_device(n, d_offs.data_ptr(), d_nbr.data_ptr(), None, d_out.data_ptr(), distinct_rows=True)
    assert r_dd["iter_q"] == r_host["iter_q"]
    assert np.array_equal(d_out.cpu().numpy(), r_host["labels"])


@pytest.mark.parametrize("weighted", [False, True])
def test_rows_with_repeated_neighbours_match_oracle(ffi, oracle, torch_cuda, weighted):
    """A caller CSR may list a neighbour twice in a row (the reference's hash
    aggregation sums such entries): the first sweep must aggregate them."""
    rng = np.random.default_rng(41)
    n = 3000
    u = rng.integers(0, n, 20000)
    v = rng.integers(0, n, 20000)
    keep = u != v
    u, v = u[keep], v[keep]
    rows = np.concatenate([u, v, u])  # every edge once more from u's side ...
    cols = np.concatenate([v, u, v])  # ... and from v's side, keeping the CSR symmetric
    rows = np.concatenate([rows, v])
    cols = np.concatenate([cols, u])
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order].astype(np.int32)
    offs = np.zeros(n + 1, dtype=np.int64)
    np.add.at(offs, rows + 1, 1)
    offs = np.cumsum(offs)
    w = rng.integers(1, 5, cols.shape[0]).astype(np.int32) if weighted else None
    if w is not None:  # symmetric weights: the weight of (a, b) equals that of (b, a) entry by entry
        key = np.minimum(rows, cols).astype(np.int64) * n + np.maximum(rows, cols)
        _, inv = np.unique(key, return_inverse=True)
        w = (inv % 4 + 1).astype(np.int32)
    g = ffi.Graph.from_csr(offs, cols, w)
    ctx = ffi.Context(n, offs[-1])
    r = ctx.louvain(g)
    ctx.close()
    o = oracle.louvain(offs, cols, w)
    _assert_same(r, o)


def test_capacity_error(ffi, torch_cuda):
    g = ffi.Graph.rmat(12, 20000, seed=1)
    ctx = ffi.Context(100, 100)
    with pytest.raises(ffi.GalaError) as e:
        ctx.louvain(g)
    assert e.value.status == 8


def test_gala_main_cli_prints_reference_format(ffi, golden, torch_cuda, tmp_path):
    exe = os.path.join(os.path.dirname(ffi.LIB_PATH), "gala_main")
    out_labels = str(tmp_path / "labels.bin")
    r = subprocess.run([exe, "-f", os.path.join(golden, "karate.txt.bin"), "-o", out_labels], capture_output=True,
                       text=True, check=True)
    lines = r.stdout.splitlines()
    assert lines[0] == "vertex number:34 edge number:78"
    assert lines[1] == "load success"
    assert lines[2] == "===============round:0==============="
    assert lines[3:7] == ["Iteration:0 Q:-0.049803", "Iteration:1 Q:0.136834", "Iteration:2 Q:0.191239",
                          "Iteration:3 Q:0.169214"]
    assert "number of communities:11 modularity:0.191239" in lines
    assert "final number of communities:34 -> 4 final modularity:0.408695" in lines
    assert lines[-1].startswith("elapsed time = ")
    labels = np.fromfile(out_labels, dtype=np.int32)
    assert labels.shape == (34,) and len(np.unique(labels)) == 4


def test_bin_limits_and_autotune_keep_the_partition(ffi, torch_cuda):
    """Degree-bin limits move rows between schedules (warp, CTA, multi-CTA hub
    path) without changing any decision; the autotuner returns limits inside
    the allowed ranges."""
    rng = np.random.default_rng(23)
    offs, nbr, w = _sym_graph(rng, 20000, 160000, True, hubs=[(5, 9000), (6, 5000), (7, 3000)])
    g = ffi.Graph.from_csr(offs, nbr, w)
    ctx = ffi.Context(offs.shape[0] - 1, offs[-1])
    base = ctx.louvain(g)
    for t in ({"bin_max": [64, 1024, 4096], "bin5_block": 256}, {"bin_max": [32, 256, 2048], "bin5_block": 512},
              {"bin_max": [128, 2048, 8192], "bin5_block": 256}):
        r = ctx.louvain(g, tuning=t)
        assert r["iter_q"] == base["iter_q"] and np.array_equal(r["labels"], base["labels"]), t
    tun = ctx.autotune(g, repeats=1)
    m4, m5, m6 = tun["bin_max"]
    assert 32 <= m4 <= m5 <= m6 <= 8192 and tun["bin5_block"] in (256, 512)
    assert tun["ms"] <= tun["default_ms"] and tun["candidates"] >= 4
    ctx.close()


def test_level_checkpoints_resume(ffi, torch_cuda, tmp_path):
    """gala_options.level_dir: every round's contracted graph and the input
    vertices' labels in it; a run resumed from level 1 continues exactly."""
    g = ffi.Graph.rmat(14, 120000, seed=6)
    n, e, _ = g.info()
    ctx = ffi.Context(n, e)
    full = ctx.louvain(g, level_dir=str(tmp_path))
    assert full["rounds"] >= 3
    lab1 = np.fromfile(str(tmp_path / "labels_1.bin"), dtype=np.int32)
    g1 = ffi.Graph.load_bin(str(tmp_path / "level_1.bin"), weighted=True)
    n1, _, _ = g1.info()
    assert n1 == full["level_c"][0] and lab1.shape[0] == n and lab1.max() == n1 - 1
    res = ctx.louvain(g1)
    assert np.array_equal(res["labels"][lab1], full["labels"])
    assert res["modularity"] == full["modularity"]
    assert res["level_q"] == full["level_q"][1:]
    ctx.close()
