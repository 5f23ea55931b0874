"""CPU tests of libgala's host side: the library loads and exports every
symbol include/gala.h declares, the .bin format is byte-compatible with the
reference (src/graph/graph.cpp:153-219), text preprocessing matches the
reference preprocess, errors come back as status codes."""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle_ffi import read_bin

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_PRE = os.path.join(ROOT, "oracle", "_ref", "preprocess")


def _header_symbols():
    src = open(os.path.join(ROOT, "include", "gala.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gala_[a-z0-9_]+)\s*\(", src)))


def test_exports_match_header(ffi):
    lib = ffi.load()
    hdr = _header_symbols()
    assert sorted(ffi.EXPORTS) == hdr
    for s in hdr:
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", ffi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gala_\w+)", out))
    assert set(hdr) <= exported


def test_load_bin_karate(ffi, golden):
    g = ffi.Graph.load_bin(os.path.join(golden, "karate.txt.bin"))
    n, e, wt = g.info()
    assert (n, e, wt) == (34, 156, False)
    offs, nbr, w = g.arrays()
    n2, offs2, nbr2, _ = read_bin(os.path.join(golden, "karate.txt.bin"))
    assert np.array_equal(offs, offs2) and np.array_equal(nbr, nbr2) and w is None


def test_store_bin_roundtrip_bytes(ffi, golden, tmp_path):
    for name in ("karate.txt.bin", "sbm_s0.txt.bin"):
        g = ffi.Graph.load_bin(os.path.join(golden, name))
        out = str(tmp_path / name)
        g.store_bin(out)
        assert open(out, "rb").read() == open(os.path.join(golden, name), "rb").read()


def test_text_to_bin_matches_reference_golden(ffi, golden, tmp_path):
    g = ffi.Graph.from_text(os.path.join(golden, "karate.txt"))
    out = str(tmp_path / "k.bin")
    g.store_bin(out)
    assert open(out, "rb").read() == open(os.path.join(golden, "karate.txt.bin"), "rb").read()


def _write_edges(path, rng, nid, m, weighted, self_loops=False):
    with open(path, "w") as f:
        f.write("# comment line\n\n")
        for _ in range(m):
            u, v = int(rng.integers(0, nid)), int(rng.integers(0, nid))
            if u == v and not self_loops:
                continue
            if weighted:
                f.write(f"{u} {v} {int(rng.integers(1, 7))}\n")
            else:
                f.write(f"{u}\t{v}\n")


@pytest.mark.skipif(not os.path.exists(REF_PRE), reason="reference preprocess not built here")
@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_preprocess_cli_byte_identical_to_reference(ffi, tmp_path, seed):
    rng = np.random.default_rng(seed)
    txt = str(tmp_path / f"g{seed}.txt")
    # sparse ids leave isolated ids to drop; duplicates and reversed pairs
    _write_edges(txt, rng, 5000, 9000, False)
    d_ref = tmp_path / "ref"
    d_new = tmp_path / "new"
    d_ref.mkdir()
    d_new.mkdir()
    subprocess.check_call([REF_PRE, "-f", txt, "-o", str(d_ref)], stdout=subprocess.DEVNULL,
                          stderr=subprocess.DEVNULL)
    exe = os.path.join(os.path.dirname(ffi.LIB_PATH), "gala_preprocess")
    out = subprocess.run([exe, "-f", txt, "-o", str(d_new)], capture_output=True, text=True, check=True).stdout
    assert "store successfully." in out
    a = open(d_ref / f"g{seed}.txt.bin", "rb").read()
    b = open(d_new / f"g{seed}.txt.bin", "rb").read()
    assert a == b


@pytest.mark.skipif(not os.path.exists(REF_PRE), reason="reference preprocess not built here")
def test_preprocess_weighted_offsets_and_ids_match_reference(ffi, tmp_path):
    # the reference writes only one weight (graph.cpp:132-143); ids and
    # offsets must still match, and our weights are the per-row sums
    rng = np.random.default_rng(9)
    txt = str(tmp_path / "w.txt")
    _write_edges(txt, rng, 300, 1500, True)
    subprocess.check_call([REF_PRE, "-f", txt, "-w"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    ref = open(txt + ".bin", "rb").read()
    g = ffi.Graph.from_text(txt, weighted=True)
    offs, nbr, w = g.arrays()
    n = offs.shape[0] - 1
    e = int(offs[-1])
    assert ref[: 4 + 8 * n + 4 * e] == (np.int32(n).tobytes() + offs[1:].tobytes() + nbr.tobytes())
    # weights: symmetric and equal to the summed duplicates of the text
    lines = [l.split() for l in open(txt) if l.strip() and not l.startswith("#")]
    acc = {}
    for a_, b_, ww in lines:
        for x, y in ((int(a_), int(b_)), (int(b_), int(a_))):
            acc[(x, y)] = acc.get((x, y), 0) + int(ww)
    ids = sorted({x for x, _ in acc})
    mp = {o: i for i, o in enumerate(ids)}
    for r in range(n):
        for j in range(offs[r], offs[r + 1]):
            assert w[j] == acc[(ids[r], ids[nbr[j]])]


def test_text_parse_equivalent_to_map_dedup(ffi, tmp_path):
    rng = np.random.default_rng(4)
    txt = str(tmp_path / "e.txt")
    _write_edges(txt, rng, 800, 4000, False)
    g = ffi.Graph.from_text(txt, nthreads=3)
    offs, nbr, _ = g.arrays()
    edges = set()
    for l in open(txt):
        if not l.strip() or l.startswith("#"):
            continue
        a, b = map(int, l.split())
        edges.add((a, b))
        edges.add((b, a))
    ids = sorted({x for x, _ in edges})
    mp = {o: i for i, o in enumerate(ids)}
    rows = [[] for _ in ids]
    for a, b in edges:
        rows[mp[a]].append(mp[b])
    assert offs.shape[0] - 1 == len(ids)
    for r in range(len(ids)):
        assert list(nbr[offs[r]:offs[r + 1]]) == sorted(rows[r])


def test_errors_are_status_codes(ffi, tmp_path):
    with pytest.raises(ffi.GalaError) as e:
        ffi.Graph.load_bin(str(tmp_path / "missing.bin"))
    assert e.value.status == 2
    p = tmp_path / "trunc.bin"
    p.write_bytes(np.int32(10).tobytes() + np.arange(1, 11, dtype=np.int64).tobytes())
    with pytest.raises(ffi.GalaError) as e:
        ffi.Graph.load_bin(str(p))
    assert e.value.status == 3
    # odd entry count (what the reference writer leaves for an odd number of
    # self-loops) is rejected instead of read out of bounds
    p2 = tmp_path / "odd.bin"
    p2.write_bytes(np.int32(2).tobytes() + np.array([1, 3], dtype=np.int64).tobytes()
                   + np.array([1, 0], dtype=np.int32).tobytes())
    with pytest.raises(ffi.GalaError) as e:
        ffi.Graph.load_bin(str(p2))
    assert e.value.status == 3
    with pytest.raises(ffi.GalaError) as e:
        ffi.Graph.from_csr(np.array([0, 1, 2]), np.array([1, 5], dtype=np.int32))
    assert e.value.status == 3


def test_host_modularity_matches_oracle(ffi, oracle, golden):
    g = ffi.Graph.load_bin(os.path.join(golden, "sbm_s0.txt.bin"))
    offs, nbr, w = g.arrays()
    r = oracle.louvain(offs, nbr, None)
    assert abs(g.modularity(r["labels"]) - oracle.modularity(offs, nbr, None, r["labels"])) < 1e-12


def test_generators_deterministic(ffi):
    a = ffi.Graph.sbm(1024, 32, 0.3, 0.005, 11).arrays()
    b = ffi.Graph.sbm(1024, 32, 0.3, 0.005, 11).arrays()
    assert all(np.array_equal(x, y) for x, y in zip(a[:2], b[:2]))
    offs, nbr, _ = a
    n = offs.shape[0] - 1
    assert n == 1024
    intra = sum(int(np.sum((nbr[offs[v]:offs[v + 1]] // 32) == v // 32)) for v in range(n)) // 2
    m = int(offs[-1]) // 2
    assert 4300 < intra < 5300 and 2100 < m - intra < 3000
    r1 = ffi.Graph.rmat(12, 30000, seed=3, nthreads=1).arrays()
    r2 = ffi.Graph.rmat(12, 30000, seed=3, nthreads=4).arrays()
    assert np.array_equal(r1[0], r2[0]) and np.array_equal(r1[1], r2[1])
    # symmetric, no self-loops, sorted unique rows
    offs, nbr, _ = r1
    for v in range(offs.shape[0] - 1):
        row = nbr[offs[v]:offs[v + 1]]
        assert np.all(np.diff(row) > 0) and not np.any(row == v)


def test_context_without_gpu_reports_no_device(ffi):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(ffi.GalaError) as e:
        ffi.Context(10, 10)
    assert e.value.status == 5


def test_cli_binaries_exist(ffi):
    d = os.path.dirname(ffi.LIB_PATH)
    for exe in ("gala_main", "gala_preprocess"):
        assert os.access(os.path.join(d, exe), os.X_OK)


def test_context_setters_reject_a_null_context(ffi):
    """The per-context switches check their arguments before any device work:
    a null context is GALA_ERR_INVALID (1), on a machine with or without a GPU."""
    L = ffi.load()
    assert L.gala_context_set_update_mode(None, 0) == 1
    assert L.gala_context_set_copy_overlap(None, 8) == 1
    assert L.gala_context_set_long_rows(None, 0) == 1
    assert L.gala_context_set_hub_table_cap(None, 0) == 1
