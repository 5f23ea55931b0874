"""CPU side of the bench: the oracle's R-MAT generator and the sequential
Louvain baseline (both test infrastructure under oracle/).

* The CPU arm of bench.py builds its graph with orc_generate_rmat so that it
  never loads the engine library; the graph must be byte-identical to the
  engine's own gala_generate_rmat, which the GPU arm times.
* orc_seq_louvain is the classic sequential (asynchronous) Louvain method of
  Blondel et al. (2008) on one thread, the sequential CPU baseline.  It is not
  the engine's checker (the synchronous oracle is); its tests pin it by
  modularity bands and by the exact host recomputation of its own Q.
"""
import os

import numpy as np
import pytest

from oracle_ffi import read_bin


@pytest.mark.parametrize("scale,nedges,seed,keep,noise",
                         [(12, 30000, 1, True, 0.0), (14, 160000, 7, False, 0.0), (13, 70000, 3, True, 0.1)])
def test_oracle_rmat_identical_to_engine_generator(ffi, oracle, scale, nedges, seed, keep, noise):
    g = ffi.Graph.rmat(scale, nedges, 0.57, 0.19, 0.19, noise=noise, seed=seed, keep_isolated=keep)
    offs, nbr, w = g.arrays()
    assert w is None
    o2, n2 = oracle.generate_rmat(scale, nedges, 0.57, 0.19, 0.19, noise=noise, keep_isolated=keep, seed=seed)
    assert offs.dtype == o2.dtype and nbr.dtype == n2.dtype
    assert offs.tobytes() == o2.tobytes()
    assert nbr.tobytes() == n2.tobytes()


def test_oracle_rmat_does_not_depend_on_threads(oracle):
    a = oracle.generate_rmat(13, 80000, seed=5, nthreads=1)
    b = oracle.generate_rmat(13, 80000, seed=5, nthreads=3)
    assert a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()


def test_oracle_rmat_rows_sorted_distinct_symmetric(oracle):
    offs, nbr = oracle.generate_rmat(11, 20000, seed=2, keep_isolated=False)
    n = offs.shape[0] - 1
    deg = np.diff(offs)
    assert (deg > 0).all()  # isolated ids dropped
    rows = np.repeat(np.arange(n), deg)
    assert (nbr != rows).all()  # no self-loops
    for v in range(0, n, max(1, n // 200)):
        r = nbr[offs[v]:offs[v + 1]]
        assert (np.diff(r) > 0).all()
    fwd = set(zip(rows.tolist(), nbr.tolist()))
    assert all((b, a) in fwd for a, b in list(fwd)[:5000])


def test_oracle_rmat_rejects_bad_arguments(oracle):
    with pytest.raises(ValueError):
        oracle.generate_rmat(0, 100)
    with pytest.raises(ValueError):
        oracle.generate_rmat(10, 100, a=0.6, b=0.3, c=0.3)


def test_seq_louvain_karate_band(oracle, golden):
    n, offs, nbr, _ = read_bin(os.path.join(golden, "karate.txt.bin"))
    r = oracle.seq_louvain(offs, nbr)
    # published sequential Louvain results on karate lie in 0.415-0.42 with
    # 4 communities
    assert 0.41 <= r["modularity"] <= 0.4199
    assert len(np.unique(r["labels"])) in (3, 4, 5)
    q = oracle.modularity(offs, nbr, None, r["labels"])
    assert abs(q - r["modularity"]) < 1e-12


def test_seq_louvain_recovers_planted_partition(ffi, oracle):
    # config 1: 1,024 vertices in 32 blocks of 32, p_in 0.3, p_out 0.005
    g = ffi.Graph.sbm(1024, 32, 0.3, 0.005, 11)
    offs, nbr, _ = g.arrays()
    r = oracle.seq_louvain(offs, nbr)
    planted = (np.arange(1024) * 32 // 1024).astype(np.int32)
    q_planted = oracle.modularity(offs, nbr, None, planted)
    assert r["modularity"] >= q_planted - 1e-3
    assert abs(oracle.modularity(offs, nbr, None, r["labels"]) - r["modularity"]) < 1e-12
    # the communities found are the planted blocks (a low-degree vertex may
    # sit better in a neighbouring block: at most one per block)
    assert len(np.unique(r["labels"])) == 32
    for b in range(32):
        _, cnt = np.unique(r["labels"][b * 32:(b + 1) * 32], return_counts=True)
        assert cnt.max() >= 31


def test_seq_louvain_weighted_and_levels(oracle):
    offs, nbr = oracle.generate_rmat(12, 40000, seed=4, keep_isolated=False)
    rows = np.repeat(np.arange(offs.shape[0] - 1), np.diff(offs))
    w = (1 + (rows + nbr) % 4).astype(np.int32)
    r = oracle.seq_louvain(offs, nbr, w)
    assert r["levels"] >= 2
    # every level raises Q and lowers the community count
    assert all(b >= a for a, b in zip(r["level_q"], r["level_q"][1:]))
    assert all(b <= a for a, b in zip(r["level_c"], r["level_c"][1:]))
    assert abs(oracle.modularity(offs, nbr, w, r["labels"]) - r["modularity"]) < 1e-12
    # the synchronous oracle and the sequential method land within a few
    # hundredths of each other on this graph
    s = oracle.louvain(offs, nbr, w, nthreads=2)
    assert abs(s["modularity"] - r["modularity"]) < 0.05
