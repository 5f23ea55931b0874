"""Regenerate the golden fixtures in this folder (run in a tree where the
reference sources are mounted; the fixtures themselves are committed).

Fixtures
--------
karate.txt / karate.txt.bin
    Zachary's karate club (34 vertices, 78 edges) as an edge list, taken from
    networkx.karate_club_graph(), and its .bin as written by the REFERENCE's
    own `preprocess` (src/preprocess.cpp + src/graph/graph.cpp, rebuilt from
    source by oracle/Makefile into oracle/_ref/).
karate_trace.json
    The per-iteration modularity and per-round community counts that the
    reference prints for this graph (README.md:55-90).
sbm_s{seed}.txt.bin
    Planted-partition SBM, 1,024 vertices in 32 blocks of 32, p_in = 0.3,
    p_out = 0.005, seeds 0 and 1, converted by the reference `preprocess`.
sbm_s{seed}.expect.json
    The oracle's multi-round result on that file (rounds, Q per round,
    community counts, and every iteration's Q).

Usage:  python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_PRE = os.path.join(ROOT, "oracle", "_ref", "preprocess")


def write_edges(path, edges):
    with open(path, "w") as f:
        f.write("# undirected edge list\n")
        for u, v in edges:
            f.write(f"{u} {v}\n")


def ref_preprocess(txt):
    if not os.path.exists(REF_PRE):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref"])
    subprocess.check_call([REF_PRE, "-f", txt], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return txt + ".bin"


def sbm_edges(n, k, p_in, p_out, seed):
    rng = np.random.default_rng(seed)
    blk = np.arange(n) // (n // k)
    iu, ju = np.triu_indices(n, 1)
    p = np.where(blk[iu] == blk[ju], p_in, p_out)
    keep = rng.random(iu.shape[0]) < p
    return list(zip(iu[keep].tolist(), ju[keep].tolist()))


def main():
    import networkx as nx

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_ffi import Oracle, read_bin  # noqa: E402

    g = nx.karate_club_graph()
    kt = os.path.join(HERE, "karate.txt")
    write_edges(kt, sorted((min(u, v), max(u, v)) for u, v in g.edges()))
    ref_preprocess(kt)
    # README.md:59-89 (reference), printed with %f
    trace = {
        "source": "reference README.md:55-90",
        "vertices": 34,
        "edges": 78,
        "rounds": [
            {"iterations_q": ["-0.049803", "0.136834", "0.191239", "0.169214"], "communities": 11,
             "modularity": "0.191239"},
            {"iterations_q": ["0.191239", "0.313116", "0.401134", "0.408695", "0.408695"],
             "communities": 4, "modularity": "0.408695"},
            {"iterations_q": ["0.408695", "0.408695"], "communities": 4, "modularity": "0.408695"},
        ],
        "final": {"from": 34, "to": 4, "modularity": "0.408695"},
    }
    with open(os.path.join(HERE, "karate_trace.json"), "w") as f:
        json.dump(trace, f, indent=1)

    orc = Oracle()
    for seed in (0, 1):
        st = os.path.join(HERE, f"sbm_s{seed}.txt")
        write_edges(st, sbm_edges(1024, 32, 0.3, 0.005, seed))
        b = ref_preprocess(st)
        os.remove(st)
        n, offs, nbr, w = read_bin(b, weighted=False)
        res = orc.louvain(offs, nbr, None, 1e-6)
        with open(os.path.join(HERE, f"sbm_s{seed}.expect.json"), "w") as f:
            json.dump({
                "source": "oracle (orc_louvain) on the reference preprocess output",
                "rounds": res["rounds"],
                "level_q": [repr(x) for x in res["level_q"]],
                "level_c": res["level_c"],
                "level_iters": res["level_iters"],
                "iter_q": [repr(x) for x in res["iter_q"]],
                "final_communities": int(res["level_c"][-1]),
            }, f, indent=1)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
