"""proposal_tool.py - trace capture and training of the learned move-proposal
network (gala_proposal_* in include/gala.h).  No counterpart in the reference.

Workflow (all on the GPU, through the C ABI):
  1. run the plain method in TRACE mode on seeded R-MAT graphs: the engine
     records the 8 features of sampled active vertices before each decision
     and labels them with the decision (moved or not);
  2. train the network on the samples with the library's own forward /
     backward kernels and Adam (gala_proposal_train);
  3. run with mode SKIP: only proposed vertices are decided, and every
     convergence is judged by a full plain sweep.

Command line:
  python proposal_tool.py --graphs 64 --scale-min 20 --scale-max 22 --out w.npy
writes the trained parameters (float32, 1377 values) to w.npy.
"""
import argparse
import json
import time

import numpy as np

import gala_ffi

# R-MAT parameters of the training graphs (mean degree about 17 after dedup)
RMAT_ABC = (0.57, 0.19, 0.19)
EDGE_FACTOR = 8.5


def rmat_graph(scale, seed, nthreads=0):
    edges = int(EDGE_FACTOR * (1 << scale))
    return gala_ffi.Graph.rmat(scale, edges, *RMAT_ABC, seed=seed, nthreads=nthreads)


def collect(proposal, graphs, sample_shift=0, ctx=None):
    """Plain runs in TRACE mode; returns the per-graph results."""
    out = []
    for g in graphs:
        n, e, _ = g.info()
        c = ctx or gala_ffi.Context(n, e)
        r = c.louvain(g, proposal=proposal, mode=gala_ffi.PROPOSAL_TRACE, sample_shift=sample_shift)
        out.append(r)
        if ctx is None:
            c.close()
    return out


def balance_weight(proposal):
    """Positive-class weight that balances moved and stayed samples."""
    n, pos = proposal.samples()
    if pos == 0:
        return 1.0
    return float(max(1.0, (n - pos) / pos))


def train(proposal, epochs=6, batch_size=4096, lr=3e-3, pos_weight=None, seed=0):
    if pos_weight is None:
        pos_weight = balance_weight(proposal)
    return proposal.train(epochs=epochs, batch_size=batch_size, lr=lr, pos_weight=pos_weight, seed=seed)


def train_on_rmat(proposal, seeds, scales, sample_shift=0, epochs=6, ctx=None, log=None):
    """Trace capture on R-MAT graphs (one per seed, scale cycling through
    `scales`), then training.  Returns (final loss, samples, positives)."""
    t0 = time.time()
    for i, s in enumerate(seeds):
        g = rmat_graph(scales[i % len(scales)], s)
        collect(proposal, [g], sample_shift, ctx)
        if log:
            log(f"traced seed {s}: samples {proposal.samples()}")
    n, pos = proposal.samples()
    loss = train(proposal, epochs=epochs)
    if log:
        log(f"trained on {n} samples ({pos} moved) in {time.time() - t0:.1f}s, loss {loss:.4f}")
    return loss, n, pos


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--graphs", type=int, default=64)
    ap.add_argument("--seed0", type=int, default=1000)
    ap.add_argument("--scale-min", type=int, default=20)
    ap.add_argument("--scale-max", type=int, default=22)
    ap.add_argument("--sample-shift", type=int, default=4)
    ap.add_argument("--max-samples", type=int, default=1 << 24)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--out", default="proposal_weights.npy")
    a = ap.parse_args()
    prop = gala_ffi.Proposal(max_samples=a.max_samples, seed=a.seed0)
    scales = list(range(a.scale_min, a.scale_max + 1))
    maxn = 1 << a.scale_max
    ctx = gala_ffi.Context(maxn, int(2 * EDGE_FACTOR * maxn) + 1)
    loss, n, pos = train_on_rmat(prop, range(a.seed0, a.seed0 + a.graphs), scales, a.sample_shift, a.epochs,
                                 ctx, log=print)
    np.save(a.out, prop.params())
    print(json.dumps({"samples": n, "positives": pos, "loss": loss, "out": a.out}))


if __name__ == "__main__":
    main()
