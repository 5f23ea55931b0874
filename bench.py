"""End-to-end Louvain throughput on one GB300 (and N independent replicas).

Workload: R-MAT, 2^22 ids, a/b/c/d = 0.57/0.19/0.19/0.05, 35.74M raw samples
-> 34.7M undirected edges after removing duplicates and self-loops (69.4M CSR
entries), unweighted, seed 1.  A step is one complete Louvain run: every
round of phase 1 + contraction until the round gain is below 1e-6.

  value   edges/s = m / (device time of one run), CSR already in HBM, timed
          with CUDA events on the stream the engine runs on
  e2e     the same through gala_louvain with host buffers: pinned CSR copied
          host->device, all rounds, labels copied device->host, every step
  e2e.learned_vs_plain  the learned move proposal's end-to-end time over
          the plain run's, and its final modularity difference
  roofline of the decide-and-move sweeps (algorithmic bytes / sweep time);
  roofline_contract  the same for the contractions
  cpu_baseline  the CPU oracle (the reference's algorithm restated on the
          host, all cores) on the same graph, and (cpu_baseline.sequential)
          the classic sequential Louvain on one core

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
N > 1 runs under torchrun: one independent replica per GPU (the path does
not shard), barrier + max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gala-mg_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, os.path.join(ROOT, "tests"))

WORKLOAD = {"workload": "rmat-s22-m34.7M", "generator": "R-MAT", "scale": 22, "raw_edges": 35_740_000,
            "a": 0.57, "b": 0.19, "c": 0.19, "d": 0.05, "seed": 1, "keep_isolated_ids": True,
            "weighted": False, "threshold": 1e-6}
SMALL = dict(WORKLOAD, workload="rmat-s16-small", scale=16, raw_edges=600_000)
METRIC = "end-to-end Louvain edges/s (all rounds to dQ<1e-6)"
FALLBACK_HBM_GBS = 6800.0


def max_over_ranks(dist, torch, value, device):
    """The slowest rank's value (every rank gets it)."""
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, units_per_replica, ms):
    """Whole-job throughput of `world` independent replicas that each process
    `units_per_replica` in `ms` (the slowest rank's time)."""
    return world * units_per_replica / (ms / 1000.0)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--small", action="store_true", help="tiny workload for a quick check")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-learned", action="store_true", help="skip the learned-proposal arm")
    p.add_argument("--no-batch", action="store_true", help="skip the batched-graphs arm")
    p.add_argument("--no-refine", action="store_true", help="skip the Leiden-style refinement arm")
    p.add_argument("--no-weighted", action="store_true", help="skip the float-weight LFR arm")
    p.add_argument("--no-calibrated", action="store_true",
                   help="skip the R-MAT stand-in without isolated vertices (scale 24)")
    p.add_argument("--tune-cache", default=None, help="JSON file caching autotuned degree bins per workload")
    p.add_argument("--threshold", type=float, default=0.3, help="proposal probability threshold")
    p.add_argument("--proposal-from", type=int, default=2,
                   help="first sweep of a level that decides only proposed vertices")
    p.add_argument("--profile", action="store_true",
                   help="one device-resident run and a short summary (for ncu captures)")
    p.add_argument("--profile-batch", type=int, default=0, metavar="G",
                   help="one batched run of the first G graphs of the batch workload (for ncu captures)")
    p.add_argument("--profile-learned", action="store_true",
                   help="one learned-proposal run (SKIP mode) after one plain run (for ncu launch lists)")
    p.add_argument("--fp64-gains", action="store_true", help="evaluate every gain in FP64")
    p.add_argument("--scale", type=int, default=0,
                   help="R-MAT scale of a smaller case of the same workload (raw samples scaled by 2^(scale-22))")
    return p.parse_args()


def make_graph(wl):
    import gala_ffi as ffi
    return ffi.Graph.rmat(wl["scale"], wl["raw_edges"], wl["a"], wl["b"], wl["c"], seed=wl["seed"],
                          noise=wl.get("noise", 0.0), keep_isolated=wl["keep_isolated_ids"])


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(name="decide_traffic_rmat-s21.md"):
    """DRAM bytes per algorithmic byte of a kernel family (the decide sweeps by
    default), from its committed ncu summary (a line
    'traffic_per_algorithmic_byte: X'), if any."""
    import re
    p = os.path.join(ROOT, "profiles", name)
    try:
        m = re.search(r"traffic_per_algorithmic_byte:\s*([0-9.]+)", open(p).read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def contraction_bytes(levels, r, weighted0=False):
    """Algorithmic bytes of the full contraction after round r (a round
    followed by another): read the row offsets (8 B), the label (4 B) of every
    vertex and write its new id (4 B); read every entry's neighbour id (4 B),
    the neighbour's label (4 B) and its weight (4 B, levels >= 1 or weighted
    input); write the new CSR: offsets (8 B per row + 1) and entries (4 B id +
    4 B weight)."""
    a, b = levels[r], levels[r + 1]
    wt = 4 if (r > 0 or weighted0) else 0
    return (a["vertices"] * (8 + 4 + 4) + a["entries"] * (4 + 4 + wt) + (b["vertices"] + 1) * 8 +
            b["entries"] * (4 + 4))


def contraction_roofline(runs, peak, peak_kind):
    """HBM roofline of the contractions that build a next level (all rounds
    but the last, which only relabels): algorithmic bytes / CUDA-event time."""
    byt = ms = 0.0
    for r in runs:
        lv = r["levels"]
        for i in range(len(lv) - 1):
            byt += contraction_bytes(lv, i)
            ms += lv[i]["contract_ms"]
    if ms <= 0:
        return None
    ach = byt / (ms / 1000.0) / 1e9
    lv = runs[-1]["levels"]
    tr = profile_traffic("contract_dram_rmat-s21.md")
    return {"bound": "hbm", "kernel": "contraction (renumber, member buckets, row aggregation, CSR write) of "
                                      "every round that builds a next level",
            "achieved": ach, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": ach / peak,
            "traffic": tr * byt / len(runs) if tr else None,
            "traffic_note": "DRAM bytes per run: ncu ratio (traffic / algorithmic bytes) measured at scale 21 "
                            "times this run's algorithmic bytes" if tr else None,
            "algorithmic_bytes_per_run": byt / len(runs), "ms_per_run": ms / len(runs),
            "level0_ms": lv[0]["contract_ms"], "level0_bytes": contraction_bytes(lv, 0) if len(lv) > 1 else None,
            "last_round_relabel_ms": lv[-1]["contract_ms"]}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def mark(self):
        """Samples before this call (warm-up) are not reported."""
        self.first = len(self.lines)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # samples of the timed region; if it was shorter than one sampling
        # period, the last warm-up sample (taken under the same load)
        first = getattr(self, "first", 0)
        lines = self.lines[first:] or self.lines[max(first - 1, 0):first]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle_run(offs, nbr, nthreads):
    from oracle_ffi import Oracle
    o = Oracle()
    t = time.perf_counter()
    r = o.louvain(offs, nbr, None, 1e-6, nthreads=nthreads)
    return time.perf_counter() - t, r


def cpu_model():
    """Host CPU model name (lscpu), for the CPU baseline record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def workload_config(wl, n, E, max_deg, world):
    """The `config` object of both arms (identical for the same workload)."""
    cfg = {k: v for k, v in wl.items()}
    cfg.update({"vertices": int(n), "edges": int(E) // 2, "csr_entries": int(E), "max_degree": int(max_deg),
                "l2": ("inputs larger than L2 (CSR %.0f MB > 129 MB)" if (E * 4 + (n + 1) * 8) > 129e6 else
                       "inputs smaller than L2 (CSR %.0f MB < 129 MB): a check run, not a bench value")
                      % ((E * 4 + (n + 1) * 8) / 1e6),
                "parallelism": f"replicas x{world}"})
    return cfg


def oracle_graph(wl):
    """The workload's graph built by the CPU oracle's generator
    (oracle/generators.c), identical to the engine library's (CPU test), so
    the CPU arm never loads the engine library."""
    from oracle_ffi import Oracle
    return Oracle().generate_rmat(wl["scale"], wl["raw_edges"], wl["a"], wl["b"], wl["c"], noise=wl.get("noise", 0.0),
                                  keep_isolated=wl["keep_isolated_ids"], seed=wl["seed"])


def seq_louvain_run(offs, nbr):
    from oracle_ffi import Oracle
    o = Oracle()
    t = time.perf_counter()
    r = o.seq_louvain(offs, nbr, None, 1e-6)
    return time.perf_counter() - t, r


def reference_arm(args, wl):
    """The reference's path on the host cores: the oracle port (the
    reference's GPU algorithm restated on the CPU, all host threads).  The
    graph comes from the oracle's generator: nothing of the engine (its
    library, kernels or Python binding) is loaded in this process."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    offs, nbr = oracle_graph(wl)
    n = offs.shape[0] - 1
    E = int(offs[-1])
    m = E // 2
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_oracle_run(offs, nbr, threads)
    times = []
    for _ in range(args.steps):
        dt, r = cpu_oracle_run(offs, nbr, threads)
        times.append(dt)
    sec = sum(times) / len(times)
    val = m / sec
    cfg = workload_config(wl, n, E, int(np.diff(offs).max()), world)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "edges/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1000, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/f64", "data": "synthetic", "config": cfg,
            "modularity": r["modularity"], "communities": r["level_c"][-1], "rounds": r["rounds"],
            "cpu_baseline": {"value": val, "unit": "edges/s", "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "full run on the whole workload (all rounds), oracle/louvain_oracle.c; "
                                       "graph from oracle/generators.c"},
            "e2e": {"value": val, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


WEIGHTS = os.path.join(ROOT, "gala-mg_gb300", "proposal_weights.npy")


def learned_arm(ffi, ctx, g, stream, args, torch, plain_ms, plain):
    """The learned move proposal (SKIP mode) end to end on the same graph:
    time relative to the plain method and final modularity difference."""
    import proposal_tool
    prop = ffi.Proposal(max_samples=1 << 22, seed=7)
    if os.path.exists(WEIGHTS):
        import numpy as np
        prop.set_params(np.load(WEIGHTS))
        source = "gala-mg_gb300/proposal_weights.npy (proposal_tool.py, 64 R-MAT graphs, seeds 1000-1063)"
    else:
        proposal_tool.train_on_rmat(prop, range(1000, 1008), [18, 19, 20], sample_shift=2, epochs=6, ctx=ctx)
        source = "trained in this run: 8 R-MAT graphs (scales 18-20, seeds 1000-1007)"
    def timed(threshold, steps, start=args.proposal_from):
        times, r = [], None
        for i in range(args.warmup + steps):
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                r = ctx.louvain(g, proposal=prop, mode=ffi.PROPOSAL_SKIP, threshold=threshold,
                                proposal_from=start)
                b.record(stream)
            torch.cuda.synchronize()
            if i >= args.warmup:
                times.append(a.elapsed_time(b))
        return sum(times) / len(times), r

    ms, r = timed(args.threshold, args.steps)
    # the proposal threshold (and the first sweep that may skip) against
    # decisions, sweeps, time and final Q
    curve = []
    for start, th in [(2, x) for x in (0.1, 0.2, 0.3, 0.4, 0.5)] + [(3, x) for x in (0.1, 0.3, 0.5)]:
        tms, tr = timed(th, min(args.steps, 3), start)
        curve.append({"threshold": th, "proposal_from": start, "ms": tms, "time_vs_plain": tms / plain_ms,
                      "decisions": tr["decisions"],
                      "skipped": tr["skipped"], "sweeps": tr["total_iterations"],
                      "verify_sweeps": tr["verify_sweeps"], "dq_vs_plain": tr["modularity"] - plain["modularity"]})
    prop.close()
    return {"mode": "skip", "threshold": args.threshold, "proposal_from": args.proposal_from, "weights": source,
            "ms_per_step": ms, "threshold_curve": curve,
            "time_vs_plain": ms / plain_ms, "modularity": r["modularity"],
            "dq_vs_plain": r["modularity"] - plain["modularity"], "decisions": r["decisions"],
            "plain_decisions": plain["decisions"], "skipped": r["skipped"], "verify_sweeps": r["verify_sweeps"],
            "iterations": r["total_iterations"], "plain_iterations": plain["total_iterations"],
            "phase_ms": {"decide": r["time_decide_ms"], "update": r["time_update_ms"],
                         "contract": r["time_contract_ms"]}}


REFINE_LFR = {"workload": "lfr-2M-unit", "vertices": 2_000_000, "tau1": 2.5, "dmin": 10, "dmax": 2000, "tau2": 1.5,
              "cmin": 20, "cmax": 5000, "mu": 0.3, "seed": 3}


def refine_arm(ffi, ctx, g, stream, args, torch, plain_ms, plain):
    """The Leiden-style refinement (gala_options.refine) end to end on the
    same graph: time and final modularity against the plain rounds."""
    times, r = [], None
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r = ctx.louvain(g, refine=True)
            b.record(stream)
        torch.cuda.synchronize()
        if i >= args.warmup:
            times.append(a.elapsed_time(b))
    ms = sum(times) / len(times)
    # a graph with planted communities (LFR-style, unit weights), where the
    # refinement is meant to help
    lg = ffi.Graph.lfr(REFINE_LFR["vertices"], REFINE_LFR["tau1"], REFINE_LFR["dmin"], REFINE_LFR["dmax"],
                       REFINE_LFR["tau2"], REFINE_LFR["cmin"], REFINE_LFR["cmax"], REFINE_LFR["mu"], False,
                       REFINE_LFR["seed"])
    lfr = {"config": REFINE_LFR}
    for key, flag in (("plain", False), ("refine", True)):
        ts = []
        for i in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rr = ctx.louvain(lg, refine=flag)
            torch.cuda.synchronize()
            if i:
                ts.append((time.perf_counter() - t0) * 1e3)
        lfr[key] = {"ms": sum(ts) / len(ts), "modularity": rr["modularity"], "rounds": rr["rounds"],
                    "communities": rr["num_communities"]}
    lfr["dq_refine_vs_plain"] = lfr["refine"]["modularity"] - lfr["plain"]["modularity"]
    return {"ms_per_step": ms, "time_vs_plain": ms / plain_ms, "modularity": r["modularity"], "lfr": lfr,
            "dq_vs_plain": r["modularity"] - plain["modularity"], "modularity_host_fp64": g.modularity(r["labels"]),
            "rounds": r["rounds"], "plain_rounds": plain["rounds"], "communities": r["num_communities"],
            "plain_communities": plain["num_communities"], "iterations": r["total_iterations"],
            "phase_ms": {"decide": r["time_decide_ms"], "update": r["time_update_ms"],
                         "contract_and_refine": r["time_contract_ms"]}}


# A second stand-in for config 2 whose vertices all have edges (ids without
# edges dropped, as the reference's preprocess does): scale 24, raw samples
# chosen so that m is about 34.7M after deduplication.
CALIBRATED = dict(WORKLOAD, workload="rmat-s24-m34.7M-no-isolated", scale=24, raw_edges=34_940_000,
                  keep_isolated_ids=False)


def calibrated_arm(ffi, args, torch, device):
    """Plain Louvain on the calibrated R-MAT (device-resident and end to end)."""
    c = CALIBRATED
    g = make_graph(c)
    offs, nbr, _ = g.arrays()
    n, E = offs.shape[0] - 1, int(offs[-1])
    g.pin()
    ctx = ffi.Context(n, E, device=device)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    d_offs = torch.from_numpy(offs).to(f"cuda:{device}")
    d_nbr = torch.from_numpy(nbr).to(f"cuda:{device}")
    d_out = torch.empty(n, dtype=torch.int32, device=f"cuda:{device}")
    dev, e2e, r, re_ = [], [], None, None
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        r = ctx.louvain_device(n, d_offs.data_ptr(), d_nbr.data_ptr(), None, d_out.data_ptr(), distinct_rows=True)
        torch.cuda.synchronize()
        if i >= args.warmup:
            dev.append(r["time_total_ms"])
    for i in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            re_ = ctx.louvain(g)
            b.record(stream)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e.append(a.elapsed_time(b))
    ctx.close()
    ms, ems = sum(dev) / len(dev), sum(e2e) / len(e2e)
    return {"config": workload_config(c, n, E, int(np.diff(offs).max()), 1), "ms_per_step": ms,
            "edges_per_s": (E // 2) / (ms / 1000.0), "e2e_ms": ems, "e2e_edges_per_s": (E // 2) / (ems / 1000.0),
            "modularity": r["modularity"], "rounds": r["rounds"], "iterations": r["total_iterations"],
            "communities": r["num_communities"],
            "labels_equal_e2e": bool((d_out.cpu().numpy() == re_["labels"]).all()),
            "phase_ms": {"decide": r["time_decide_ms"], "update": r["time_update_ms"],
                         "contract": r["time_contract_ms"]}}


WEIGHTED = {"workload": "lfr-16M-200M-f32", "generator": "LFR-style", "vertices": 16_000_000, "tau1": 2.5,
            "dmin": 10, "dmax": 20000, "tau2": 1.5, "cmin": 20, "cmax": 50000, "mu": 0.3,
            "weights": "lognormal(0,1) float32", "seed": 1}


def weighted_arm(ffi, args, torch, device):
    """Float-weight LFR-style graph (16M vertices, about 200M edges): the
    whole run through gala_louvain (host graph in, labels out), weights as
    64-bit fixed point, gains in FP64; modularity against the host FP64
    recomputation on the float weights."""
    c = WEIGHTED
    t0 = time.perf_counter()
    g = ffi.Graph.lfr(c["vertices"], c["tau1"], c["dmin"], c["dmax"], c["tau2"], c["cmin"], c["cmax"], c["mu"],
                      True, c["seed"])
    gen_s = time.perf_counter() - t0
    n, e, _ = g.info()
    m = e // 2
    g.pin()
    ctx = ffi.Context(n, e, device=device)
    steps = max(1, min(args.steps, 2))
    times, r = [], None
    for i in range(1 + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.louvain(g)
        torch.cuda.synchronize()
        if i >= 1:
            times.append(time.perf_counter() - t0)
    ctx.close()
    sec = statistics.median(times)
    q_host = g.modularity(r["labels"])
    return {"config": dict(c, edges=m, csr_entries=e, generation_s=gen_s),
            "metric": "end-to-end Louvain edges/s (float weights, all rounds to dQ<1e-6)", "value": m / sec,
            "unit": "edges/s", "seconds": sec, "seconds_each": times, "device_ms": r["time_total_ms"],
            "h2d_ms": r["time_h2d_ms"], "d2h_ms": r["time_d2h_ms"], "host_ms": r["host_ms"], "steps": steps,
            "warmup": 1,
            "phase_ms": {"decide": r["time_decide_ms"], "update": r["time_update_ms"],
                         "contract": r["time_contract_ms"]},
            "modularity": r["modularity"], "modularity_host_fp64": q_host,
            "abs_diff_vs_host": abs(q_host - r["modularity"]), "rounds": r["rounds"],
            "iterations": r["total_iterations"], "communities": r["num_communities"]}


BATCH = {"workload": "sbm-batch-4096", "graphs": 4096, "n_min": 200, "n_max": 3500, "k_min": 8, "k_max": 64,
         "deg_min": 12.0, "deg_max": 40.0, "mix_min": 0.1, "mix_max": 0.4, "seed": 1}


def batch_arm(ffi, args, torch, device):
    """4096 uneven planted-partition graphs (about 60M edges) in one batched
    run (gala_louvain_batch, host graphs in, host labels out), against
    single-graph runs of a sample of the same graphs."""
    b = BATCH
    gs = ffi.Graph.sbm_batch(b["graphs"], b["n_min"], b["n_max"], b["k_min"], b["k_max"], b["deg_min"],
                             b["deg_max"], b["mix_min"], b["mix_max"], seed=b["seed"])
    ns = [g.info()[0] for g in gs]
    es = [g.info()[1] for g in gs]
    m = sum(es) // 2
    ctx = ffi.Context(sum(ns), sum(es), device=device)
    # page-lock the host graphs (untimed, as for the main graph): when every
    # graph is page-locked the GPU reads them in place; otherwise the run
    # copies them through the context's pinned staging
    pinned = 0
    for g in gs:
        try:
            g.pin()
            pinned += 1
        except ffi.GalaError:
            pass
    # degree bins tuned on this batch (untimed; cached in --tune-cache when given)
    tuning = None
    if args.tune_cache and os.path.exists(args.tune_cache):
        tuning = json.load(open(args.tune_cache)).get(b["workload"])
    if tuning is None:
        tuning = ctx.autotune(gs, repeats=1, use_graphs=1, batch_mode=1)  # the bins tune the union run
        if args.tune_cache:
            cache = json.load(open(args.tune_cache)) if os.path.exists(args.tune_cache) else {}
            cache[b["workload"]] = tuning
            json.dump(cache, open(args.tune_cache, "w"))
    def timed(mode):
        times, r = [], None
        for i in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = ctx.louvain_batch(gs, use_graphs=True, tuning=tuning, batch_mode=mode)
            torch.cuda.synchronize()
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
        return statistics.median(times), r

    # the union run (every sweep one set of launches for all graphs), for
    # comparison; then the default: one persistent launch, one CTA per graph
    usec, ur = timed(1)
    sec, r = timed(0)
    for a, b_ in zip(r["labels"], ur["labels"]):
        assert (a == b_).all()
    ctx.close()
    sample = list(range(0, b["graphs"], 128))
    single = ffi.Context(max(ns), max(es), device=device)
    st, equal, maxdq = 0.0, 0, 0.0
    for i in sample:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s1 = single.louvain(gs[i])
        torch.cuda.synchronize()
        st += time.perf_counter() - t0
        equal += int((s1["labels"] == r["labels"][i]).all())
        maxdq = max(maxdq, abs(s1["modularity"] - r["modularity"][i]))
    single.close()
    seq_est = st / len(sample) * b["graphs"]
    return {"config": dict(b, vertices=sum(ns), edges=m, max_vertices=max(ns), min_vertices=min(ns)),
            "metric": "batched Louvain edges/s (host graphs in, labels out)", "value": m / sec, "unit": "edges/s",
            "seconds": sec, "device_ms": r["time_total_ms"], "h2d_ms": r["time_h2d_ms"], "d2h_ms": r["time_d2h_ms"],
            "input": ("page-locked host graphs, read in place by the GPU (one gather kernel)" if pinned == len(gs)
                      else "host graphs (%d of %d page-locked): raw copies into the context's pinned staging, one "
                           "transfer, ids shifted on the device" % (pinned, len(gs))),
            "phase1_ms": r["time_phase1_ms"],
            "contract_ms": r["time_contract_ms"], "levels": r["num_levels"], "iterations": r["total_iterations"],
            "kernel_launches": r["kernel_launches"],
            "mode": "one persistent launch, one CTA per graph (all rounds)" if r["kernel_launches"] < 10 else "union",
            "union_run": {"seconds": usec, "device_ms": ur["time_total_ms"], "kernel_launches": ur["kernel_launches"],
                          "tuning": tuning, "cuda_graphs": True, "labels_equal": True},
            "sequential_single_runs_s_est": seq_est, "speedup_vs_sequential": seq_est / sec,
            "checked_graphs": len(sample), "labels_equal_single_runs": equal, "max_dq_vs_single": maxdq}


def main():
    args = parse()
    wl = SMALL if args.small else WORKLOAD
    if args.scale:
        wl = dict(WORKLOAD, workload=f"rmat-s{args.scale}", scale=args.scale,
                  raw_edges=WORKLOAD["raw_edges"] >> (22 - args.scale))
    if args.impl == "reference":
        reference_arm(args, wl)
        return
    import torch
    import gala_ffi as ffi
    if args.profile_batch:
        b = BATCH
        gs = ffi.Graph.sbm_batch(args.profile_batch, b["n_min"], b["n_max"], b["k_min"], b["k_max"], b["deg_min"],
                                 b["deg_max"], b["mix_min"], b["mix_max"], seed=b["seed"])
        bctx = ffi.Context(sum(g.info()[0] for g in gs), sum(g.info()[1] for g in gs))
        r = bctx.louvain_batch(gs)
        torch.cuda.synchronize()
        print(json.dumps({"profile_batch": args.profile_batch, "device_ms": r["time_total_ms"],
                          "kernel_launches": r["kernel_launches"], "levels": r["num_levels"]}), flush=True)
        bctx.close()
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    g = make_graph(wl)
    offs, nbr, _ = g.arrays()
    n = offs.shape[0] - 1
    E = int(offs[-1])
    m = E // 2
    max_deg = int((offs[1:] - offs[:-1]).max())
    g.pin()
    ctx = ffi.Context(n, E, device=local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    d_offs = torch.from_numpy(offs).to(f"cuda:{local}")
    d_nbr = torch.from_numpy(nbr).to(f"cuda:{local}")
    d_out = torch.empty(n, dtype=torch.int32, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def run_device():
        # the generator deduplicates every row
        return ctx.louvain_device(n, d_offs.data_ptr(), d_nbr.data_ptr(), None, d_out.data_ptr(),
                                  fp64_gains=args.fp64_gains, distinct_rows=True)

    if args.profile_learned:
        import numpy as np
        prop = ffi.Proposal(max_samples=1 << 16, seed=7)
        prop.set_params(np.load(WEIGHTS))
        r0 = ctx.louvain(g)
        r = ctx.louvain(g, proposal=prop, mode=ffi.PROPOSAL_SKIP, threshold=args.threshold)
        torch.cuda.synchronize()
        print(json.dumps({"profile_learned": wl["workload"], "plain_ms": r0["time_total_ms"],
                          "learned_ms": r["time_total_ms"], "decisions": r["decisions"],
                          "plain_decisions": r0["decisions"], "sweeps": r["total_iterations"],
                          "plain_sweeps": r0["total_iterations"]}), flush=True)
        prop.close()
        ctx.close()
        return
    if args.profile:
        r = run_device()
        torch.cuda.synchronize()
        print(json.dumps({"profile": wl["workload"], "ms": r["time_total_ms"], "rounds": r["rounds"],
                          "iterations": r["total_iterations"], "modularity": r["modularity"],
                          "decide_ms": r["time_decide_ms"], "update_ms": r["time_update_ms"],
                          "contract_ms": r["time_contract_ms"], "decide_bytes": r["decide_bytes"],
                          "sweeps": r["decide_sweeps"], "fp64_decisions": r["fp64_decisions"],
                          "levels": r["levels"]}), flush=True)
        ctx.close()
        return

    # the clock sampler starts before the warm-up: its start-up (NVML
    # initialisation in a separate process) stays out of the timed region
    clocks = Clocks(local)
    clocks.start()
    for _ in range(args.warmup):
        r = run_device()
    # ---- device-resident timed region ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.mark()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    l0 = ffi.launch_count()
    dec_bytes = dec_ms = 0.0
    sweeps = 0
    runs = []
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            r = run_device()
            runs.append(r)
            dec_bytes += r["decide_bytes"]
            dec_ms += r["time_decide_ms"]
            sweeps += r["decide_sweeps"]
        ev1.record(stream)
    torch.cuda.synchronize()
    launches = ffi.launch_count() - l0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    if dist:
        ms = max_over_ranks(dist, torch, ms, f"cuda:{local}")
        dist.barrier()
    value = replica_throughput(world, m, ms)

    # ---- end to end through the C ABI with host buffers ----
    r_e2e = None
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r_e2e = ctx.louvain(g)
            b.record(stream)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append(a.elapsed_time(b))
    e2e_step = sum(e2e_ms) / len(e2e_ms)
    if dist:
        e2e_step = max_over_ranks(dist, torch, e2e_step, f"cuda:{local}")

    peak, peak_kind = measured_peak()
    achieved = (dec_bytes / (dec_ms / 1000.0)) / 1e9 if dec_ms > 0 else 0.0
    tr = profile_traffic()
    roof = {"bound": "hbm", "kernel": "decide-and-move sweep (all degree bins of one iteration)",
            "achieved": achieved, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": (tr * dec_bytes / max(sweeps, 1)) if tr else None,
            "traffic_note": "DRAM bytes per sweep: ncu ratio (traffic / algorithmic bytes) measured at "
                            "scale 21 times this run's algorithmic bytes per sweep" if tr else None,
            "algorithmic_bytes_per_sweep": dec_bytes / max(sweeps, 1),
            "sweep_ms": dec_ms / max(sweeps, 1), "sweeps_per_run": sweeps / args.steps}

    last = runs[-1]
    contract_roof = contraction_roofline(runs, peak, peak_kind)
    cfg = workload_config(wl, n, E, max_deg, world)
    e2e = {"value": world * m / (e2e_step / 1000.0), "unit": "edges/s", "ms_per_step": e2e_step,
           "h2d_bytes_per_step": r_e2e["h2d_bytes"], "d2h_bytes_per_step": r_e2e["d2h_bytes"],
           "h2d_ms": r_e2e["time_h2d_ms"], "d2h_ms": r_e2e["time_d2h_ms"], "host_ms": r_e2e["host_ms"]}
    # bulky secondary arms first, the headline keys after them (the end of
    # the line is what a truncated log keeps).  The float-weight arm runs
    # first: its 3.4 GB host-to-device copy took 376 ms in a run where it came
    # after the refinement and batch arms (the batch arm page-locks thousands
    # of small graphs), against 20-38 ms in a process of its own.
    line = {}
    if not args.no_weighted:
        line["weighted"] = weighted_arm(ffi, args, torch, local)
    if not args.no_calibrated:
        line["calibrated"] = calibrated_arm(ffi, args, torch, local)
    if not args.no_refine:
        line["refine"] = refine_arm(ffi, ctx, g, stream, args, torch, e2e_step, r_e2e)
    if not args.no_batch:
        line["batch"] = batch_arm(ffi, args, torch, local)
    line.update({"metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world, "steps": args.steps,
                 "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                 "vs_baseline": None, "dtype": "int32/f64", "data": "synthetic", "config": cfg,
                 "seconds_per_run": ms / 1000.0, "modularity": last["modularity"],
                 "communities": last["num_communities"], "rounds": last["rounds"],
                 "iterations": last["total_iterations"], "fp64_decisions": last["fp64_decisions"],
                 "phase_ms": {"phase1": last["time_phase1_ms"], "decide": last["time_decide_ms"],
                              "update": last["time_update_ms"], "contract": last["time_contract_ms"]},
                 "gpu_launches": launches})
    if not args.no_learned:
        lr = learned_arm(ffi, ctx, g, stream, args, torch, e2e_step, r_e2e)
        line["learned"] = lr
        # the second half of the headline metric: learned-prune time / plain
        # time end to end, at |dQ| <= 0.002
        e2e["learned_vs_plain"] = {"time_vs_plain": lr["time_vs_plain"], "dq_vs_plain": lr["dq_vs_plain"],
                                   "plain_ms": e2e_step, "learned_ms": lr["ms_per_step"],
                                   "threshold": lr["threshold"], "proposal_from": lr["proposal_from"],
                                   "decisions": lr["decisions"],
                                   "plain_decisions": lr["plain_decisions"], "target": "<= 0.5 at |dQ| <= 0.002"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        dt, ro = cpu_oracle_run(offs, nbr, threads)
        sdt, so = seq_louvain_run(offs, nbr)
        line["cpu_baseline"] = {"value": m / dt, "unit": "edges/s", "cores": threads, "kind": "port",
                                "cpu_model": cpu_model(),
                                "sample": "one full run (all rounds) of the oracle on the whole workload",
                                "seconds": dt, "modularity": ro["modularity"],
                                "labels_equal_gpu": bool((ro["labels"] == r_e2e["labels"]).all()),
                                "sequential": {"value": m / sdt, "unit": "edges/s", "cores": 1,
                                               "kind": "sequential",
                                               "algorithm": "Blondel et al. 2008 asynchronous Louvain, "
                                                            "oracle/seq_louvain.c, -O3, 1 thread",
                                               "sample": "one full run (all levels) on the whole workload",
                                               "seconds": sdt, "modularity": so["modularity"],
                                               "levels": so["levels"], "communities": so["level_c"][-1]}}
    line["e2e"] = e2e
    line["roofline"] = roof
    if contract_roof:
        line["roofline_contract"] = contract_roof
    line["clocks"] = clk
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
