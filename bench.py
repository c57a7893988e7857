"""Benchmark: exact treedepth solves on GB300.

Workload (default, ``--workload dp-c2``): the single-graph subset DP at scale,
8 connected G(n, p) graphs (n in {28, 30, 32}, p in {0.1, 0.2, 0.3}, seeds
1-8) plus the 5 x 6 grid. One step solves all 9 graphs exactly (DP table +
elimination tree). The DP tables (256 MiB - 4 GiB) are larger than L2, so no
flush is needed between steps.

The same line carries more measurements of the run:
  dp_c3      batched uneven DP, 4096 graphs n in [10, 24] (three families), one
             persistent launch per step replayed from a CUDA graph, tile sizes
             per vertex count planned from the autotuner's rates;
  bottom_up  the bottom-up union-find heuristic DP at n = 20 / 26 / 30, and the
             oracle's restatement on one host thread at n = 20;
  bnb_c4     plain vs learned-guided GPU branch and bound on 256 sparse graphs
             n in [40, 64] (random geometric, random 3-regular, deleted grids)
             with a 10 s per-graph cap, on three graph samples: plain =
             ascending candidate order (the reference's DefaultAttemptOrder)
             and the reference heuristic's incumbent; learned = the GNN's score
             order, the better of that incumbent and a score-greedy
             elimination, and its td estimate as the first level. The GNN is
             trained in the run, on the GPU, from ~201 K labels the GPU DP
             computes;
  bnb_c5     the config-5 stream (1024 graphs, n in [20, 80], 60 s cap), the
             same arms, plus the size-dispatch hybrid.

Arms:
  default            gtd on the GPU; ``value`` = solves/s with inputs resident
                     on the device; ``e2e`` = the same through the host-buffer
                     C-ABI call gtd_dp_solve (H2D/D2H copies inside the timed
                     region).
  --impl reference   the reference's CPU algorithm (the oracle restatement of
                     DynamicGPU's recurrence, dynamic_gpu.cu:68-112, on all
                     host threads) on the same 9 graphs: each step solves one
                     graph (table, tree, elimination order), cycling through
                     all of them, and the rate is the workload's 9 graphs over
                     the sum of their mean times. The ``config`` object is the
                     same in both arms.

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "exact-treedepth solves/s & p50 time-to-proof: learned-guided vs plain GPU B&B"
WORKLOAD_C2 = ("dp-c2 (config 2: 8 connected G(n,p), n in {28,30,32}, p in {0.1,0.2,0.3}, seeds 1-8, "
               "+ grid 5x6; exact DP + elimination tree per graph)")
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gtd", choices=["gtd", "reference"])
    ap.add_argument("--workload", default="dp-c2", choices=["dp-c2", "bnb-c5"],
                    help="dp-c2: the default line; bnb-c5: the config-5 B&B stream")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--partition", action="store_true",
                    help="N > 1: split the workload's graphs over the ranks, size-balanced (strong scaling) "
                         "instead of every rank solving all of them (replicas, weak scaling)")
    ap.add_argument("--only-n", type=int, default=0,
                    help="restrict the workload to its graphs with this n (profiling)")
    ap.add_argument("--tile-bits", type=int, default=0,
                    help="DP tile bits (0 = the library's default)")
    ap.add_argument("--no-c3", action="store_true", help="skip the batched DP measurement")
    ap.add_argument("--no-bottom-up", action="store_true", help="skip the bottom-up heuristic measurement")
    ap.add_argument("--c3-graphs", type=int, default=4096, help="graphs of the batched DP measurement (config 3)")
    ap.add_argument("--no-bnb", action="store_true", help="skip the plain vs learned B&B measurement")
    ap.add_argument("--bnb-graphs", type=int, default=None,
                    help="B&B graphs (default 256 of config 4; 1024 of config 5 with --workload bnb-c5)")
    ap.add_argument("--bnb-cap-s", type=float, default=None,
                    help="B&B per-graph cap on time to proof (default 10 s; 60 s with --workload bnb-c5)")
    ap.add_argument("--cpu-bnb-sample", type=int, default=32, help="config-4 graphs in the CPU B&B baseline")
    ap.add_argument("--cpu-bnb-nodes", type=int, default=20_000_000,
                    help="search-node cap per graph of the CPU B&B baseline")
    ap.add_argument("--c4-seeds", type=int, nargs="+", default=[4, 41, 42],
                    help="config-4 graph sample seeds, one plain-vs-learned run each (spread over runs)")
    ap.add_argument("--no-c5", action="store_true", help="skip the config-5 stream in the default line")
    ap.add_argument("--c5-graphs", type=int, default=1024, help="graphs of the config-5 stream")
    ap.add_argument("--c5-cap-s", type=float, default=60.0, help="per-graph cap of the config-5 stream")
    ap.add_argument("--bnb-memo-log2", type=int, default=0,
                    help="B&B memo slots per graph as a power of two (0 = sized from free HBM)")
    ap.add_argument("--label-graphs", type=int, default=10500,
                    help="graphs (n <= 24, config-2/3 families) whose DP tables label the GNN training set "
                         "(each gives itself and up to 20 distinct sampled subgraphs: ~201K labels at the "
                         "default)")
    args = ap.parse_args()
    c5 = args.workload == "bnb-c5"
    if args.bnb_graphs is None:
        args.bnb_graphs = 1024 if c5 else 256
    if args.bnb_cap_s is None:
        args.bnb_cap_s = 60.0 if c5 else 10.0
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def job_rate(units_per_rank, elapsed_s, world):
    """Whole-job throughput of N replicas: every rank's units over the slowest
    rank's time (max over ranks by an all-reduce of the process group when
    world > 1). Returns (rate, slowest elapsed seconds)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(elapsed_s)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_s = float(t.item())
    return units_per_rank * world / elapsed_s, elapsed_s


def partition_graphs(graphs, world):
    """Size-balanced split of a graph list over `world` ranks (longest first
    to the least-loaded rank; the cost of a DP solve is 2^n): rank r solves
    the graphs at the indices parts[r]. Deterministic, so every rank computes
    the same split without communicating."""
    loads = [0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(graphs)), key=lambda i: (-graphs[i].n, i)):
        r = min(range(world), key=lambda r: (loads[r], r))
        parts[r].append(i)
        loads[r] += 2 ** graphs[i].n
    return [sorted(p) for p in parts]


def job_rate_total(units, elapsed_s, world):
    """Whole-job throughput when the ranks share one workload: the sum of
    the ranks' units over the slowest rank's time (all-reduces of the
    process group when world > 1). Returns (rate, slowest elapsed seconds)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(elapsed_s)], dtype=torch.float64)
        u = torch.tensor([float(units)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        elapsed_s, units = float(t.item()), float(u.item())
    return units / elapsed_s, elapsed_s


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def ncu_profile_figure(key):
    """A figure of the DP tile kernel's ncu capture on an n = 28 launch
    (profiles/dp_tile_kernel.md, line '<key>: <value>')."""
    path = os.path.join(ROOT, "profiles", "dp_tile_kernel.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def ncu_bytes_per_subset():
    """DRAM bytes per subset of the DP tile kernel (ncu, n = 28 launch)."""
    return ncu_profile_figure("dram_bytes_per_subset")


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


# ---------------------------------------------------------------------------
# CPU legs (the oracle is loaded only here).
# ---------------------------------------------------------------------------

def config_c2(graphs):
    """The workload's config object, identical in both arms."""
    return {"workload": WORKLOAD_C2, "graphs": [g.name for g in graphs],
            "l2": "working set (DP tables 256 MiB-4 GiB) > L2"}


def cpu_sample_graphs(graphs):
    """One graph of each vertex count of the workload (the bounded sample of
    the GPU arm's CPU baseline)."""
    seen, out = set(), []
    for g in graphs:
        if g.n not in seen:
            seen.add(g.n)
            out.append(g)
    return out


def workload_rate(graphs, samples):
    """Solves/s of the whole workload from per-graph CPU times: the workload's
    graph count over the sum of each graph's mean time; a graph that was not
    timed takes the mean time of the timed graphs with its vertex count."""
    by_name, by_n = {}, {}
    for g, t in samples:
        by_name.setdefault(g.name, []).append(t)
        by_n.setdefault(g.n, []).append(t)
    total = 0.0
    for g in graphs:
        ts = by_name.get(g.name) or by_n.get(g.n)
        if not ts:
            return None
        total += statistics.mean(ts)
    return len(graphs) / total


def cpu_dp_solve(port, g, threads):
    """The oracle's restatement of DynamicGPU (dynamic_gpu.cu:68-112: the
    all-subsets table), its tree (dynamic_cpu.hpp:59-81) and GetElimination
    order (dynamic_gpu.hpp:48-64) for one graph: (td, parent, order)."""
    T = port.dp_table(g, nthreads=threads)
    td, par = port.tree_from_table(g, T)
    order = port.get_elimination(g, T, (1 << g.n) - 1)
    del T
    return td, par, order


def time_cpu_dp(graphs, steps, threads, start=0):
    """Steps of one graph each, cycling through `graphs` from index `start`:
    [(graph, seconds, (td, parent, order))]."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    port = oracle.Port()
    out = []
    for i in range(steps):
        g = graphs[(start + i) % len(graphs)]
        t0 = time.perf_counter()
        res = cpu_dp_solve(port, g, threads)
        out.append((g, time.perf_counter() - t0, res))
    return out


def time_cpu_bnb(graphs, node_limit, threads):
    """The oracle's restatement of the reference BranchAndBound (EdgeLowerBound,
    HighestDegree(Variance) incumbent) on `threads` host threads, one graph per
    thread at a time, each capped at node_limit search nodes."""
    from concurrent.futures import ThreadPoolExecutor
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    port = oracle.Port()

    def one(g):
        t0 = time.perf_counter()
        st, td, _, nodes = port.bnb(g, node_limit=node_limit)
        return st, td, nodes, time.perf_counter() - t0

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:  # ctypes calls release the GIL
        res = list(ex.map(one, graphs))
    return res, time.perf_counter() - t0


def run_reference(args, graphs):
    """The reference's algorithm for this workload on the host cores: every
    step solves one graph of the workload (table, tree and elimination order),
    cycling through all of them; the rate is the whole workload's (its graph
    count over the sum of the graphs' mean times), so both arms report the
    same quantity on the same graphs."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    small = [g for g in graphs if g.n == min(x.n for x in graphs)]
    time_cpu_dp(small, args.warmup, threads)  # warm-up on the smallest graphs
    res = time_cpu_dp(graphs, args.steps, threads)
    samples = [(g, t) for g, t, _ in res]
    value = workload_rate(graphs, samples)
    timed = sorted({g.name for g, _ in samples})
    desc = (f"all {len(graphs)} graphs of the workload, one per step in turn ({len(timed)} timed); "
            f"oracle restatement of DynamicGPU's all-subsets recurrence (dynamic_gpu.cu:68-112) with the "
            f"tree and GetElimination order, on {threads} host threads; rate = graphs / sum of per-graph "
            f"mean times")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * sum(t for _, t in samples) / len(samples), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": config_c2(graphs), "parallelism": f"{threads} host threads",
        "per_graph_s": {name: statistics.mean(t for g, t in samples if g.name == name) for name in timed},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": desc, "cpu": cpu_model()},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm.
# ---------------------------------------------------------------------------

def measure_dp_c3(h, steps, warmup, count=4096):
    """Batched uneven DP on config 3 (4096 graphs), device time from the
    library's events and host time of the whole C-ABI call."""
    import numpy as np

    from gisbdw_gb300 import _lib
    from gisbdw_gb300 import graphs as G
    from gisbdw_gb300.validate import check_tree
    graphs = G.config3_graphs(count=count)
    packed = _lib.pack_batch(graphs)
    t0 = time.perf_counter()
    rates, mixed_eff = h.dp_autotune(10, 24, with_mixed=True)  # subsets/us per (n, tile bits 8..12)
    tune_s = time.perf_counter() - t0
    for _ in range(warmup):
        td, pars, st = h.dp_solve_batch(graphs, packed=packed)
    # every graph: a valid tree of height td, and the same td and parent array
    # as the single-graph entry point (a separate launch path and layout)
    bad = [g.name for g, t, p in zip(graphs, td, pars) if not check_tree(g, int(t), p)]
    single_differs = []
    for g, t, p in zip(graphs, td, pars):
        std, spar, _, _ = h.dp_solve(g.adj64(), g.n, want_order=False)
        if std != int(t) or spar.tolist() != p.tolist():
            single_differs.append(g.name)
    dev, host = [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        td, pars, st = h.dp_solve_batch(graphs, packed=packed)
        host.append(time.perf_counter() - t0)
        dev.append(st["dp_ms"])
    # the same batch at every single tile size: what the plan chose against
    one_size = {}
    for lb in range(8, 13):
        h.dp_solve_batch(graphs, packed=packed, tile_bits=lb)
        one_size[str(lb)] = statistics.median(h.dp_solve_batch(graphs, packed=packed, tile_bits=lb)[2]["dp_ms"]
                                              for _ in range(max(3, steps // 2)))
    peak, peak_kind = peaks()
    ms = statistics.median(dev)
    return {"graphs": len(graphs), "solves_per_s": len(graphs) / (ms / 1e3), "dp_ms": ms,
            "tile_bits_by_n": st["tile_bits_by_n"], "mixed_sizes": len(set(st["tile_bits_by_n"].values())) > 1,
            "one_size_dp_ms": one_size,
            "autotune_rates_subsets_per_us": {str(10 + i): [round(float(x), 1) for x in row]
                                              for i, row in enumerate(rates)},
            "autotune_mixed_kernel_efficiency": [round(float(x), 3) for x in mixed_eff],
            "e2e_solves_per_s": len(graphs) / statistics.median(host), "alg_bytes": st["alg_bytes"],
            "alg_GBps": st["alg_bytes"] / (ms / 1e3) / 1e9, "frac_of_" + peak_kind + "_hbm":
            st["alg_bytes"] / (ms / 1e3) / 1e9 / peak, "tile_bits": st["tile_bits"], "ctas": st["ctas"],
            "cuda_graph_replayed": bool(st["graph_replayed"]), "trees_checked": len(graphs),
            "trees_invalid": bad, "td_parent_equal_to_single_solves": not single_differs,
            "differs_from_single": single_differs[:8],
            "autotune_s": tune_s, "autotune_best_bits_n24": int(8 + rates[-1].argmax())}


def measure_bottom_up(h, cpu=1):
    """The bottom-up union-find heuristic DP (gtd_bottom_up) on connected
    G(n, 0.2) graphs: device time per graph, its algorithmic bytes (per
    subset S: |S| child rows of 32 B and |S| child heights read, one 32-byte
    row, a height and a history byte written) over that time, and the
    oracle's restatement timed on one host thread at the smallest n with its
    order compared."""
    from gisbdw_gb300 import graphs as G
    peak, peak_kind = peaks()
    out = {"graphs": {}}
    for n in (20, 26, 30):
        g = G.gnp_connected(n, 0.2, 900 + n)
        h.bottom_up(g)  # warm-up (allocation)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            td, par, order = h.bottom_up(g)
            ts.append(time.perf_counter() - t0)
        t = min(ts)
        alg = (2 ** n) * (33 * n / 2 + 34)
        out["graphs"][g.name] = {"n": n, "td": int(td), "ms": 1e3 * t, "alg_GBps": alg / t / 1e9,
                                 "frac_of_" + peak_kind + "_hbm": alg / t / 1e9 / peak}
        if cpu and n == 20:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            t0 = time.perf_counter()
            otd, opar, oorder = oracle.Port().bottom_up(g)
            cpu_s = time.perf_counter() - t0
            out["cpu_baseline"] = {"graph": g.name, "value_ms": 1e3 * cpu_s, "cores": 1, "kind": "port",
                                   "same_order_and_td": oorder == order.tolist() and otd == td,
                                   "gpu_over_cpu_speedup": cpu_s / t}
    out["note"] = "ms = whole gtd_bottom_up call (n launches + order + host replay); alg bytes per subset " \
                  "(|S| (32 + 1) read + 34 written) over that time"
    return out


def train_guidance(h, n_label):
    """The GNN trained on the GPU from exact DP labels (n <= 24 graphs of the
    config-2/3 families); returns (net, info)."""
    from gisbdw_gb300 import gnn
    base = gnn.training_graphs(n_label, seed=11)
    t0 = time.perf_counter()
    samples = gnn.label_set(h, base, per_graph=20, seed=1)
    t1 = time.perf_counter()
    train_set, test_set = samples.split(0.9)
    net = gnn.GNN(h, seed=1)
    losses = gnn.train(net, train_set, epochs=4, batch_graphs=256, lr=3e-3)
    t2 = time.perf_counter()
    info = {"labels": len(samples), "label_s": t1 - t0, "train_s": t2 - t1, "train_steps": len(losses),
            "held_out": gnn.root_accuracy(net, test_set), "layers": gnn.LAYERS, "hidden": gnn.HIDDEN,
            "weights": "bf16 (fp32 master, fp32 accumulation)"}
    return net, info


def bnb_arms(h, net, graphs, cap_s, memo_log2=0):
    """Plain and learned-guided B&B on the same graphs: (summary, raw results).
    Plain = ascending candidate order (the reference's DefaultAttemptOrder),
    the reference heuristic chain's incumbent, top-down levels; learned = the
    GNN's order, the better incumbent, its td estimate as the first level."""
    import numpy as np
    from gisbdw_gb300 import _lib, gnn
    from gisbdw_gb300.validate import check_tree
    cap_ns = int(cap_s * 1e9)
    h.bnb_solve_batch(graphs[:4], deadline_ns=10**8, memo_log2=memo_log2)  # warm-up (allocation, module load)
    tp = time.perf_counter()
    std, spar = h.heuristic_batch(graphs, 0)  # the reference heuristic chain's incumbents, counted in e2e
    packed = _lib.pack_bnb(graphs, seeds=list(zip(std.tolist(), spar)))
    t_seed = time.perf_counter() - tp
    plain = h.bnb_solve_batch(graphs, deadline_ns=cap_ns, memo_log2=memo_log2, packed=packed)
    t3 = time.perf_counter()
    gd = gnn.guidance(net, graphs)
    t_inf = time.perf_counter() - t3
    learned = h.bnb_solve_batch(graphs, orders=gd["orders"], seeds=gd["seeds"], hints=gd["hints"],
                                deadline_ns=cap_ns, memo_log2=memo_log2)
    cap_ms = cap_s * 1e3

    def summary(res, extra_s=0.0):
        ok = res["status"] == 0
        pm = res["proof_ms"]
        capped = np.where(ok, pm, cap_ms)
        fam = {}
        for f in ("rgg", "reg3", "grid", "tree"):
            sel = np.array([g.name.startswith(f) for g in graphs])
            if sel.any():
                fam[f] = f"{int((ok & sel).sum())}/{int(sel.sum())}"
        gaps = (res["td"] - res["lower_bound"])[~ok]
        return {"solved": int(ok.sum()), "solves_per_s": float(ok.sum() / (res["stats"]["ms"] / 1e3)),
                "e2e_solves_per_s": float(ok.sum() / (res["stats"]["total_ms"] / 1e3 + extra_s)),
                "p50_proof_ms_solved": float(np.median(pm[ok])) if ok.any() else None,
                "p50_proof_ms_capped": float(np.median(capped)),
                "p99_proof_ms_capped": float(np.percentile(capped, 99)),
                "unproven_gap_td_minus_lb": np.bincount(gaps).tolist() if gaps.size else [],
                "nodes": int(res["nodes"].sum()), "batch_ms": res["stats"]["ms"], "by_family": fam,
                "launches": 1, "passes": int(res["stats"].get("passes", 0)),
                "nodes_per_s": float(res["nodes"].sum() / (res["stats"]["ms"] / 1e3)),
                "p50_nodes_per_proven_graph": float(np.median(res["nodes"][ok])) if ok.any() else None,
                "trees_valid": all(check_tree(g, int(t), par) for g, t, par in
                                   zip(graphs, res["td"], res["parents"]))}
    ps, ls = summary(plain, t_seed), summary(learned, t_inf)
    solved = learned["status"] == 0
    ls["td_estimate_mae_on_proven"] = float(np.abs(gd["td_est"][solved] - learned["td"][solved]).mean()) \
        if solved.any() else None
    both = (plain["status"] == 0) & (learned["status"] == 0)
    out = {"graphs": len(graphs), "cap_s": cap_s, "plain": ps, "learned": ls, "both_solved": int(both.sum()),
           "td_identical_on_both": bool(np.array_equal(plain["td"][both], learned["td"][both])),
           "lower_bounds_consistent": bool(np.all(np.maximum(plain["lower_bound"], learned["lower_bound"]) <=
                                                  np.minimum(plain["td"], learned["td"]))),
           "p50_capped_plain_over_learned": ps["p50_proof_ms_capped"] / ls["p50_proof_ms_capped"],
           "inference_s": t_inf, "plain_seed_s": t_seed}
    if both.any():
        pp, lp = np.median(plain["proof_ms"][both]), np.median(learned["proof_ms"][both])
        out["p50_proof_ms_both"] = {"plain": float(pp), "learned": float(lp), "plain_over_learned": float(pp / lp)}
    return out, (plain, learned, gd)


def measure_bnb(h, n_graphs, cap_s, n_label, memo_log2=0, cpu_sample=0, cpu_nodes=0, family="c4",
                seeds=(4,), net=None, gnn_info=None):
    """Plain vs learned-guided B&B on the config 4 family (one run per graph
    sample seed, identical graphs in both arms) or the config 5 stream, the
    GNN trained here on DP labels."""
    import numpy as np
    from gisbdw_gb300 import graphs as G
    from gisbdw_gb300.validate import check_tree
    if net is None:
        net, gnn_info = train_guidance(h, n_label)
    runs = []
    first = None
    for seed in seeds:
        graphs = G.config4_graphs(count=n_graphs, seed=seed) if family == "c4" else \
            G.config5_graphs(count=n_graphs, seed=seed)
        summ, raw = bnb_arms(h, net, graphs, cap_s, memo_log2)
        summ["graph_seed"] = seed
        runs.append(summ)
        if first is None:
            first = (graphs, raw)
    out = dict(runs[0])
    out["gnn"] = gnn_info
    if len(runs) > 1:
        def spread_of(vals):
            vals = [v for v in vals if v is not None]
            return {"min": min(vals), "median": statistics.median(vals), "max": max(vals)} if vals else None

        def spread(key, arm=None):
            return spread_of([(r[arm][key] if arm else r.get(key)) for r in runs])
        out["runs"] = [{"graph_seed": r["graph_seed"], "plain_solved": r["plain"]["solved"],
                        "learned_solved": r["learned"]["solved"], "both_solved": r["both_solved"],
                        "p50_capped": [r["plain"]["p50_proof_ms_capped"], r["learned"]["p50_proof_ms_capped"]],
                        "p99_capped": [r["plain"]["p99_proof_ms_capped"], r["learned"]["p99_proof_ms_capped"]],
                        "p50_both_plain_over_learned": r.get("p50_proof_ms_both", {}).get("plain_over_learned"),
                        "td_identical_on_both": r["td_identical_on_both"]} for r in runs]
        out["spread"] = {"plain_solved": spread("solved", "plain"), "learned_solved": spread("solved", "learned"),
                         "p50_both_plain_over_learned": spread_of(
                             [x["p50_both_plain_over_learned"] for x in out["runs"]]),
                         "p50_capped_plain_over_learned": spread("p50_capped_plain_over_learned")}
    graphs, (plain, learned, gd) = first
    if family == "c5":
        # the same stream with the small graphs (n <= 28) given to the subset DP
        from gisbdw_gb300 import solve_exact
        cap_ns = int(cap_s * 1e9)
        hy = solve_exact(h, graphs, dp_max_n=28, deadline_ns=cap_ns, guidance=gd, memo_log2=memo_log2)
        ok = hy["status"] == 0
        by_dp = np.array([s == "dp" for s in hy["solver"]])
        agree = (learned["status"] == 0) & ok
        out["hybrid_learned"] = {
            "solved": int(ok.sum()), "by_dp": int(by_dp.sum()),
            "p50_proof_ms_capped": float(np.median(np.where(ok, hy["proof_ms"], cap_s * 1e3))),
            "td_identical_to_learned_bnb": bool(np.array_equal(hy["td"][agree], learned["td"][agree])),
            "trees_valid": all(check_tree(g, int(t), par) for g, t, par in zip(graphs, hy["td"], hy["parents"]))}
    if cpu_sample:
        threads = os.cpu_count() or 1
        sample = graphs[:cpu_sample]
        res, wall = time_cpu_bnb(sample, cpu_nodes, threads)
        solved = [r[0] == 0 for r in res]
        gpu_td = {i: int(learned["td"][i]) for i in range(len(sample)) if learned["status"][i] == 0}
        out["cpu_baseline"] = {
            "value": sum(solved) / wall, "unit": "solves/s", "cores": threads, "kind": "port",
            "solved": int(sum(solved)), "of": len(sample), "wall_s": wall, "node_limit": cpu_nodes,
            "nodes_per_s": sum(r[2] for r in res) / sum(r[3] for r in res),
            "gpu_learned_solved_in_sample": int((learned["status"][:len(sample)] == 0).sum()),
            "gpu_plain_solved_in_sample": int((plain["status"][:len(sample)] == 0).sum()),
            "td_agree": all(r[1] == gpu_td[i] for i, r in enumerate(res) if r[0] == 0 and i in gpu_td),
            "sample": f"first {len(sample)} config-{family[1]} graphs; oracle restatement of BranchAndBound "
                      f"(branch_and_bound.cpp:51-114, EdgeLowerBound, HighestDegree(Variance)), "
                      f"{cpu_nodes} nodes per graph, {threads} host threads ({cpu_model()})"}
    return out, net, gnn_info


def run_gpu(args, graphs):
    import numpy as np
    import torch

    from gisbdw_gb300 import Handle
    from gisbdw_gb300.validate import check_tree

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    all_graphs = graphs
    partitioned = world > 1 and args.partition
    if partitioned:
        if world > len(all_graphs):
            raise SystemExit(f"--partition needs at most {len(all_graphs)} ranks")
        graphs = [all_graphs[i] for i in partition_graphs(all_graphs, world)[rank]]
    # The library runs on this torch stream, so the CUDA events below bracket
    # its kernels on the stream they are launched on.
    stream = torch.cuda.Stream()
    h = Handle(local, stream=stream.cuda_stream)

    d_adj = [torch.from_numpy(g.adj64().view(np.int64)).cuda() for g in graphs]
    d_td = torch.zeros(len(graphs), dtype=torch.int32, device="cuda")
    d_par = torch.zeros((len(graphs), 64), dtype=torch.int32, device="cuda")

    def enqueue_step():
        for i, g in enumerate(graphs):
            h.dp_solve_device(d_adj[i].data_ptr(), g.n, d_td[i:].data_ptr(), d_par[i].data_ptr(),
                              tile_bits=args.tile_bits)

    def step():
        """One step solve by solve, each synchronised for its kernel times."""
        st = []
        for i, g in enumerate(graphs):
            h.dp_solve_device(d_adj[i].data_ptr(), g.n, d_td[i:].data_ptr(), d_par[i].data_ptr(),
                              tile_bits=args.tile_bits)
            st.append(h.sync())
        return st

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    # correctness of what the timed loop computes (tree valid, height = td)
    tds = d_td.cpu().tolist()
    pars = d_par.cpu().numpy()
    for i, g in enumerate(graphs):
        if not check_tree(g, tds[i], pars[i, :g.n]):
            raise SystemExit(f"invalid elimination tree for {g.name}")

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    # The timed steps are enqueued back to back on the library's stream (each
    # solve's kernels follow the previous solve's in stream order; errors are
    # collected once at the end), so host scheduling does not enter the
    # device time.
    ev0.record(stream)
    for _ in range(args.steps):
        enqueue_step()
    ev1.record(stream)
    torch.cuda.synchronize()
    h.sync()
    barrier()
    elapsed_ms = ev0.elapsed_time(ev1)
    clocks = sampler.stop()
    # per-launch kernel times for the roofline: the same steps, solve by solve
    kstats = []
    for _ in range(args.steps):
        kstats.extend(step())
    rate = job_rate_total if partitioned else job_rate
    value, elapsed_s = rate(len(graphs) * args.steps, elapsed_ms / 1000.0, world)
    elapsed_ms = elapsed_s * 1000.0

    # e2e: host buffers through the C ABI call (adjacency H2D, results D2H)
    h2d = sum(8 * g.n for g in graphs)
    d2h = len(graphs) * (136 * 4)
    adjs = [g.adj64() for g in graphs]
    for _ in range(max(1, args.warmup // 2)):
        for i, g in enumerate(graphs):
            h.dp_solve(adjs[i], g.n, tile_bits=args.tile_bits)
    barrier()
    gpu_out = {}
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for i, g in enumerate(graphs):
            gpu_out[g.name] = h.dp_solve(adjs[i], g.n, tile_bits=args.tile_bits)[:3]
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_value, _ = rate(len(graphs) * args.steps, e2e_s, world)

    # roofline of the dominant kernel (dp_tile_kernel), from live events
    alg = sum(s["alg_bytes"] for s in kstats)
    kms = sum(s["dp_ms"] for s in kstats)
    launches = len(kstats)
    peak, peak_kind = peaks()
    achieved = alg / (kms / 1000.0) / 1e9
    per_graph_ms = [s["dp_ms"] + s["tree_ms"] for s in kstats[-len(graphs):]]
    by_n = {}
    for g, s in zip(graphs * args.steps, kstats):
        by_n.setdefault(g.n, []).append(s)
    by_n_out = {str(n): {"dp_ms": statistics.median(x["dp_ms"] for x in v),
                         "alg_GBps": statistics.median(x["alg_bytes"] / (x["dp_ms"] / 1e3) / 1e9 for x in v)}
                for n, v in sorted(by_n.items())}
    # ncu's DRAM bytes per subset (n = 28 capture) scaled to each launch's 2^n
    bps = ncu_bytes_per_subset()
    traffic = (bps * statistics.mean(2.0 ** g.n for g in graphs)) if bps else None

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True, "scaling": "strong" if partitioned else "weak", "vs_baseline": None,
        "dtype": "u8", "data": "synthetic",
        "config": config_c2(all_graphs),
        "parallelism": (f"graphs partitioned over {world} ranks" if partitioned else
                        "replicas" if world > 1 else "1 GPU"),
        "p50_time_to_proof_ms": statistics.median(per_graph_ms),
        "treedepths": tds,
        "roofline": {"bound": "hbm", "kernel": "dp_tile_kernel", "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "traffic_note": "profiled constant, not measured in this run: ncu DRAM read+write bytes "
                                     "per subset of one n=28 launch (profiles/dp_tile_kernel.md), scaled by "
                                     "2^n and averaged over the workload's launches",
                     "frac_note": "achieved counts 1 + n/2 algorithmic bytes per subset (one written, one "
                                  "gathered per child); the tile layout serves the in-tile children from "
                                  "shared memory and most cross-tile children from L2, so DRAM moves about "
                                  "1.1 B per subset (traffic) and frac can exceed 1; the kernel is bound "
                                  "by instruction issue and the cross-tile L2 latency",
                     "issue_active_frac_profiled_n28": ncu_profile_figure("issue_active_frac"),
                     "alg_bytes_per_launch_mean": alg / launches,
                     "launch_ms_mean": kms / launches, "by_n": by_n_out},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": 3 * launches,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_c3:
        line["dp_c3"] = measure_dp_c3(h, args.steps, args.warmup, args.c3_graphs)
    if rank == 0 and not args.no_bottom_up:
        line["bottom_up"] = measure_bottom_up(h, 0 if args.no_cpu_baseline else 1)
    if rank == 0 and not args.no_bnb:
        line["bnb_c4"], net, gnn_info = measure_bnb(
            h, args.bnb_graphs, args.bnb_cap_s, args.label_graphs, args.bnb_memo_log2,
            0 if args.no_cpu_baseline else args.cpu_bnb_sample, args.cpu_bnb_nodes,
            seeds=tuple(args.c4_seeds))
        if not args.no_c5:
            line["bnb_c5"], _, _ = measure_bnb(h, args.c5_graphs, args.c5_cap_s, args.label_graphs,
                                               args.bnb_memo_log2, family="c5", seeds=(5,), net=net,
                                               gnn_info=gnn_info)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = cpu_sample_graphs(graphs)
        res = time_cpu_dp(sample, len(sample), threads)
        same = {}
        for g, _, (ctd, cpar, corder) in res:
            gtd, gpar, gorder = gpu_out[g.name]
            same[g.name] = {"td": ctd == gtd, "parent": cpar.tolist() == gpar.tolist(),
                            "order": corder == gorder.tolist()}
        line["cpu_baseline"] = {
            "value": workload_rate(graphs, [(g, t) for g, t, _ in res]), "unit": "solves/s", "cores": threads,
            "kind": "port",
            "sample": f"one graph per vertex count ({', '.join(g.name for g in sample)}), each solved once "
                      f"(table, tree, GetElimination order) by the oracle restatement of DynamicGPU's "
                      f"recurrence on {threads} host threads ({cpu_model()}); rate = the workload's "
                      f"{len(graphs)} graphs over the sum of their times, each graph taking the time of the "
                      f"sampled graph with its vertex count",
            "per_graph_s": {g.name: t for g, t, _ in res},
            "parity_bit_exact": all(all(v.values()) for v in same.values()),
            "parity": same}
    if rank == 0:
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_bnb_stream(args):
    """--workload bnb-c5: the config-5 mixed stream (1024 graphs, n in
    [20, 80], 60 s per-graph cap) solved in one persistent B&B launch per arm;
    the headline is the learned arm's proven solves/s."""
    import torch
    from gisbdw_gb300 import Handle
    rank, world, local = dist_env()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    h = Handle(local)
    sampler = ClockSampler(local)
    sampler.start()
    r, _, _ = measure_bnb(h, args.bnb_graphs, args.bnb_cap_s, args.label_graphs, args.bnb_memo_log2,
                          0 if args.no_cpu_baseline else args.cpu_bnb_sample, args.cpu_bnb_nodes, family="c5",
                          seeds=(5,))
    clocks = sampler.stop()
    L = r["learned"]
    line = {
        "metric": METRIC, "value": L["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": L["batch_ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int (bit masks)", "data": "synthetic",
        "config": {"workload": f"bnb-c5 (config 5: {r['graphs']} graphs, n in [20, 80], random geometric / "
                               f"3-regular / deleted grids / trees plus edges; {args.bnb_cap_s:g} s per-graph cap)",
                   "l2": "search state in shared memory, memo in HBM"},
        "p50_time_to_proof_ms": L["p50_proof_ms_capped"], "bnb": r, "roofline": None,
        "roofline_note": "integer-issue-bound search (profiles/bnb_kernel.md); no byte or FLOP roofline applies",
        "e2e": {"value": L["e2e_solves_per_s"], "unit": "solves/s", "h2d_bytes_per_step": None,
                "d2h_bytes_per_step": None},
        "gpu_launches": 4, "clocks": clocks,
    }
    if "cpu_baseline" in r:
        line["cpu_baseline"] = r["cpu_baseline"]
    print(json.dumps(line), flush=True)
    h.close()


def main():
    args = parse_args()
    from gisbdw_gb300 import graphs as G
    if args.workload == "bnb-c5":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the config-5 CPU B&B is reported inside the "
                              "gtd line's cpu_baseline"}), flush=True)
            return
        run_bnb_stream(args)
        return
    graphs = G.config2_graphs()
    if args.only_n:
        graphs = [g for g in graphs if g.n == args.only_n]
    if args.impl == "reference":
        run_reference(args, graphs)
    else:
        run_gpu(args, graphs)


if __name__ == "__main__":
    main()
