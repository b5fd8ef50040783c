"""Benchmark: DCFR iterations per second on the 48,255-node turn tree.

Workload (turn_c3, the ~52k-node turn spot): seeded 4-card board, 60% of combos
at weight U(0.5,1) and the rest U(0,0.2) (all 1128 combos per side), pot
100, stack 400, bets {25, 50, 100, 150}% + all-in on both streets, raises
2x, max 4 bets per street. A step is one DCFR iteration (both alternating
half-steps) over the whole tree; the data is synthetic (splitmix64, see
pps/workloads.py).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0). ``value`` is device-timed (CUDA events on the
solver's stream, tree resident in HBM); ``e2e`` is the same metric through
the C ABI from host buffers (compile + upload + K iterations + FP64 stats
readback); ``roofline`` covers the dominant kernel class from a launch-by-
launch CUDA-event profile pass, with every class's achieved bandwidth and
the whole iteration's algorithmic bandwidth beside it (the terminal groups
are bound on chip, so the iteration figure is the one to set against HBM);
``cpu_baseline`` times the CPU oracle
(restatement of the reference iteration) on this host's cores.
N > 1: replicas only (one spot per GPU, no collective in the data path);
``value`` sums the ranks' iterations over the max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "cuda-poker-solver_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "DCFR iters/s (52k-node turn)"
WORKLOAD = "turn_c3"


def workload_config(spot, n_nodes):
    return {"workload": "turn_c3: %d-node turn tree, 1000-iteration solve" % n_nodes,
            "board": spot.board_text(), "ranges": "all 1128 combos, 60% U(0.5,1) / 40% U(0,0.2)",
            "pot": spot.pot, "stack": spot.stack, "bets": "0.25,0.5,1,1.5,a", "raises": "2",
            "max_bets_per_street": 4, "iterations_e2e": 1000,
            "l2": "inputs larger than L2 (row working set > 129 MB); no flush needed",
            "parallelism": "replicas"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_traffic(kernel, algo_bytes_per_launch):
    """Per-launch DRAM bytes of the kernel class: the DRAM/algorithmic byte
    ratio of one ncu-captured launch (profiles/traffic.json) scaled to this
    run's average launch, or None without a capture of the class."""
    path = os.path.join(REPO, "profiles", "traffic.json")
    try:
        d = json.load(open(path)).get(kernel)
    except (OSError, ValueError):
        return None, None
    if not isinstance(d, dict) or "dram_over_algorithmic" not in d:
        return None, None
    return d["dram_over_algorithmic"] * algo_bytes_per_launch, d.get("source")


def cpu_baseline(spot, seconds=12.0):
    """The CPU oracle (f32, all host threads) on a bounded sample: one
    warm-up iteration, then iterations until ~`seconds` have passed."""
    from oracle.cpu_oracle import oracle_for
    threads = os.cpu_count() or 1
    o = oracle_for(spot, threads)
    o.iterate(1)
    t0 = time.perf_counter()
    n = 0
    while True:
        o.iterate(1)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 50:
            break
    return {"value": n / el, "unit": "iters/s", "cores": threads, "kind": "port",
            "sample": "%d DCFR iterations of turn_c3 (after 1 warm-up), CPU oracle f32 "
                      "restatement of the reference iteration, OpenMP over chance branches"
                      % n}


def accuracy(threads=None):
    """Each result's error against an FP64 run of the same iterations (the
    CPU oracle in double precision, as the checker): the product's root EV
    and exploitability (its FP64 walks) and root strategy (range-weighted
    frequencies of the root actions) after the spot's iterations, and its
    regret and strategy rows after one iteration (later rows are
    ill-conditioned: where exact regrets are zero, f32 rounding picks the
    strategy, so row errors of O(0.1) appear in any f32 arithmetic). Beside
    each, the same errors of a plain f32 restatement of the reference's
    arithmetic (the oracle in single precision). Sizes the oracle finishes
    in seconds: the river spot at its full 1,000 iterations, the 6,333-node
    per-street turn at 200 and the 48,255-node benchmark turn at 30."""
    import numpy as np
    import pps
    from pps import workloads as wl
    from oracle.cpu_oracle import oracle_for

    def root_freqs(rows, na, w):
        n = len(w)
        r = np.asarray(rows[:na * n], dtype=np.float64).reshape(na, n)
        tot = r.sum(axis=0)
        sig = np.where(tot > 0, r / np.where(tot > 0, tot, 1), 1.0 / na)
        return (sig * w[None, :]).sum(axis=1) / w.sum()

    def normwise(a, b):
        b = np.asarray(b, dtype=np.float64)
        return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - b))) / max(
            float(np.max(np.abs(b))), 1e-30)

    def make(spot):
        streets = None
        if spot.street_cfgs:
            streets = [{"bets": c.bet_text(), "raises": c.raise_text() or [],
                        "max_raises": c.max_raises} for c in spot.street_cfgs]
        return pps.Solver(board=spot.board_text(), oop=spot.oop, ip=spot.ip, pot=spot.pot,
                          stack=spot.stack, bets=spot.cfg.bet_text(),
                          raises=spot.cfg.raise_text() or [], max_raises=spot.cfg.max_raises,
                          streets=streets)

    out = {"reference": "CPU oracle in FP64, same tree, schedule and iteration count",
           "fields": "ev_err: |EV_oop - FP64| chips (FP64 walks); expl_ratio: exploitability / "
                     "FP64's; strategy_linf: root frequencies; rows_1_iteration: max |row - "
                     "FP64| / max |FP64| over regret and strategy rows after one iteration; "
                     "f32_restatement: the same errors of a plain f32 restatement of the "
                     "reference iteration; gpu_per_node_kernels: the product's per-node "
                     "kernels (engine 1), the same formulas in another f32 order. Where an "
                     "iteration count leaves the solve far from equilibrium (turn_c3 at 30, "
                     "exploitability ~5% of pot), f32 rounding flips regret-matching choices "
                     "at exactly-zero regrets, so every f32 order drifts from FP64 by O(0.1) "
                     "chips; the spread of the three f32 entries shows that noise"}
    for name, iters in (("river_c1", 1000), ("turn_c2", 200), ("turn_c3", 30)):
        spot = wl.NAMED[name]()
        s = make(spot)
        s.solve(1)
        # The per-node kernels (engine 1): the same formulas in another f32
        # evaluation order, for the spread between valid f32 orders.
        s1 = make(spot)
        s1.set_engine(1)
        s1.solve(1)
        o64 = oracle_for(spot, threads, precision=64)
        o32 = oracle_for(spot, threads, precision=32)
        o64.iterate(1)
        o32.iterate(1)
        rows1 = [max(normwise(x.read_rows(k) if x is not o32 else x.rows(k), o64.rows(k))
                     for k in (0, 1)) for x in (s, o32, s1)]
        s.solve(iters)
        st = s.stats()
        s1.solve(iters)
        st1 = s1.stats()
        o64.iterate(iters - 1)
        o32.iterate(iters - 1)
        e64, e32 = o64.stats(spot.pot), o32.stats(spot.pot)
        na = len(s.decide_nodes()[0]["actions"])
        w0 = np.asarray(s.player_weights(0), dtype=np.float64)
        f64 = root_freqs(o64.rows(1), na, w0)

        def errs(ev, expl, freqs, r1):
            return {"ev_err": abs(ev - e64["ev_oop"]),
                    "expl_ratio": expl / max(e64["exploitability"], 1e-12),
                    "strategy_linf": float(np.max(np.abs(np.asarray(freqs) - f64))),
                    "rows_1_iteration": r1}
        out[name] = {"iterations": iters, "nodes": s.num_nodes,
                     "fp64_ev_oop": e64["ev_oop"], "fp64_exploitability": e64["exploitability"],
                     "gpu": errs(st["ev_oop"], st["exploitability"], s.root_strategy(), rows1[0]),
                     "gpu_per_node_kernels": errs(st1["ev_oop"], st1["exploitability"],
                                                  s1.root_strategy(), rows1[2]),
                     "f32_restatement": errs(e32["ev_oop"], e32["exploitability"],
                                             root_freqs(o32.rows(1), na, w0), rows1[1])}
        del s, s1, o64, o32
    return out


def max_over_ranks(x, dist, device="cpu"):
    """The job's time is the slowest rank's (identity without a process
    group)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard(items, rank, world):
    """Batched spots per rank: independent units, no exchange between
    ranks (replicas of the batch engine, one per GPU)."""
    return list(items)[rank::world]


def _submit(batch, sp):
    from pps import pps_native as pn
    w = lambda r: pn.parse_range(r) if isinstance(r, str) else r
    return batch.submit(sp.board_text(), w(sp.oop), w(sp.ip), sp.pot, sp.stack,
                        bets=sp.cfg.bet_text(), raises=sp.cfg.raise_text() or [],
                        max_raises=sp.cfg.max_raises, target=0.005 * sp.pot)


def batched_bench(spots, loop_sample, check_every=64):
    """Batched: every spot solved to 0.5%-pot exploitability in one batch
    (all submitted at once, host compile threads, one device forest), next
    to the plain loop (pps.Solver per spot, solve with the same target,
    stats, destroy) over the same spots (all of them by default)."""
    import pps
    import numpy as np
    from pps import pps_native as pn
    b = pps.Batch(check_every=check_every, max_iterations=4096)
    t0 = time.perf_counter()
    tickets = [_submit(b, sp) for sp in spots]
    ok = b.run(timeout=600)
    el = time.perf_counter() - t0
    res = [b.result(t) for t in tickets]
    info = b.info()
    b.close()
    its = np.array([r["iterations"] for r in res])
    w = lambda r: pn.parse_range(r) if isinstance(r, str) else r
    t1 = time.perf_counter()
    for sp in loop_sample:
        s = pps.Solver(board=sp.board_text(), oop=w(sp.oop), ip=w(sp.ip), pot=sp.pot,
                       stack=sp.stack, bets=sp.cfg.bet_text(), raises=sp.cfg.raise_text() or [],
                       max_raises=sp.cfg.max_raises)
        s.solve(4096, "dcfr", 0.005 * sp.pot)
        s.stats()
        del s
    loop_s = time.perf_counter() - t1
    batched = len(spots) / el
    loop = len(loop_sample) / loop_s
    rivers = lambda ss: sum(1 for sp in ss if len(sp.board) == 5)
    same = len(loop_sample) == len(spots)
    sample = ("the same %d spots (%d river, %d turn)" % (len(spots), rivers(spots),
                                                         len(spots) - rivers(spots))
              if same else "first %d of the %d spots (%d river, %d turn)"
              % (len(loop_sample), len(spots), rivers(loop_sample),
                 len(loop_sample) - rivers(loop_sample)))
    return {"spots": len(spots), "finished": ok, "seconds": el, "solves_per_s": batched,
            "converged": int(sum(r["converged"] for r in res)),
            "failed": int(sum(r["status"] != 0 for r in res)),
            "iterations_mean": float(its.mean()), "iterations_max": int(its.max()),
            "target": "exploitability <= 0.5%% of pot; adaptive checks: the first after 32 "
                      "iterations, then where the measured decay predicts the target, every "
                      "16-%d iterations" % check_every,
            "max_expl_frac_pot": float(max(r["exploitability"] / sp.pot
                                           for r, sp in zip(res, spots))),
            "mix": "%d river, %d turn" % (rivers(spots), len(spots) - rivers(spots)),
            "one_at_a_time": {"solves_per_s": loop, "seconds": loop_s, "sample": sample,
                              "path": "pps.Solver + solve(target, checks every 128) + stats"},
            "speedup_vs_one_at_a_time": batched / loop,
            "device_bytes_peak": info["peak_used_bytes"],
            "time_split_ms": {k: info[k] for k in ("admit_ms", "iterate_ms", "check_ms",
                                                  "retire_ms", "idle_ms")}}


def served_bench(spots, lam, count, seed=7):
    """Served: Poisson arrivals at rate lam (a submitting thread sleeps
    to each arrival time) into a serving batch (its own driver thread);
    latency = finish - submit on the library clock."""
    import pps
    import numpy as np
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / lam, count))
    b = pps.Batch(check_every=32, max_iterations=4096)
    b.start()
    tickets = []
    t0 = time.perf_counter()
    for i in range(count):
        dt = arrivals[i] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append(_submit(b, spots[i % len(spots)]))
    res = [b.wait(t, timeout=600) for t in tickets]
    info = b.info()
    b.stop()
    b.close()
    done = [r for r in res if r is not None and r["status"] == 0]
    lat = np.array([r["latency_ms"] for r in done]) if done else np.array([float("nan")])
    first = min(r["submit_ms"] for r in done) if done else 0.0
    last = max(r["finish_ms"] for r in done) if done else 1.0
    rate = len(done) / max((last - first) / 1000.0, 1e-9)
    its = [r["iterations"] for r in done] or [0]
    return {"lambda_per_s": lam, "requests": count, "completed": len(done),
            "solves_per_s": rate,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "peak_active": info["peak_active"], "offered_seconds": float(arrivals[-1]),
            "iterations_mean": float(np.mean(its)),
            "converged": int(sum(r["converged"] for r in done)),
            "device_bytes_peak": info["peak_used_bytes"],
            "saturated": bool(rate < 0.9 * lam)}


def _workloads():
    """pps/workloads.py (the synthetic spot definitions; standard library
    only) loaded by its path, so that the reference arm never imports the
    product package or maps its library."""
    import importlib.util
    name = "spot_workloads"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(PKG, "pps", "workloads.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def _reference_weights(r):
    """1326 combo weights of a spot side: a list as given, or a range string
    as the reference's own parser read it (tests/golden/ranges.json, written
    by the reference's parseRange)."""
    import numpy as np
    if not isinstance(r, str):
        return np.asarray(r, dtype=np.float64)
    table = json.load(open(os.path.join(REPO, "tests", "golden", "ranges.json")))
    if table.get(r) is None:
        raise KeyError("no reference parse of range %r" % r)
    return np.asarray(table[r], dtype=np.float64)


def reference_kernels(steps, warmup):
    """The reference's own GPU kernels (cuda/gpu_cfr.cu compiled from its
    source for sm_103a, oracle/ref/ref_gpu.cpp's host runner: the
    reference's layout, graph and launch sequence) timed on this GPU with
    CUDA events over graph replays, per spot. Their input is the
    reference's layout as the oracle restates it (bit-exact against the
    reference's init()); no product code runs in this arm."""
    from oracle import ref_gpu
    from oracle import cpu_oracle as co
    if not ref_gpu.fatbin_present():
        return {"unavailable": "oracle/_ref/gpu_cfr_kernels.fatbin not built (the reference "
                               "sources are needed to build it)"}
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
    except ImportError:
        return {"unavailable": "no torch"}
    wl = _workloads()
    out = {"unit": "iters/s", "kind": "reference kernels on this GPU",
           "method": "CUDA events over graph replays after warm-up",
           "input": "the reference's layout restated by the oracle (bit-exact against the "
                    "reference's init()); no product code in this arm"}
    for name in ("turn_c3", "turn_w52", "flop_164k"):
        spot = wl.NAMED[name]()
        exp = co.reference_layout(spot.board, _reference_weights(spot.oop),
                                  _reference_weights(spot.ip), spot.pot, spot.stack,
                                  co.cfg_from(spot.cfg))
        r = ref_gpu.RefKernels(exp, spot.pot)
        n = max(1, min(steps, 300))
        ms = r.ms_per_iteration(max(3, warmup), n)
        r.close()
        out[name] = {"value": 1000.0 / ms, "iterations": n,
                     "nodes": int(exp["numNodes"][0])}
    return out


def run_reference(args, rank):
    """--impl reference: the CPU restatement of the reference iteration on
    the host cores (the reference has no CPU implementation of this path:
    its CPU river solver was removed). Beside it, ``gpu_kernels`` times the
    reference's own GPU kernels on the same GPU."""
    if rank != 0:
        return
    wl = _workloads()
    from oracle.cpu_oracle import oracle_for
    spot = wl.turn_c3()
    threads = os.cpu_count() or 1
    o = oracle_for(spot, threads)
    for _ in range(max(1, min(args.warmup, 2))):
        o.iterate(1)
    steps = max(1, args.steps)
    budget = 60.0
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        o.iterate(1)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    v = done / el
    line = {"metric": METRIC, "value": v, "unit": "iters/s", "n_gpus": args.gpus,
            "steps": done, "warmup": args.warmup, "ms_per_step": 1000.0 * el / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(spot, o.num_nodes),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "iters/s", "cores": threads, "kind": "port",
                             "sample": "%d of %d requested steps within %.0f s (bounded); "
                                       "CPU oracle restatement of cuda/gpu_cfr.cu's iteration"
                                       % (done, steps, budget)},
            "e2e": {"value": v, "unit": "iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    del o
    try:
        line["gpu_kernels"] = reference_kernels(args.steps, args.warmup)
    except Exception as e:  # reported, not fatal: the CPU line above stands
        line["gpu_kernels"] = {"unavailable": "%s: %s" % (type(e).__name__, e)}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-iters", type=int, default=1000,
                    help="iterations of the end-to-end solve (the workload's 1000)")
    ap.add_argument("--batch-spots", type=int, default=256,
                    help="spots of the batched solve (0 skips batched and served)")
    ap.add_argument("--loop-sample", type=int, default=0,
                    help="spots of the one-at-a-time loop the batched solve is set against "
                         "(0: the same spots as the batch)")
    ap.add_argument("--served-requests", type=int, default=100,
                    help="requests per arrival rate of the served run (0 skips it)")
    ap.add_argument("--served-rates", default="4,50,200",
                    help="Poisson arrival rates (requests/s) of the served run: one "
                         "below the ~8 solves/s a GB300 sustains on this distribution, "
                         "two above it")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")
    if args.impl == "reference":
        run_reference(args, rank)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch
    torch.cuda.set_device(local)
    import pps
    from pps import workloads as wl

    spot = wl.turn_c3()

    def make():
        return pps.Solver(board=spot.board_text(), oop=spot.oop, ip=spot.ip, pot=spot.pot,
                          stack=spot.stack, bets=spot.cfg.bet_text(), raises=spot.cfg.raise_text(),
                          max_raises=spot.cfg.max_raises)

    # The autotuner picks the launch shape once per tree-size class and
    # caches it (tune.h); a first solver of the class does that here, so the
    # timed end-to-end solve below takes the cached shape, as every later
    # solve of the class does.
    warm = make()
    warm.solve(64)
    shape = warm.launch_shape()
    del warm
    # e2e through the public API from host buffers: compile + upload, the
    # configured 1000 iterations, FP64 stats back to the host.
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = make()
    s.solve(args.e2e_iters)
    st = s.stats()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    info = s.info()
    e2e = {"value": args.e2e_iters / e2e_s, "unit": "iters/s",
           "h2d_bytes_per_step": int(info.h2d_bytes) // args.e2e_iters,
           "d2h_bytes_per_step": int(info.d2h_bytes) // args.e2e_iters,
           "includes": "compile + upload + %d iterations + FP64 stats walks; launch shape "
                       "from the autotuner's per-class cache (tuned once before)" % args.e2e_iters,
           "stats": {"ev_oop": st["ev_oop"], "ev_ip": st["ev_ip"],
                     "exploitability": st["exploitability"]}}

    # Device-timed region: K graph replays, CUDA events on the solver stream.
    s.time_iterations(args.warmup)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = s.time_iterations(args.steps)
    torch.cuda.synchronize()
    if dist:
        ms = max_over_ranks(ms, dist, "cuda")
        dist.barrier()
    value = world * args.steps / (ms / 1000.0)

    # Dominant kernel class: launch-by-launch CUDA-event profile.
    prof = s.profile(min(args.steps, 20))
    name, (launches, pms, pbytes) = max(prof.items(), key=lambda kv: kv[1][1])
    peak, peak_kind = measured_peaks()
    achieved = (pbytes / launches) / (pms / launches / 1000.0) / 1e9
    traffic, traffic_src = committed_traffic(name, pbytes / launches)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                "kernel": name,
                "algo_bytes_per_launch": pbytes / launches,
                "avg_launch_us": 1000.0 * pms / launches, "peak_source": peak_kind,
                "iteration_gbs": (sum(v[2] for v in prof.values()) / min(args.steps, 20)) *
                                 (value / world) / 1e9,
                "profile": {k: {"launches": v[0], "ms": v[1], "algo_bytes": v[2],
                                "achieved_gbs": (v[2] / v[0]) / (v[1] / v[0] / 1000.0) / 1e9
                                if v[0] and v[1] > 0 else None,
                                "frac": (v[2] / v[1] * 1000.0 / 1e9) / peak if v[1] > 0 else None}
                            for k, v in prof.items()},
                "iteration_frac": None}
    roofline["iteration_frac"] = roofline["iteration_gbs"] / peak
    # The terminal classes (showdown, fold groups) are bound on chip - the
    # showdown groups by the shared-memory pipe - and move few bytes for
    # their time; the decide levels are the HBM-bound classes.
    onchip = {"bwd_showdown": "shared-memory pipe", "bwd_fold": "load latency"}
    hbm = {k: v["frac"] for k, v in roofline["profile"].items()
           if k in ("bwd_interior", "fwd_level") and v["frac"] is not None}
    roofline["note"] = (
        "dominant class %s%s; HBM-bound classes: %s; whole iteration %.3f of peak"
        % (name, " (bound on chip: %s, see profiles/turn_c3_top_kernels_ncu.md)" % onchip[name]
           if name in onchip else "",
           ", ".join("%s %.3f" % kv for kv in sorted(hbm.items())), roofline["iteration_frac"]))
    batched = None
    if args.batch_spots > 0:
        spots = wl.batched(args.batch_spots)
        mine = shard(spots, rank, world)
        if dist:
            dist.barrier()
        loop = mine if args.loop_sample <= 0 else mine[:max(1, min(args.loop_sample, len(mine)))]
        batched = batched_bench(mine, loop)
        if dist:
            slowest = max_over_ranks(batched["seconds"], dist, "cuda")
            batched.update({"spots": len(spots), "ranks": world, "seconds": slowest,
                            "solves_per_s": len(spots) / slowest,
                            "speedup_vs_one_at_a_time": len(spots) / slowest /
                            (world * batched["one_at_a_time"]["solves_per_s"])})
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {"metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(spot, info.num_nodes),
            "e2e": e2e, "roofline": roofline, "clocks": clk.summary(),
            "gpu_launches": int(info.launches_per_iteration) * args.steps,
            "launch_shape": shape,
            "engine": {0: "staged: terminal groups on side streams + decide records",
                       1: "per-node terminals", 2: "fused backward levels"}.get(info.engine,
                                                                               "?")}
    # The timed value uses the reference's plain f32 cumulative-strategy
    # sums; the compensated (two-float) form is timed beside it.
    sc = make()
    sc.set_compensated(True)
    sc.time_iterations(args.warmup)
    n_comp = max(min(args.steps, 1000), 100)
    line["strategy_sums"] = {"timed": "plain f32 (the reference's update)",
                             "compensated": {"value": n_comp / (sc.time_iterations(n_comp) / 1000.0),
                                             "unit": "iters/s", "iterations": n_comp}}
    del sc
    # The reference's own published spot (tools/quality/bench_turn.sh:40-41,
    # 51,903 nodes; ~747-807 it/s on an RTX 4070, docs/STATUS.md:69).
    w52 = wl.turn_w52()
    sw = pps.Solver(board=w52.board_text(), oop=w52.oop, ip=w52.ip, pot=w52.pot, stack=w52.stack,
                    bets=w52.cfg.bet_text(), raises=w52.cfg.raise_text(),
                    max_raises=w52.cfg.max_raises)
    sw.time_iterations(args.warmup)
    w52_ms = sw.time_iterations(max(args.steps, 100))
    line["w52"] = {"value": max(args.steps, 100) / (w52_ms / 1000.0), "unit": "iters/s",
                   "nodes": sw.num_nodes, "published_rtx4070": "747-807 iters/s"}
    del sw
    # The reference's flop bench spots (docs/STATUS.md:75-84).
    line["flop"] = {}
    for fname, pub, iters in (("flop_164k", "~201 iters/s", 100), ("flop_615k", "~55 iters/s", 100),
                              ("flop_wide", "~0.57 iters/s", 10)):
        fs = wl.NAMED[fname]()
        t0 = time.perf_counter()
        sf = pps.Solver(board=fs.board_text(), oop=fs.oop, ip=fs.ip, pot=fs.pot, stack=fs.stack,
                        bets=fs.cfg.bet_text(), raises=fs.cfg.raise_text(),
                        max_raises=fs.cfg.max_raises)
        compile_s = time.perf_counter() - t0
        sf.time_iterations(min(args.warmup, 3))
        fms = sf.time_iterations(iters)
        line["flop"][fname] = {"value": iters / (fms / 1000.0), "unit": "iters/s",
                               "nodes": sf.num_nodes, "compile_upload_s": compile_s,
                               "published_rtx4070": pub}
        del sf
    if batched is not None:
        line["batched"] = batched
    if world == 1 and args.batch_spots > 0 and args.served_requests > 0:
        stream = wl.c3_stream(args.served_requests)
        rates = [served_bench(stream, float(lam), args.served_requests)
                 for lam in args.served_rates.split(",")]
        line["served"] = {"distribution": "turn_c3 distribution: %d distinct 48,255-node turn "
                                          "spots (seeded boards and mixture ranges, pot 100, "
                                          "stack 400); target 0.5%% pot" % len(stream),
                          "requests_per_rate": args.served_requests,
                          "rates": rates}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(spot)
        line["accuracy"] = accuracy()
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
