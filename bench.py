"""Benchmark of the GB300 PRIME20 DMD event engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c3|c2|c1|c4] [--events E]

Workload (default c3): 32 independent replicas (seeded 8-96 chains of
random 16-residue sequences at 5 mM, T* evenly spaced over 0.18-0.50),
advanced together by one persistent launch.  A step commits E events in
every replica (the reference's collision count).  ``value`` is committed
events/s of the whole job with the state resident in HBM, timed with CUDA
events on the launching stream; ``e2e`` is the same metric through the
public C ABI with host buffers (create from host arrays, run, read the
state back).  The plain one-system-per-launch path on the same replicas
and the CPU restatement on the host cores are reported beside it.

``--impl reference`` times the CPU restatement of the reference engine (the
reference itself is Fortran + MPI and cannot be built here) on all host
cores for the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "parallel-dmd-for-biomolecules_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "DMD events/s on 1 GB300: batched vs plain GPU vs host CPU; p50/p99 latency"
UNIT = "events/s"


# --------------------------------------------------------------- workloads
def make_workload(name: str, rank: int = 0, gen=None):
    """The named workload, generated by gen (systems.generate by default;
    the CPU arm passes the oracle library's copy of the generator so that it
    loads nothing of the engine)."""
    from dmdgb import sharding, systems

    gen = gen or systems.generate

    if name == "c3":
        specs = systems.config_c3(32, seed=sharding.replica_seed(rank))
        desc = "C3: 32 replicas, 8-96 chains x 16-mer random sequences, 5 mM, T* 0.18-0.50"
    elif name == "c2":
        specs = [systems.config_c2(seed=1 + rank)]
        desc = "C2: 48 x KLVFFAE (1,344 beads), 5 mM, T* 0.18"
    elif name == "c1":
        specs = [systems.config_c1(seed=1 + rank)]
        desc = "C1: 8 x KLVFFAE (224 beads), 5 mM, T* 0.20"
    elif name == "c4":
        specs = [systems.config_c4(seed=1 + rank)]
        desc = "C4: 1000 x random 10-mer (~40,000 beads), 10 mM, T* 0.22"
    else:
        raise SystemExit(f"unknown workload {name}")
    for s in specs:
        gen(s)
    return specs, desc


def algorithmic_bytes_per_event(nbr_mean: float) -> float:
    """Minimal unique bytes one committed pair event touches: i and j
    read+written (2 x 96), their per-bead constants (2 x 33), and for every
    neighbour of i and j its position/velocity, identity, pair type, list
    index and prediction read+write (86 bytes)."""
    return 289.0 + 86.0 * 2.0 * nbr_mean


def rebuild_bytes(n: int, nbr_mean: float) -> float:
    return n * (24 + 4) + n * nbr_mean * (4 + 54)


def fp64_flops_per_event(nbr_mean: float) -> float:
    """Double-precision operations of one committed pair event: the
    re-predictions of both beads against their neighbours (2 * nbr_mean
    pairs) and of the two beads themselves, about 27 operations each
    (relative position and velocity, minimum image, three dot products, the
    discriminant, one square root and one division counted as one each),
    plus about 40 for the collision impulse."""
    return 27.0 * (2.0 * nbr_mean + 2.0) + 40.0


FP64_PEAK_GFLOPS = 1250.0   # GB300 nominal dense FP64 (no measured figure in the peaks file)


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


# ------------------------------------------------------------ clock sampler
class ClockSampler:
    def __init__(self, index: int = 0):
        self.samples = []
        self.index = index
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self):
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 3 + k and s[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ------------------------------------------------------------ CPU baseline
def _cpu_worker(args):
    """One host process: its share of the replicas, one after another."""
    part, n_events = args
    sys.path.insert(0, REPO)
    sys.path.insert(0, PKG)
    from oracle.oracle import Oracle

    busy = 0.0
    for spec in part:
        o = Oracle(spec)
        t0 = time.perf_counter()
        o.run(n_events)
        busy += time.perf_counter() - t0
    return n_events * len(part), busy


def cpu_rate(specs, events_per_replica: int, cores: int):
    """Aggregate events/s of the CPU restatement: every replica advanced by
    events_per_replica, the replicas dealt round-robin to `cores` processes;
    the rate is all events over the busiest process's time."""
    parts = [specs[k::cores] for k in range(min(cores, len(specs)))]
    work = [(p, events_per_replica) for p in parts if p]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(len(work)) as pool:
        res = pool.map(_cpu_worker, work)
    wall = time.perf_counter() - t0
    total = sum(r[0] for r in res)
    slowest = max(r[1] for r in res)
    return total / slowest, total, wall


def _single_core_worker(args):
    """One host process: the CPU restatement on one system, events/s over
    n_events after creation (its start-up overlap check skipped: it is not
    part of the event loop)."""
    name, n_events = args
    sys.path.insert(0, REPO)
    sys.path.insert(0, PKG)
    from oracle import oracle as ora
    from dmdgb import abi, systems

    spec = {"c1": systems.config_c1, "c2": systems.config_c2, "c4": systems.config_c4}[name]()
    ora.generate(spec)
    o = ora.Oracle(spec, flags=abi.FLAG_ALLOW_OVERLAP)
    t0 = time.perf_counter()
    o.run(n_events)
    dt = time.perf_counter() - t0
    return name, spec.n_beads, n_events, n_events / dt, dt


def cpu_single_core(samples=(("c1", 300000), ("c2", 300000), ("c4", 100000))) -> dict:
    """The CPU restatement on one core for the single-system workloads
    (each in its own process, run one after another)."""
    ctx = mp.get_context("spawn")
    out = {"cores": 1, "kind": "port", "cpu_model": cpu_model()}
    with ctx.Pool(1) as pool:
        for name, n_beads, n_ev, rate, dt in pool.map(_single_core_worker, list(samples)):
            out[name] = {"events_per_s": rate, "beads": n_beads, "sample": f"{n_ev} events after creation, {dt:.2f} s"}
    return out


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_event():
    """DRAM bytes per committed event of the persistent kernel, from the
    committed ncu capture summary (profiles/), or None."""
    p = os.path.join(REPO, "profiles", "k_run_traffic.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["dram_bytes"]) / float(d["events"])
    except Exception:
        return None


# ----------------------------------------------------------------- arms
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as ora

    specs, desc = make_workload(args.workload, gen=ora.generate)
    cores = max(1, min(os.cpu_count() or 1, 64))
    n_ev = args.events
    for _ in range(args.warmup):
        cpu_rate(specs, max(1000, n_ev // 10), cores)
    rates, times = [], []
    total_ev = 0
    for _ in range(args.steps):
        r, tot, wall = cpu_rate(specs, n_ev, cores)
        rates.append(r)
        times.append(tot / r)
        total_ev += tot
    value = total_ev / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "events_per_replica_per_step": n_ev},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "cpu_model": cpu_model(),
                         "sample": f"all {len(specs)} replicas, {n_ev} events each, dealt to {cores} processes"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(args):
    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    import __graft_entry__ as g

    g.build()
    from dmdgb import abi
    from dmdgb.engine import Batch, Engine

    specs, desc = make_workload(args.workload, rank)
    E = args.events
    batch = Batch(specs)
    lib = batch.lib
    tuned = batch.autotune(min(25000, max(2000, E // 4)), cache=args.tune_cache) if not args.no_tune else None
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        batch.run(E)
        flush.fill_(1.0)
    barrier()
    d0 = [batch.diagnostics(r) for r in range(len(specs))]
    ms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(2.0)          # evict the state from L2 between steps
            torch.cuda.synchronize()
            batch.run(E)
            ms.append(lib.dmd_batch_last_run_ms(batch.h))
    barrier()
    d1 = [batch.diagnostics(r) for r in range(len(specs))]
    step_s = sum(ms) / 1000.0
    events = E * len(specs) * args.steps
    from dmdgb import sharding
    step_s = sharding.max_over_ranks(step_s, device="cuda")   # the slowest rank's time
    value = events * world / step_s
    pair_events = sum(b["n_pair"] - a["n_pair"] for a, b in zip(d0, d1))
    nbr = float(np.mean([d["nbr_mean"] for d in d1]))
    rebuilds = sum(b["n_updates"] - a["n_updates"] for a, b in zip(d0, d1))
    nbeads = int(np.mean([s.n_beads for s in specs]))
    alg_bytes = pair_events * algorithmic_bytes_per_event(nbr) + rebuilds * rebuild_bytes(nbeads, nbr)
    per_launch_bytes = alg_bytes / args.steps
    launch_s = step_s / args.steps
    hbm, peak_kind = peaks()
    achieved = per_launch_bytes / launch_s / 1e9
    tpe = traffic_per_event()
    traffic = tpe * E * len(specs) if tpe else None
    fp64_gflops = pair_events * fp64_flops_per_event(nbr) / step_s / 1e9

    # the rate over a longer stretch: ten more segments of the same batch,
    # each segment's committed events/s (the lists and aggregates grow)
    segments = []
    if rank == 0 and args.segments > 0:
        for _ in range(args.segments):
            batch.run(args.segment_events)
            segments.append(args.segment_events * len(specs) / (lib.dmd_batch_last_run_ms(batch.h) / 1000.0))

    # rebuild cycles replayed from a captured CUDA graph: every launch ends
    # each replica at its next list rebuild (the host regains control every
    # launches_per_graph cycles); the same events as the persistent launch
    cycles = None
    if rank == 0 and not args.no_cycles:
        per_graph = 8
        batch.run_cycles(max(1000, E // 4), per_graph)      # capture and warm-up
        flush.fill_(3.0)
        torch.cuda.synchronize()
        k = batch.run_cycles(E, per_graph)
        cyc_s = lib.dmd_batch_last_run_ms(batch.h) / 1000.0
        cycles = {"value": E * len(specs) / cyc_s, "unit": UNIT, "events_per_replica": E, "launches": k,
                  "launches_per_graph": per_graph,
                  "note": "same batch continued; each launch runs every replica to its next neighbour-list rebuild"}

    # the plain one-system-per-launch path on the same replicas
    plain_events, plain_s = 0, 0.0
    n_plain = min(len(specs), args.plain_replicas)
    Ep = min(E, args.plain_events)
    for s in specs[:n_plain]:
        with Engine(s) as eng:
            eng.run(Ep)          # warm-up of this system
            eng.run(Ep)
            plain_s += eng.lib.dmd_last_run_ms(eng.h) / 1000.0
            plain_events += Ep
    plain_value = plain_events / plain_s if plain_s > 0 else None

    # end to end through the public API with host buffers
    e2e_times, h2d, d2h = [], 0, 0
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b2 = Batch(specs)
        h2d = int(b2.lib.dmd_batch_upload_bytes(b2.h))   # the pools' heads from the pinned host image
        d2h = int(b2.lib.dmd_batch_readback_bytes(b2.h))  # one state block per replica
        b2.run(E)
        states = [b2.state(r) for r in range(len(specs))]
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
        b2.close()
        del states
    e2e_value = E * len(specs) * world / statistics.median(e2e_times)

    serving = None
    if rank == 0 and not args.no_serve:
        serving = run_serving(args)
        # the stated serving load (1e6-1e7 events per request) over a bounded window
        serving["c5_full"] = run_serving_full(args)
    single = None
    if rank == 0 and not args.no_single:
        single = run_single_systems(min(E, args.single_events))

    sidechain = None
    if rank == 0 and not args.no_sidechain:
        sidechain = run_sidechain(with_cpu=not args.no_cpu)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = max(1, min(os.cpu_count() or 1, 64))
        r, tot, wall = cpu_rate(specs, E, cores)
        cpu = {"value": r, "unit": UNIT, "cores": cores, "kind": "port", "cpu_model": cpu_model(),
               "sample": f"CPU restatement: all {len(specs)} replicas, {E} events each, dealt to {cores} processes, {wall:.1f} s wall",
               "single_core": cpu_single_core()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * step_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "replicas": len(specs), "events_per_replica_per_step": E,
                       "beads_total": int(sum(s.n_beads for s in specs)), "l2": "flushed (256 MB write) between steps",
                       "parallelism": f"replicas: one cluster of {batch.cluster} CTA(s) per system, {world} GPU(s)",
                       "autotuned": tuned},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "plain_gpu": {"value": plain_value, "unit": UNIT, "replicas_timed": n_plain,
                          "note": "same replicas, one system per launch, one after another"},
            "gpu_launches": args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": traffic, "peak_kind": f"{peak_kind} hbm_gbs",
                         "bytes_per_event": algorithmic_bytes_per_event(nbr), "nbr_mean": nbr,
                         "fp64": {"achieved": fp64_gflops, "peak": FP64_PEAK_GFLOPS, "unit": "GFLOP/s",
                                  "frac": fp64_gflops / FP64_PEAK_GFLOPS, "peak_kind": "nominal",
                                  "flops_per_event": fp64_flops_per_event(nbr)}},
            "rebuild_cycle_graph": cycles,
            "segments": {"events_per_replica": args.segment_events, "events_per_s": segments,
                         "note": "the batch continued after the timed steps, one launch per segment"},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "serving": serving,
            "single_system": single,
            "sidechain_search": sidechain,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_single_systems(E: int) -> dict:
    """The single-system workloads on the plain path (one system per launch,
    autotuned cluster): 8 x KLVFFAE (224 beads), 48 x KLVFFAE (1,344 beads)
    and 1,000 random 10-mers (40,000 beads), committed events/s over E events
    after a warm-up."""
    from dmdgb import systems

    out = {}
    for name, spec in (("c1_224_beads", systems.config_c1()), ("c2_1344_beads", systems.config_c2()),
                       ("c4_40000_beads", systems.config_c4())):
        systems.generate(spec)
        from dmdgb.engine import Batch
        b = Batch([spec])
        t = b.autotune(max(2000, E // 4))
        b.run(E)
        b.run(E)
        ms = b.lib.dmd_batch_last_run_ms(b.h)
        out[name] = {"events_per_s": E / ms * 1e3, "cluster": t["cluster"], "cell_div": t["cell_div"]}
        b.close()
    return out


def run_sidechain(with_cpu: bool) -> dict:
    """The initial-configuration generator's side-chain placement search on
    its own 22-residue template (the committed fixture of its inputs and
    results): 22 x 1,401^3 grid points on the GPU, host-timed through the
    public call (tables, copies, search, read-back) after a warm-up, checked
    against the fixture's winners; with with_cpu, the CPU restatement's rate
    on a bounded sample (one residue, 200^3 points)."""
    import json
    import numpy as np
    from dmdgb import systems
    from dmdgb.params import default_tables

    with open(os.path.join(REPO, "tests", "golden", "sidechain_template.json")) as fh:
        d = json.load(fh)
    t = default_tables()
    t.rca, t.rnh, t.rco, t.sqz = (np.array(d[k]) for k in ("rca", "rnh", "rco", "sqz"))
    args = [np.array(d[k]) for k in ("ca", "nh", "co", "side_start")]
    res = d["residues"]
    systems.sidechain_search(*args, res, d["move"], d["step"], tables=t)   # warm-up
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        out, rmin, idx = systems.sidechain_search(*args, res, d["move"], d["step"], tables=t)
        times.append(time.perf_counter() - t0)
    m = int(systems.abi.load_engine().dmd_sidechain_grid(d["move"], d["step"]))
    points = len(res) * m ** 3
    sec = statistics.median(times)
    out_d = {"workload": f"genconfig template, {len(res)} residues x {m}^3 grid points", "ms": sec * 1e3,
             "points_per_s": points / sec, "matches_reference_fixture": bool(np.array_equal(idx, d["oracle_index"]))}
    if with_cpu:
        from oracle import oracle as ora
        t0 = time.perf_counter()
        ora.sidechain_search(*args, res, 0.5, d["step"], tables=t, only=(1, 2))
        cs = time.perf_counter() - t0
        cm = len(ora.sidechain_grid(0.5, d["step"]))
        out_d["cpu_points_per_s"] = cm ** 3 / cs
        out_d["cpu_sample"] = f"CPU restatement, 1 core: one residue, {cm}^3 points, {cs:.2f} s"
        out_d["cpu_s_for_workload"] = points / out_d["cpu_points_per_s"]
    return out_d


def run_serving(args, scale: float = None) -> dict:
    """The serving workload: Poisson arrivals at 20 requests/s of systems of
    4-200 chains x 6-40 residues, 2-10 mM, T* 0.15-0.30, replayed for
    --serve-seconds with each request's 1e6-1e7 events scaled by
    --serve-scale so that the run stays within the bench's time."""
    from dmdgb import systems
    import numpy as np
    from dmdgb.serving import Server, poisson_arrivals, serve_trace

    arr = poisson_arrivals(20.0, args.serve_seconds, seed=1)
    reqs = []
    for k in range(len(arr)):
        spec = systems.generate(systems.serving_request(k, seed=1))
        reqs.append((spec, max(1000, int(spec.n_events * (scale if scale is not None else args.serve_scale)))))
    with Server(max_slots=args.serve_slots, chunk_events=args.serve_chunk) as srv:
        res = serve_trace(srv, arr, reqs)
    out = res.summary()
    out.update({"arrival_rate_per_s": 20.0, "trace_seconds": args.serve_seconds,
                "events_scale": scale if scale is not None else args.serve_scale,
                "slots": args.serve_slots, "chunk_events": args.serve_chunk,
                "beads_per_request_mean": float(np.mean([s.n_beads for s, _ in reqs])) if reqs else 0.0,
                "note": "latency = completion - arrival on the host clock; events/s over the trace's wall time"})
    return out


def run_serving_full(args) -> dict:
    """The serving workload at its stated size: Poisson arrivals at 20
    requests/s of 4-200 chains x 6-40 residues with 1e6-1e7 events each,
    over a bounded arrival window and a wall-clock horizon.  The offered
    load (about 1.1e8 events/s) is above what one GPU serves, so the report
    is the backlog: requests and events offered, served and left at the
    horizon, how fast the backlog grows, p50/p99 of the requests completed,
    and lower bounds of p50/p99 over all arrived requests (an unfinished
    request counts with its age at the horizon)."""
    from dmdgb import systems
    import numpy as np
    from dmdgb.serving import Server, poisson_arrivals, serve_trace

    arr = poisson_arrivals(20.0, args.full_serve_seconds, seed=1)
    reqs = []
    for k in range(len(arr)):
        spec = systems.generate(systems.serving_request(k, seed=1))
        reqs.append((spec, int(spec.n_events)))
    with Server(max_slots=args.serve_slots, chunk_events=args.serve_chunk) as srv:
        res = serve_trace(srv, arr, reqs, horizon_s=args.full_serve_horizon)
    out = res.summary()
    offered = int(sum(n for _, n in reqs))
    out.update({"arrival_rate_per_s": 20.0, "trace_seconds": args.full_serve_seconds,
                "horizon_s": args.full_serve_horizon, "events_scale": 1.0,
                "requests_arrived": len(arr), "events_offered": offered,
                "offered_events_per_s": offered / args.full_serve_seconds,
                "note": "stated request sizes (1e6-1e7 events); stopped at the horizon with a backlog"})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3")
    ap.add_argument("--events", type=int, default=300000,
                    help="events per replica per step (both arms, and the CPU baseline's sample); "
                         "the workload asks 10^7 per replica")
    ap.add_argument("--plain-replicas", type=int, default=32)
    ap.add_argument("--plain-events", type=int, default=20000, help="events per system on the plain path")
    ap.add_argument("--single-events", type=int, default=100000, help="events of the single-system runs")
    ap.add_argument("--segments", type=int, default=10)
    ap.add_argument("--segment-events", type=int, default=100000)
    ap.add_argument("--full-serve-seconds", type=float, default=15.0,
                    help="arrival window of the full-size serving trace")
    ap.add_argument("--full-serve-horizon", type=float, default=45.0,
                    help="wall-clock bound of the full-size serving trace")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--no-single", action="store_true")
    ap.add_argument("--no-sidechain", action="store_true")
    ap.add_argument("--no-cycles", action="store_true")
    ap.add_argument("--tune-cache", default=None, help="JSON file keeping the autotuner's choices")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-scale", type=float, default=0.01)
    ap.add_argument("--serve-slots", type=int, default=256)
    ap.add_argument("--serve-chunk", type=int, default=20000)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
