#!/usr/bin/env python
"""Mining benchmark: one JSON line on stdout (rank 0).

A step is one complete mining job - every frequent pattern with at most k
edges and its exact MNI support - over one seeded synthetic graph:

  default workload  Chung-Lu power-law graph, 100,000 vertices, 1,080,000
                    edges, exponent 2.1, expected-degree cap 1,400, 29 vertex
                    labels Zipf(1.0), 1 edge label, seed 1; min support
                    10,000; patterns up to 3 edges.

value  = mining time per job in milliseconds (lower is better), graph already
         resident in HBM, results delivered to host memory.
e2e    = the same through the C ABI from pinned host buffers: graph upload
         (host->device, adjacency build), mining, results back to host.
embeddings_per_s = extended embeddings per second: child embeddings of
         frequent patterns, the count the reference's extension produces.  The
         GPU's mask path counts most of them without enumerating them one by
         one, so this is a rate of the job, not of per-child work.
roofline = the dominant kernel: algorithmic bytes / CUDA-event time, against
         the measured HBM copy bandwidth.
cpu_baseline = the CPU oracle port (the reference's algorithm, OpenMP on all
         host cores, last level counted without storing it) on a bounded
         sample of the same job: everything above the last level plus one
         slice of the last level's parent embeddings, scaled to a whole job.

--impl reference times that CPU implementation on the same job (rank 0; other
ranks exit): step i runs the levels above the last plus slice i of K of the
last level's parent embeddings, so the K timed steps together cover the whole
last level once; value = median time above the last level + the sum of the
slices' last-level times.  The slices' extended-embedding counts are checked
to add up to the whole job's.

--workload serving: a Poisson stream (mean --rate jobs/s) of jobs over
resident graphs of the three single-graph sizes; jobs/s with p50/p95/p99
latency, each result checked against the same job run alone.
--workload batch_256: the batched engine against the plain one (k 3 by
default; --batch-k 4 runs the stated size, minutes per job).
--workload chung_lu_3_7m / chung_lu_3_7m_k4 / chung_lu_3_7m_k4_s20k /
chung_lu_100k_wide: other single-graph jobs (the large graph at 3 edges, at
4 edges with support 100,000, at 4 edges with its stated support 20,000 -
minutes per job, its 3-edge level generated rather than stored - and a wide
label space).
--fused-last 0|1|2 and --prune set the miner's options of the same names.
--workload text_load: loading a graph from gSpan text on the device against
the host reader and upload.

Multi-GPU (torchrun, N > 1): replicas only - every rank mines the same job on
its own GPU; value = slowest rank's time / jobs on all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "mining time & embeddings/s, batched vs plain on 1 GB300 (exact patterns+MNI)"
UNIT = "ms/job"
EMB_UNIT = "embeddings/s"


def load_datagen():
    """The seeded generators, loaded as a plain module: the reference arm must
    not map this repository's native library (the package's top level loads it
    on first use of a native name, and datagen needs none)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gspan_gb300_datagen",
                                                  os.path.join(ROOT, "gspan_gb300", "datagen.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workloads():
    """Single-graph jobs.  cpu: whether the streaming CPU port finishes the whole
    job within minutes on a 16-core host (the 3.7M-vertex jobs take hours)."""
    datagen = load_datagen()
    return {
        "chung_lu_100k": dict(
            make=lambda: datagen.chung_lu_100k(1), min_support=10000, k=3, cpu=True,
            desc="Chung-Lu 100,000 V / 1,080,000 E, exponent 2.1, degree cap 1,400, 29 vertex labels Zipf(1.0), "
                 "1 edge label, seed 1"),
        # Smaller case of the same kernels for profiler captures: the same graph
        # at a threshold that leaves one frequent 2-edge pattern to extend.
        "chung_lu_100k_s15k": dict(
            make=lambda: datagen.chung_lu_100k(1), min_support=15000, k=3, cpu=True,
            desc="Chung-Lu 100,000 V / 1,080,000 E (as chung_lu_100k), min support 15,000"),
        # The large single graph, at 3 edges: its 4-edge level needs a level-3
        # embedding table of about 1.1e12 rows, beyond the device.
        "chung_lu_3_7m": dict(
            make=lambda: datagen.chung_lu_3_7m(3), min_support=20000, k=3, cpu=False,
            desc="Chung-Lu 3,700,000 V / 16,500,000 E, exponent 2.3, degree cap sqrt(2m), 37 vertex labels "
                 "Zipf(0.8), 1 edge label, seed 3"),
        # The large graph at four edges, at the highest support range where its
        # level-3 embedding table fits the device (about 8.6e9 rows).
        "chung_lu_3_7m_k4": dict(
            make=lambda: datagen.chung_lu_3_7m(3), min_support=100000, k=4, cpu=False,
            desc="Chung-Lu 3,700,000 V / 16,500,000 E (as chung_lu_3_7m), min support 100,000, 4 edges"),
        # The large graph at four edges and its stated support: the 3-edge
        # level (about 1e12 embeddings) is generated inside the 4-edge row
        # pass, never stored.
        "chung_lu_3_7m_k4_s20k": dict(
            make=lambda: datagen.chung_lu_3_7m(3), min_support=20000, k=4, cpu=False,
            desc="Chung-Lu 3,700,000 V / 16,500,000 E (as chung_lu_3_7m), min support 20,000, 4 edges"),
        # A wide label space: 100 vertex labels x 3 edge labels = 300 tuple keys
        # (the row pass's 16-word build).
        "chung_lu_100k_wide": dict(
            make=lambda: datagen.chung_lu(100_000, 1_080_000, 2.1, 100, 1.0, 5, max_deg=1400, nelabels=3),
            min_support=3000, k=3, cpu=True,
            desc="Chung-Lu 100,000 V / 1,080,000 E, exponent 2.1, degree cap 1,400, 100 vertex labels Zipf(1.0), "
                 "3 edge labels, seed 5"),
        "er_3300": dict(
            make=lambda: datagen.er_3300(0), min_support=20, k=3, cpu=True,
            desc="Erdos-Renyi 3,300 V / 4,700 E, 6 uniform vertex labels, 1 edge label, seed 0"),
    }


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_port(graph_path: str, min_support: int, k: int, cores: int, shard: tuple[int, int] | None = None) -> dict:
    """One run of the CPU oracle port with its last level streamed (optionally
    one slice of it); returns its counts and times."""
    port = os.path.join(ROOT, "oracle", "_port", "fsm_port")
    if not os.path.exists(port):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    env = dict(os.environ, OMP_NUM_THREADS=str(cores), CUDA_VISIBLE_DEVICES="")
    args = [port, graph_path, str(min_support), str(k), "--stats", "--stream-last"]
    if shard:
        args += ["--shard", f"{shard[0]}/{shard[1]}"]
    r = subprocess.run(args, capture_output=True, text=True, check=True, env=env)
    out = json.loads(r.stderr.strip().splitlines()[-1])
    out["lines"] = r.stdout.splitlines()[:-1]
    return out


NO_CPU = "the CPU port needs hours for this job (about 4e12 extended embeddings at 3 edges)"


def cpu_sample(graph_path: str, wl: dict, cores: int, slices: int = 4) -> dict:
    """cpu_baseline: the port on the levels above the last plus one slice of
    `slices` of the last level, scaled to a whole job."""
    r = run_port(graph_path, wl["min_support"], wl["k"], cores, shard=(0, slices))
    upper = r["fsm_s"] - r["last_s"]
    job_ms = 1e3 * (upper + slices * r["last_s"])
    return {"value": job_ms, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{wl['desc']}; min support {wl['min_support']}; {wl['k']} edges; every level above the "
                      f"last ({upper:.3f} s) plus slice 1 of {slices} of the last level's parent embeddings "
                      f"({r['last_extended']} extended embeddings in {r['last_s']:.3f} s), last level scaled "
                      f"x{slices}; oracle port, OpenMP, last level streamed"}


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, settle_s: float = 0.3):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.settle_s = settle_s

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(self.settle_s)   # nvidia-smi's own start-up stays out of the timed steps
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 9 and parts[1].isdigit():
                        rows.append(parts)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [int(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace('.', '').isdigit())
                if any(r[3].replace('.', '').isdigit() for r in rows) else None}


def max_over_ranks(values, device=None):
    """Element-wise MAX over all ranks (the values unchanged without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def replica_value(world: int, units_per_rank: float, slowest_ms: float) -> float:
    """Whole-job throughput of `world` replicas: every rank's units over the slowest time."""
    return world * units_per_rank / (slowest_ms / 1e3)


def replica_ms_per_job(world: int, jobs_per_rank: int, slowest_ms: float) -> float:
    """Whole-job time per job of `world` replicas: the slowest rank's time over
    the jobs all ranks completed."""
    return slowest_ms / (world * jobs_per_rank)


def measured_traffic(workload: str, kernel: str):
    """DRAM bytes per launch of `kernel` on `workload` from an ncu capture
    (profiles/dram_traffic.json), or None when none was taken."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if not os.path.exists(path):
        return None, None
    with open(path) as f:
        rec = json.load(f).get(workload)
    if not rec or not kernel.startswith(rec["kernel"]):
        return None, None
    return rec["bytes_per_launch"], rec["source"]


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reference_arm(args, wl) -> None:
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    if not wl["cpu"]:
        print(json.dumps({"impl": "reference", "unavailable": NO_CPU}), flush=True)
        return
    cores = host_cores()
    g = wl["make"]()
    slices = max(args.steps, 1)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "g.bin")
        g.save(path)
        for w in range(args.warmup):
            run_port(path, wl["min_support"], wl["k"], cores, shard=(w % slices, slices))
        runs = [run_port(path, wl["min_support"], wl["k"], cores, shard=(i, slices)) for i in range(slices)]
    upper_s = statistics.median(r["fsm_s"] - r["last_s"] for r in runs)
    last_s = sum(r["last_s"] for r in runs)
    job_ms = 1e3 * (upper_s + last_s)
    upper_ext = runs[0]["extended"] - runs[0]["last_extended"]
    assert all(r["extended"] - r["last_extended"] == upper_ext for r in runs), "levels above the last differ"
    extended = upper_ext + sum(r["last_extended"] for r in runs)
    sample = (f"{wl['desc']}; min support {wl['min_support']}; {wl['k']} edges; step i = every level above the "
              f"last plus slice i of {slices} of the last level's parent embeddings; the slices cover the last "
              f"level once; oracle port, OpenMP, last level streamed")
    line = {
        "impl": "reference", "metric": METRIC, "value": job_ms, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(r["fsm_s"] for r in runs),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator)",
        "config": {"workload": args.workload, "description": wl["desc"], "min_support": wl["min_support"],
                   "k": wl["k"], "parallelism": "cpu"},
        "cpu_baseline": {"value": job_ms, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": job_ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "embeddings_per_s": extended / (job_ms / 1e3), "extended_per_job": extended,
        "job_ms_parts": {"above_last_level_median": 1e3 * upper_s, "last_level_sum": 1e3 * last_s},
    }
    print(json.dumps(line), flush=True)


def hbm_peak() -> tuple[float, str]:
    """The roofline denominator: the measured copy bandwidth of this machine's
    GB300s when MEASURED_PEAKS.json is present, else the earlier measurement
    of 6,800 GB/s on a GB300, labelled as a fallback."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            peak = json.load(f).get("hbm_gbs")
        if peak:
            return float(peak), "MEASURED_PEAKS.json hbm_gbs (measured)"
    return 6800.0, "fallback: 6,800 GB/s, an earlier GB300 measurement (no MEASURED_PEAKS.json hbm_gbs)"


def gpu_arm(args, wl) -> None:
    import numpy as np
    import torch
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from gspan_gb300 import Miner

    g = wl["make"]()
    k, sup = wl["k"], wl["min_support"]
    dev = torch.device("cuda", local)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    # Pinned host copies of the graph for the end-to-end leg.
    off_h = torch.from_numpy(np.ascontiguousarray(g.offsets, dtype=np.int32)).pin_memory()
    vl_h = torch.from_numpy(np.ascontiguousarray(g.vlabels, dtype=np.int32)).pin_memory()
    ed_h = torch.from_numpy(np.ascontiguousarray(g.edges, dtype=np.int32)).pin_memory()
    h2d_graph = off_h.numel() * 4 + vl_h.numel() * 4 + ed_h.numel() * 4

    cpu = None
    if not wl["cpu"]:
        cpu = {"unavailable": NO_CPU}
    elif rank == 0 and world == 1 and not args.no_cpu_baseline:
        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, "g.bin")
            g.save(path)
            cpu = cpu_sample(path, wl, host_cores())

    with Miner(device=local, profile=True, fused_last=args.fused_last, prune=args.prune) as m:
        with ClockSampler(local, settle_s=1.0) as clk:
            # The clock sampler starts before the warm-up, so its start-up does not
            # land on a timed step; it samples through the timed region.
            dg = m.upload_arrays(off_h, vl_h, ed_h)
            for _ in range(args.warmup):
                patterns, st = m.mine(dg, k, sup)
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            step_ms, stats = [], []
            barrier()
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize(dev)
                start.record()
                patterns, st = m.mine(dg, k, sup)
                end.record()
                end.synchronize()
                step_ms.append(start.elapsed_time(end))
                stats.append(st)
            barrier()
            # End to end through the C ABI from pinned host memory.
            e2e_ms, e2e_d2h = [], []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize(dev)
                start.record()
                dg2 = m.upload_arrays(off_h, vl_h, ed_h)
                pats2, st2 = m.mine(dg2, k, sup)
                m.free(dg2)
                end.record()
                end.synchronize()
                e2e_ms.append(start.elapsed_time(end))
                e2e_d2h.append(st2["d2h_bytes"] + sum(20 * len(c) + 4 for c, _ in pats2))
            barrier()
        clocks = clk.summary()
        m.free(dg)
    total_ms = sum(step_ms)
    e2e_total = sum(e2e_ms)
    ext = sum(s["extended"] for s in stats)
    total_ms, e2e_total = max_over_ranks([total_ms, e2e_total], device=dev)
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    value = replica_ms_per_job(world, len(step_ms), total_ms)
    e2e_value = replica_ms_per_job(world, len(e2e_ms), e2e_total)
    # Dominant kernel family by CUDA-event time over the timed steps.
    fams = {"k_mask_rows (mask path row pass)": ("rows_ms", "rows_bytes", "rows_launches"),
            "k_expand Count/Support (per-candidate path)": ("expand_ms", "expand_bytes", "expand_launches"),
            "k_mask_sweep (mask path adjacency sweep)": ("sweep_ms", "sweep_bytes", "rows_launches"),
            "k_expand Materialize (child rows)": ("materialize_ms", "materialize_bytes", "materialize_launches")}
    fam_ms = {name: sum(s[f[0]] for s in stats) for name, f in fams.items()}
    dom = max(fam_ms, key=fam_ms.get)
    exp_ms = fam_ms[dom]
    exp_bytes = sum(s[fams[dom][1]] for s in stats)
    exp_launches = sum(s[fams[dom][2]] for s in stats)
    peak, peak_source = hbm_peak()
    achieved = exp_bytes / (exp_ms / 1e3) / 1e9 if exp_ms > 0 else 0.0
    traffic, traffic_source = measured_traffic(args.workload, dom)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / len(step_ms), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "config": {"workload": args.workload, "description": wl["desc"], "min_support": sup, "k": k,
                   "l2": "flushed between steps (512 MiB write)", "parallelism": "replicas" if world > 1 else "1 GPU",
                   "engine": "plain (level-synchronous)", "fused_last": ["auto", "off", "always"][args.fused_last],
                   "prune": bool(args.prune)},
        "e2e": {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_total / len(e2e_ms),
                "h2d_bytes_per_step": int(h2d_graph + stats[-1]["h2d_bytes"]),
                "d2h_bytes_per_step": int(statistics.median(e2e_d2h))},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic, "traffic_source": traffic_source,
                     "kernel": dom, "launches_per_step": exp_launches / len(stats),
                     "peak_source": peak_source},
        "cpu_baseline": cpu,
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "clocks": clocks,
        "embeddings_per_s": {"value": replica_value(world, ext, total_ms),
                             "e2e": replica_value(world, ext, e2e_total), "unit": EMB_UNIT,
                             "note": "counted, not enumerated: the mask path sums most children per adjacency "
                                     "segment instead of producing them one by one"},
        "extended_per_step": stats[-1]["extended"], "patterns": stats[-1]["patterns"],
        "mining_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)},
        "kernel_ms_per_step": {**{name: ms / len(stats) for name, ms in fam_ms.items()},
                               "seed": sum(s["seed_ms"] for s in stats) / len(stats),
                               "domain sizes": sum(s["domain_ms"] for s in stats) / len(stats)},
        "paths": {"mask_parents": stats[-1]["mask_parents"], "candidate_parents": stats[-1]["candidate_parents"]},
        "fused_rows_per_step": stats[-1]["fused_rows"],
        "host_ms_per_step": {"mine_call": statistics.median(s["mine_ms"] for s in stats),
                             "blocked_in_sync": statistics.median(s["sync_ms"] for s in stats)},
        "pruned": {"vertices": stats[-1]["pruned_vertices"], "entries": stats[-1]["pruned_entries"]},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def batch_arm(args) -> None:
    """256 independent instances: the batched engine (one device store, every
    level of every instance in the same launches) against the plain engine
    mining the instances one by one, on the same GPU, same results."""
    import torch
    from gspan_gb300 import Miner, datagen
    count = 256 if args.workload == "batch_256" else 16
    k = args.batch_k
    t0 = time.time()
    graphs, sups = datagen.batch_instances(2, count)
    gen_s = time.time() - t0
    dev = torch.device("cuda", 0)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    from gspan_gb300 import decode_results
    with Miner(profile=True, fused_last=args.fused_last) as m:
        bg = m.upload_batch(graphs)
        singles = [m.upload(g) for g in graphs]
        for _ in range(args.warmup):
            res, st = m.mine_batch(bg, k, sups, raw=True)
            plain = [m.mine(dg, k, s, raw=True) for dg, s in zip(singles, sups)]
        per_inst = decode_results(res, count)
        assert all(per_inst[i] == decode_results(plain[i][0], 1)[0] for i in range(count)), \
            "batched and plain results differ"
        ext = st["extended"]
        batch_ms, plain_ms = [], []
        # Both engines deliver every pattern to host memory (one flat buffer
        # per call) inside the timed region.
        with ClockSampler(0) as clk:
            for _ in range(args.steps):
                torch.cuda.synchronize(dev)
                start.record()
                res, st = m.mine_batch(bg, k, sups, raw=True)
                end.record()
                end.synchronize()
                batch_ms.append(start.elapsed_time(end))
            for _ in range(args.steps):
                torch.cuda.synchronize(dev)
                start.record()
                plain = [m.mine(dg, k, s, raw=True) for dg, s in zip(singles, sups)]
                end.record()
                end.synchronize()
                plain_ms.append(start.elapsed_time(end))
        clocks = clk.summary()
    bval = statistics.median(batch_ms)
    pval = statistics.median(plain_ms)
    line = {
        "metric": METRIC, "value": bval, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": bval, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "config": {"workload": args.workload, "instances": count, "k": k,
                   "description": "Chung-Lu instances, n log-uniform in [1k, 200k], average degree U[4, 24], "
                                  "8-32 vertex labels Zipf(1.0), exponent 2.1, degree cap sqrt(2m), "
                                  f"min support 2% of n, seed 2; patterns up to {k} edges",
                   "engine": "batched", "fused_last": ["auto", "off", "always"][args.fused_last]},
        "plain": {"value": pval, "unit": UNIT, "ms_per_step": pval},
        "batched_over_plain": pval / bval,
        "embeddings_per_s": {"batched": ext / (bval / 1e3), "plain": ext / (pval / 1e3), "unit": EMB_UNIT,
                             "note": "counted, not enumerated"},
        "extended_per_step": ext, "patterns": st["patterns"], "fused_rows_per_step": st["fused_rows"],
        "generate_s": gen_s, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def serving_arm(args) -> None:
    """Serving: a Poisson stream (mean 50 jobs/s) of mining jobs over a
    resident pool of graphs of the three single-graph sizes (70/25/5 %), min
    support uniform in [1 %, 5 %] of n.  A step is one stream of
    --serving-jobs jobs submitted at their arrival times to a server with
    --slots concurrent contexts; every job's result is checked against the
    same job run alone (a one-slot server, before the timed steps)."""
    import threading
    import torch
    from gspan_gb300 import Server, datagen
    t0 = time.time()
    pool = datagen.serving_pool(4)
    gen_s = time.time() - t0
    classes = [c for c, _ in pool]
    sizes = [g.n for _, g in pool]

    def run_stream(srv, ids, jobs):
        handles = [None] * len(jobs)
        start = time.perf_counter()

        def submit():
            for j, (t, gi, k, sup) in enumerate(jobs):
                delay = start + t - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                handles[j] = srv.submit(ids[gi], k, sup)

        th = threading.Thread(target=submit)
        th.start()
        out = []
        for j in range(len(jobs)):
            while handles[j] is None:
                time.sleep(0.0005)
            out.append(srv.wait(handles[j]))
        th.join()
        return out, time.perf_counter() - start

    results = []
    with Server(slots=1) as alone_srv:
        ids = [alone_srv.add_graph(g) for _, g in pool]
        rate = args.rate if args.rate > 0 else 50.0
        stream_jobs = [datagen.serving_jobs(classes, sizes, args.serving_jobs, rate, seed=40 + i)
                       for i in range(args.steps)]
        if args.rate <= 0:   # capacity: every job of a stream arrives at once
            stream_jobs = [[(0.0,) + j[1:] for j in jobs] for jobs in stream_jobs]
        alone = []
        for jobs in stream_jobs:
            alone.append([alone_srv.wait(alone_srv.submit(ids[gi], k, sup))[0] for _, gi, k, sup in jobs])
    torch.cuda.synchronize()
    with Server(slots=args.slots) as srv:
        ids = [srv.add_graph(g) for _, g in pool]
        warm = [(0.0 if args.rate <= 0 else t, gi, k, sup)
                for t, gi, k, sup in datagen.serving_jobs(classes, sizes, args.serving_jobs, rate, seed=30)]
        for _ in range(args.warmup):
            run_stream(srv, ids, warm)
        lat, qms, ext, walls, retried = [], [], 0, [], 0
        with ClockSampler(0) as clk:
            for step, jobs in enumerate(stream_jobs):
                out, wall = run_stream(srv, ids, jobs)
                walls.append(wall)
                for j, (res, info) in enumerate(out):
                    assert res == alone[step][j], f"job {j} of stream {step} differs from its result alone"
                    lat.append(info["latency_ms"])
                    qms.append(info["queued_ms"])
                    ext += info["stats"]["extended"]
                    retried += info["retried_alone"]
        clocks = clk.summary()
    lat.sort()

    def pct(p):
        return lat[min(len(lat) - 1, int(round(p / 100.0 * (len(lat) - 1))))]

    njobs = len(lat)
    line = {
        "metric": "serving: jobs/s with p50/p95/p99 job latency (exact patterns+MNI)", "value": njobs / sum(walls),
        "unit": "jobs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(walls), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "config": {"workload": "serving", "rate_jobs_per_s": args.rate if args.rate > 0 else "all at once", "jobs_per_step": args.serving_jobs,
                   "slots": args.slots, "mix": "70/25/5 % Erdos-Renyi 3,300 V / Chung-Lu 100,000 V / "
                   "Chung-Lu 3,700,000 V (8/3/1 resident graphs, seed 4)",
                   "min_support": "uniform [1 %, 5 %] of n", "k": "3 or 4 (3,300 V), 3 (others)"},
        "latency_ms": {"p50": pct(50), "p95": pct(95), "p99": pct(99), "max": lat[-1],
                       "mean_queued": statistics.mean(qms)},
        "embeddings_per_s": ext / sum(walls), "jobs": njobs, "retried_alone": retried,
        "all_equal_alone": True, "generate_s": gen_s, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def text_arm(args) -> None:
    """Loading a graph from gSpan text: on the device (gspan_graph_upload_text:
    tokens to device store on the GPU) against the host path (the convert tool's
    reader and CSR build, writing and reading the .bin, then the upload)."""
    from gspan_gb300 import Miner, datagen
    g = datagen.chung_lu_100k(1)
    text = datagen.to_gspan_text(g).encode()
    convert = os.path.join(ROOT, "gspan_gb300", "_lib", "convert")
    dev_ms, host_ms = [], []
    with Miner() as m, tempfile.TemporaryDirectory() as tmp:
        src, dst = os.path.join(tmp, "g.txt"), os.path.join(tmp, "g.bin")
        with open(src, "wb") as f:
            f.write(text)
        # Outside the timed region: both loaders must give the same graph, as
        # seen by mining it (every pattern and support at 2 edges).
        subprocess.run([convert, src, dst], check=True, capture_output=True)
        dg_text, dg_host = m.upload_text(text), m.upload(datagen.load_bin(dst))
        same = m.mine(dg_text, 2, 10000)[0] == m.mine(dg_host, 2, 10000)[0]
        m.free(dg_text)
        m.free(dg_host)
        assert same, "device text loader and host reader give different graphs"
        for step in range(args.warmup + args.steps):
            t = time.perf_counter()
            dg = m.upload_text(text)
            d = time.perf_counter() - t
            m.free(dg)
            t = time.perf_counter()
            subprocess.run([convert, src, dst], check=True, capture_output=True)
            dg = m.upload(datagen.load_bin(dst))
            h = time.perf_counter() - t
            m.free(dg)
            if step >= args.warmup:
                dev_ms.append(1e3 * d)
                host_ms.append(1e3 * h)
    print(json.dumps({
        "metric": "graph load from gSpan text (device loader vs host reader + upload)",
        "value": statistics.median(dev_ms), "unit": "ms", "higher_is_better": False, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "data": "synthetic (seeded generator)",
        "config": {"workload": "text_load", "description": "chung_lu_100k as gSpan text",
                   "text_bytes": len(text)}, "same_graph_checked": True,
        "host_ms": statistics.median(host_ms)}), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", default="chung_lu_100k")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fused-last", type=int, default=0, choices=[0, 1, 2],
                    help="next-to-last level: 0 auto, 1 stored, 2 generated inside the last row pass")
    ap.add_argument("--prune", action="store_true", help="drop vertices of infrequent labels before mining")
    ap.add_argument("--batch-k", type=int, default=3,
                    help="batch_256 / batch_16: pattern size in edges (4 is the stated size: one batched job "
                         "takes minutes, so the batched-vs-plain comparison defaults to 3)")
    ap.add_argument("--slots", type=int, default=4, help="serving: concurrent contexts")
    ap.add_argument("--serving-jobs", type=int, default=100, help="serving: jobs per stream (one step)")
    ap.add_argument("--rate", type=float, default=50.0, help="serving: mean arrivals per second (0: all at once)")
    args = ap.parse_args()
    if args.workload == "serving":
        serving_arm(args)
        return
    if args.workload == "text_load":
        text_arm(args)
        return
    if args.workload in ("batch_256", "batch_16"):
        batch_arm(args)
        return
    wl = workloads()[args.workload]
    if args.impl == "reference":
        reference_arm(args, wl)
    else:
        gpu_arm(args, wl)


if __name__ == "__main__":
    main()
