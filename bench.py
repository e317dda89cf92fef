#!/usr/bin/env python
"""Benchmark: shortest-path node centrality (closeness + betweenness) on one GB300.

Workload: the city-scale primal lattice -- 450x450 jittered lattice (202,500 nodes) at 80 m,
jitter +-15 m, 10% of streets dropped, 5% of nodes with a diagonal shortcut of length
euclid * U(1.0, 1.3); every node a source; distances 500/1000/2000/5000 m (beta = 4/d rounded to
5 dp).  A step is one pass of the hot path over all 202,500 sources.

  value  sources/s with the CSR and accumulators resident in HBM (C-ABI call, CUDA events)
  e2e    sources/s through the public API (NetworkStructure.centrality_shortest) with the CSR
         copied host->device and the result rows device->host inside every timed step
  cpu_baseline  the CPU oracle (a C restatement of the reference's rust centrality) on this
         host's cores, over a bounded, evenly strided sample of the same sources

`--impl reference` times that same CPU restatement as the reference arm (the reference itself is
Rust + PyO3 and cannot be built here).  Multi-GPU: sources are independent, so every rank runs a
full replica of the workload and `value` sums ranks (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "sources/s at 200k nodes, d<=5 km (shortest-path closeness + betweenness)"
UNIT = "sources/s"
WORKLOAD = "lattice450_c2"


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def build_workload(side: int | None = None):
    from cityseer_gb300 import synth

    p, dists = synth.lattice_config("c2", side=side)
    ns = synth.primal_structure(p)
    return ns, dists


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": float(max(smax)) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def cpu_baseline(ns, dists, n_total: int, target_seconds: float, nthreads: int | None = None):
    """Times the CPU oracle over an evenly strided sample of the sources, sized to ~target_seconds."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    # thresholds from the oracle's own restatement of pair_distances_betas_time
    # (rust/src/common.rs:239-270), so that this leg loads no code of the library it is compared with
    d = [int(x) for x in dists]
    b = oracle.betas_from_distances(d)
    s = oracle.seconds_from_distances(d, 1.33333)
    og = oracle.OracleGraph(ns)
    # rayon's pool in the reference runs on all cores but one (rust/src/lib.rs:21-33)
    nthreads = nthreads or oracle.default_threads()
    plan = oracle.all_sources_plan(ns)
    allsrc = plan["sources"]

    def run(count):
        idx = np.linspace(0, len(allsrc) - 1, count).astype(np.int64)
        pl = dict(plan)
        pl["sources"] = allsrc[idx]
        t0 = time.perf_counter()
        oracle.centrality_shortest(og, d, b, s, plan=pl, nthreads=nthreads)
        return time.perf_counter() - t0

    probe = max(nthreads * 8, 128)
    run(probe)  # first call pays one-time costs (library load, first touch of the output rows)
    tp = run(probe)
    count = int(min(n_total, max(probe, probe * target_seconds / max(tp, 1e-6))))
    t = run(count)
    if t < 0.5 * target_seconds and count < n_total:  # the probe overestimated the per-source cost
        count = int(min(n_total, count * target_seconds / max(t, 1e-6)))
        t = run(count)
    return {
        "value": count / t,
        "unit": UNIT,
        "cores": nthreads,
        "kind": "port",
        "sample": f"{count} of {n_total} sources (evenly strided), {t:.1f} s on {nthreads} threads; "
                  f"C restatement of the reference rust centrality (oracle/cs_oracle.c)",
        "seconds": t,
    }


def traffic_ratio(kernel: str = "primal_sync_kernel"):
    """DRAM bytes per algorithmic byte of the timed kernel, from the ncu figures kept in
    profiles/traffic.json (one capture of that kernel on a smaller lattice of the same recipe)."""
    try:
        return float(json.loads((ROOT / "profiles" / "traffic.json").read_text())[kernel]["traffic_per_alg_byte"])
    except (OSError, KeyError, ValueError, TypeError):
        return None


def flush_l2(buf):
    buf.add_(1.0)


def loaded_native_libraries():
    """Shared objects of this repository mapped into the process (from /proc/self/maps)."""
    found = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if line.strip() else ""
                if path.endswith(".so") and path.startswith(str(ROOT)):
                    found.add(str(Path(path).relative_to(ROOT)))
    except OSError:
        pass
    return sorted(found)


def run_reference(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    ns, dists = build_workload(args.side)  # numpy graph store only: no device code is loaded
    n = ns.node_count()
    times = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(ns, dists, n, args.cpu_seconds)
        if i >= args.warmup:
            times.append(r)
    val = float(np.mean([t["value"] for t in times]))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": val,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": float(np.mean([t["seconds"] for t in times]) * 1000.0),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "nodes": n, "distances": dists},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": times[-1]["cores"], "kind": times[-1]["kind"],
                         "sample": f"{len(times)} timed steps of: " + times[-1]["sample"]},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_libraries": loaded_native_libraries(),
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    from cityseer_gb300 import _native, centrality, common

    ws, rank, local = _dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    lib = _native.load()
    ns, dists = build_workload(args.side)
    n_nodes = ns.node_count()
    speed = 1.33333
    d, b, s = common.pair_distances_betas_time(speed, distances=dists)
    K = len(d)
    # ---- resident state (as the public API leaves it after a first call)
    first = ns.centrality_shortest(distances=dists)
    csr = centrality._primal_csr(ns)
    wsp = centrality._workspace(ns, csr, 0, K, speed, max(s))
    sp = centrality.prepare_source_sampling(ns, None, None, None, None)
    proc_t = torch.from_numpy(sp.process).to(dev)
    wt_t = torch.from_numpy(sp.src_wt).to(dev)
    el_t = torch.from_numpy(sp.eligible).to(dev)
    q = centrality._make_query(d, b, s, speed, float(centrality.TIE_EPSILON), True, True, False, proc_t, wt_t,
                               el_t)
    g = csr.struct(speed)
    nb = csr.n_bound
    out = torch.zeros((7, K, nb), dtype=torch.float64, device=dev)
    reach = torch.zeros(K, dtype=torch.int32, device=dev)
    outs = _native.Outputs(out.data_ptr(), reach.data_ptr())
    stream = torch.cuda.current_stream()
    l2 = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2

    def hot():
        rc = lib.cs_centrality_shortest(C.byref(g), C.byref(q), C.byref(wsp.plan), wsp.ptr, wsp.nbytes, outs,
                                        stream.cuda_stream)
        _native.check(rc, "cs_centrality_shortest")

    for _ in range(args.warmup):
        out.zero_()
        hot()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    times = []
    counters = []
    launches = 0
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        out.zero_()
        flush_l2(l2)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        hot()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1000.0)
        c = centrality.last_counters()
        counters.append(c)
        launches += c[3]
    ph = (C.c_int64 * 8)()
    lib.cs_last_phase_cycles(ph, 8)
    ph = [int(x) for x in ph][:7]
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    step_s = float(np.mean(times))
    n_src = len(sp.process)
    from cityseer_gb300.replicas import job_throughput

    value, t_max = job_throughput(n_src, step_s, dev)
    # ---- parity guard: the timed outputs equal the public API's first result
    res_rows = out.cpu().numpy()
    idx = np.asarray(ns.node_indices())
    assert np.array_equal(res_rows[0, -1][idx], first.node_density[d[-1]]), "timed run diverged"
    # ---- roofline: algorithmic bytes (12 B per relaxed edge, 24 B per settled node, 8 B per f64
    # accumulation with M = 7 per reached target per threshold)
    _, e_relax, n_settled, _ = counters[-1]
    reach_sum = float(res_rows[0].sum())  # sum_k sum_t density = sum_k N_reach,k (unit weights)
    alg_bytes = 12.0 * e_relax + 24.0 * n_settled + 8.0 * 7.0 * reach_sum
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / step_s / 1e9
    roofline = {
        "bound": "hbm",
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": (traffic_ratio() * alg_bytes) if traffic_ratio() else None,
        "traffic_note": "DRAM bytes per launch: the ncu traffic per algorithmic byte of a smaller lattice "
                        "(profiles/traffic.json) times this launch's algorithmic bytes",
        "peak_kind": peak_kind,
        "alg_bytes_per_launch": alg_bytes,
        "edges_relaxed": int(e_relax),
        "nodes_settled": int(n_settled),
        "reached_target_thresholds": int(reach_sum),
    }
    # ---- e2e through the public API: CSR host->device, results device->host, every step
    host = centrality._primal_host(ns)
    h2d = host.nbytes(speed) + sp.process.nbytes + sp.src_wt.nbytes + sp.eligible.nbytes
    d2h = 7 * K * nb * 8 + K * 4
    e2e_times = []
    for i in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        centrality.drop_device_state(ns)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ns.centrality_shortest(distances=dists)
        _ = r.node_betweenness
        torch.cuda.synchronize()
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
    e2e_v = job_throughput(n_src, float(np.mean(e2e_times)), dev)[0] if e2e_times else None
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_max * 1000.0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded jittered lattice, see cityseer_gb300/synth.py)",
        "config": {
            "workload": WORKLOAD,
            "nodes": n_nodes,
            "directed_edges": int(csr.m),
            "distances": d,
            "sources_per_step": n_src,
            "l2": "flushed between timed steps (256 MB write)",
            "parallelism": f"replicas x{ws}",
            # search slots of the shortest-path launches (plans sized for the 4-block budget hold
            # more; the block-synchronous shortest-path kernel runs with 3 blocks per SM)
            "slots": int(min(wsp.plan.n_slots, lib.cs_device_sm_count() * 3 * 8)
                         if wsp.plan.variant == 0 else wsp.plan.n_slots),
            "cap": int(wsp.plan.cap),
            "delta_s": float(wsp.plan.delta_seconds),
        },
        "e2e": {"value": e2e_v, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": roofline,
        "gpu_launches": int(launches),
        "phase_share": {nm: round(v / max(1, sum(ph)), 4) for nm, v in
                        zip(("search", "sort", "replay", "closeness", "sigma", "backward", "reset"), ph)},
        "clocks": clk,
    }
    if rank == 0 and ws == 1 and not args.no_cpu:  # the CPU baseline is reported at N = 1 only
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(ns, dists, n_nodes, args.cpu_seconds).items()
                                if k != "seconds"}
    if rank == 0 and ws == 1 and not args.no_extra:
        # the rest of the headline metric, each leg bounded: batched vs plain, served latency,
        # simplest paths on the curved lattice's dual
        centrality.drop_device_state(ns)
        del out, l2
        torch.cuda.empty_cache()
        line.update(extra_legs(args))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def extra_legs(args) -> dict:
    """Summaries of the batched, served and curved-dual legs for the default bench line."""
    import torch

    out = {}
    t0 = time.perf_counter()
    b = run_batch(argparse.Namespace(**{**vars(args), "graphs": args.extra_graphs, "steps": 3, "warmup": 1,
                                        "plain_steps": 1}))
    out["batched"] = {
        "workload": b["config"]["workload"], "graphs": b["config"]["graphs"],
        "reduced_from": "the 96-graph batched configuration: its first %d graphs" % b["config"]["graphs"],
        "items_per_s": b["value"], "plain_items_per_s": b["plain"]["value"],
        "batched_over_plain": b["batched_over_plain"], "parity_max_rel": b["parity_max_rel"],
        "ms_per_step": b["ms_per_step"], "plain_ms_per_step": b["plain"]["ms_per_step"],
        "leg_seconds": round(time.perf_counter() - t0, 1),
    }
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    sv = run_serve(argparse.Namespace(**{**vars(args), "serve_rates": "500", "serial_seconds": 15.0}))
    at = sv["sweep"][0]
    out["served"] = {
        "workload": sv["config"]["workload"], "rate_req_s": at["rate_req_s"], "requests": at["requests"],
        "saturated": at["saturated"], "sources_per_s": at["sources_per_s"],
        "p50_ms_le_1k_sources": at["le_1k_sources"].get("p50_ms"),
        "p99_ms_le_1k_sources": at["le_1k_sources"].get("p99_ms"),
        "shortest": at["shortest"], "simplest": at["simplest"],
        "serial_plain_sources_per_s": sv["serial_plain"]["sources_per_s"],
        "served_over_serial_sources_per_s": sv["served_over_serial_sources_per_s"],
        "leg_seconds": round(time.perf_counter() - t0, 1),
    }
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    c3 = run_c3(argparse.Namespace(**{**vars(args), "side": None, "steps": 2, "warmup": 1}))
    out["simplest"] = {
        "workload": c3["config"]["workload"], "dual_nodes": c3["config"]["dual_nodes"],
        "dual_sources_per_s": c3["value"], "ms_per_step": c3["ms_per_step"],
        "segment_sources_per_s": c3["segment"]["value"],
        "sources_redone_exactly": c3["simplest_sources_redone_exactly"],
        "phase_share": c3["simplest_phase_share"],
        "replay_rounds_per_source": c3["simplest_replay_rounds_per_source"],
        "leg_seconds": round(time.perf_counter() - t0, 1),
    }
    return out


BATCH_METRIC = "sources/s, 96 mixed-size graphs (2k-150k nodes), shortest + segment: batched vs plain GPU"


def run_batch(args):
    """Batched form: 96 lattices of log-uniform size 2k-150k nodes (built like the 40x40 case, own
    seeds), 2-4 thresholds each from {400, 800, 1200, 1600, 3200, 4800} m, every node a source of a
    shortest-path job (closeness + betweenness) and of a segment job.  `value` replays the captured
    batched launch (CUDA graph) with everything resident; `plain` runs the same jobs as per-graph
    C-ABI calls of the plain path (each with its own plan and a workspace re-initialised in place),
    also resident and timed with CUDA events on the same stream."""
    import torch

    from cityseer_gb300 import _native, centrality, device, synth
    from cityseer_gb300.batch import Batch
    from cityseer_gb300.common import pair_distances_betas_time

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    lib = _native.load()
    t0 = time.perf_counter()
    work = synth.batch_workload(n_graphs=args.graphs)
    graphs = [(synth.primal_structure(p), d) for p, d in work]
    t_build = time.perf_counter() - t0
    jobs = []
    for ns, dists in graphs:
        jobs.append(dict(ns=ns, mode="shortest", distances=dists))
        jobs.append(dict(ns=ns, mode="segment", distances=dists))
    t0 = time.perf_counter()
    b = Batch(jobs, tune=False)
    t_setup = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    # ---- batched: one captured graph = zero outputs + header reset + one persistent launch + prefixes
    b.capture()
    for _ in range(args.warmup):
        b.replay()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.graph.replay()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1000.0)
    overflowed, done = b.status()
    clk = clocks.stop()
    if overflowed:
        b.replay()  # re-run with in-call retry so the parity check below sees complete results
    t_batch = float(np.mean(times))
    counters = centrality.last_counters()
    batched_rows = [jb["out"].clone() for jb in b.jobs]
    # e2e of the batched form: replay + every job's result rows device->host
    e2e = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.graph.replay()
        host_rows = [jb["out"].cpu() for jb in b.jobs]
        e2e.append(time.perf_counter() - t0)
    d2h = sum(r.numel() * 8 for r in host_rows)
    # ---- plain: per-graph calls of the plain C-ABI path, resident inputs and outputs
    plain_jobs = []
    ws_bytes = 0
    for j, spec in enumerate(jobs):
        ns = spec["ns"]
        mode = 0 if spec["mode"] == "shortest" else 1
        jb = b.jobs[j]
        csr = jb["csr"]
        d, bb, s = pair_distances_betas_time(1.33333, distances=spec["distances"])
        r = centrality.estimate_reach(ns, csr, 1.33333, max(s))
        cap = int(min(csr.n_bound, max(1024, -(-int(r * 1.3) // 256) * 256)))
        plan = device.plan_primal(csr, mode, len(d), 1.33333, cap=cap, mem_budget=centrality._mem_budget(dev))
        ws_bytes = max(ws_bytes, int(plan.workspace_bytes))
        q = centrality._make_query(d, bb, s, 1.33333, float(centrality.TIE_EPSILON), True, True, False,
                                   jb["keep"][0], jb["keep"][1], jb["keep"][2])
        out = torch.zeros_like(jb["out"])
        plain_jobs.append((mode, csr.struct(1.33333), q, plan, csr.n_bound, out))
    del b.graph
    b.graph = None
    torch.cuda.empty_cache()
    wsbuf = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)

    def plain_pass():
        for mode, g, q, plan, nb, out in plain_jobs:
            out.zero_()
            _native.check(lib.cs_workspace_init(C.byref(plan), nb, wsbuf.data_ptr(), ws_bytes, stream.cuda_stream),
                          "cs_workspace_init")
            fn = lib.cs_centrality_shortest if mode == 0 else lib.cs_segment_centrality
            _native.check(fn(C.byref(g), C.byref(q), C.byref(plan), wsbuf.data_ptr(), ws_bytes,
                             _native.Outputs(out.data_ptr(), None), stream.cuda_stream), "plain call")

    plain_pass()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ptimes = []
    for _ in range(max(1, args.plain_steps)):
        e0.record(stream)
        plain_pass()
        e1.record(stream)
        e1.synchronize()
        ptimes.append(e0.elapsed_time(e1) / 1000.0)
    t_plain = float(np.mean(ptimes))
    # ---- parity guard: every job's batched rows equal its plain rows (order-of-summation tolerance)
    worst = 0.0
    for (mode, g, q, plan, nb, out), rows in zip(plain_jobs, batched_rows):
        a, c = rows.double(), out.double()
        if mode == 0:
            assert torch.equal(a[0], c[0]), "batched density differs from the plain call"
        worst = max(worst, float(((a - c).abs() / c.abs().clamp_min(1e-3)).max()))
    assert worst < 1e-6, f"batched rows differ from plain rows (rel {worst})"
    n_items = sum(len(jb["proc"]) for jb in b.jobs)  # (job, source) pairs: a fused item serves two
    n_nodes = sum(ns.node_count() for ns, _ in graphs)
    line = {
        "metric": BATCH_METRIC,
        "value": n_items / t_batch,
        "unit": UNIT,
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_batch * 1000.0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded jittered lattices, cityseer_gb300/synth.py batch_workload)",
        "config": {
            "workload": f"batch{len(graphs)}_mixed_2k_150k",
            "graphs": len(graphs),
            "jobs": len(jobs),
            "nodes_total": n_nodes,
            "items_per_step": n_items,
            "launch_items_per_step": b.n_items,
            "fused_jobs": b.n_fused,
            "l2": "inputs larger than L2 (workspace + 96 graphs)",
            "slots": int(b.plan.n_slots),
            "cap": int(b.plan.cap),
            "variant": int(b.plan.variant),
        },
        "plain": {"value": n_items / t_plain, "ms_per_step": t_plain * 1000.0, "launch_calls": len(plain_jobs)},
        "batched_over_plain": t_plain / t_batch,
        "e2e": {"value": n_items / float(np.min(e2e)), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(d2h)},
        "edges_relaxed_per_s": counters[1] / t_batch,
        "parity_max_rel": worst,
        "setup_s": {"graphs": round(t_build, 2), "batch": round(t_setup, 2)},
        "gpu_launches": 2,
        "clocks": clk,
    }
    return line


SERVE_METRIC = "served p50/p99 latency and sources/s, 6 resident graphs (50k-1.2M nodes), Poisson arrivals"


def _serve_requests(prims, duals, rate: float, duration: float, seed: int):
    """Poisson request stream: graph uniform, source subset log-uniform 1-8192 drawn uniformly,
    1-4 thresholds with the maximum U(400, 5000) m, shortest w.p. 0.8 else simplest on the dual."""
    from cityseer_gb300.serve import Query

    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    idx = {g: np.asarray(ns.node_indices()) for g, ns in prims.items()}
    didx = {g: np.asarray(ns.node_indices()) for g, ns in duals.items()}
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        gid = int(rng.integers(0, len(prims)))
        simplest = bool(rng.random() < 0.2)
        pool = didx[gid] if simplest else idx[gid]
        size = min(len(pool), int(np.exp(rng.uniform(0.0, np.log(8192.0)))))
        src = rng.choice(pool, size=size, replace=False)
        k = int(rng.integers(1, 5))
        dmax = int(rng.uniform(400, 5000))
        dists = sorted(set([dmax] + [int(rng.uniform(100, dmax)) for _ in range(k - 1)]))
        out.append((t, Query(gid, src.tolist(), dists, "simplest" if simplest else "shortest")))
    return out


def run_serve(args):
    """Served form: 6 device-resident lattices (C1 recipe) of 50k-1.2M nodes plus their duals; Poisson
    request streams at each rate; latency = arrival -> rows complete on the device.  Beside it, the
    same 500 req/s stream as a serial loop of plain C-ABI calls (resident, one call per request)."""
    import torch

    from cityseer_gb300 import _native, centrality, dual, synth
    from cityseer_gb300.common import pair_distances_betas_time
    from cityseer_gb300.serve import Server, latency_summary

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    sizes = [int(x) for x in args.serve_sizes.split(",")]
    t0 = time.perf_counter()
    prims, duals = {}, {}
    for gid, n in enumerate(sizes):
        p = synth.lattice(side=int(round(np.sqrt(n))), spacing=100.0, jitter=20.0, drop=0.15, seed=500 + gid)
        prims[gid] = synth.primal_structure(p)
        duals[gid] = synth.dual_structure(p)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    srv = Server(prims, duals, max_distance=5000, max_thresholds=4, keep_results=False)
    t_setup = time.perf_counter() - t0
    srv.start()
    # warm-up: a few queries of each mode on each graph
    from cityseer_gb300.serve import Query

    warm = []
    for gid in prims:
        warm.append(srv.submit(Query(gid, list(range(0, 64)), [800, 5000], "shortest")))
        warm.append(srv.submit(Query(gid, list(range(0, 8)), [800], "simplest")))
    srv.drain(timeout=600)
    rates = [float(x) for x in args.serve_rates.split(",")]
    sweep = []
    clocks = ClockSampler(0)
    clocks.start()
    streams = {}
    for ri, rate in enumerate(rates):
        reqs = _serve_requests(prims, duals, rate, args.serve_seconds, seed=900 + ri)
        streams[rate] = reqs
        tickets = []
        start = time.perf_counter()
        for at, q in reqs:
            now = time.perf_counter() - start
            if at > now:
                time.sleep(at - now)
            tickets.append(srv.submit(q, t_arrival=start + at))
        saturated = False
        try:
            srv.drain(timeout=max(30.0, 10.0 * args.serve_seconds))
        except TimeoutError:
            saturated = True
            srv.cancel()
            srv.drain(timeout=900)
        ok = [t for t in tickets if t.done and t.error is None]
        end = max(t.t_done for t in ok) if ok else start
        n_src = sum(len(t.query.sources) for t in ok)
        errs = [t.error for t in tickets if t.error is not None and "cancelled" not in str(t.error)]
        if errs:
            raise errs[0]
        sweep.append({
            "rate_req_s": rate, "requests": len(reqs), "completed": len(ok), "saturated": saturated,
            "sources": n_src, "sources_per_s": n_src / max(1e-9, end - start),
            "all": latency_summary(ok), "le_1k_sources": latency_summary(ok, 1000),
            "shortest": latency_summary([t for t in ok if t.query.mode == "shortest"]),
            "simplest": latency_summary([t for t in ok if t.query.mode == "simplest"]),
        })
        if saturated:
            break
    clk = clocks.stop()
    st = srv.stats()
    srv.stop()
    del srv
    torch.cuda.empty_cache()
    # plain simplest-path calls share one dual workspace sized for the largest dual graph
    big = max(duals, key=lambda g: duals[g].node_bound())
    dcap = max(dual.estimate_states(ns, 1.33333, 3751) for ns in duals.values())
    dplan = _native.Plan()
    _native.check(_native.load().cs_plan_dual(C.byref(dual.dual_csr(duals[big]).struct(1.33333)), 0, 4, dcap, 0,
                                              centrality._mem_budget(dev) // 3, C.byref(dplan)), "cs_plan_dual")
    dws = dual.DualWorkspace(dplan, dplan.n_bound, dev)
    # ---- serial loop of plain calls on the 500 req/s stream (or the nearest rate)
    rate_ser = min(streams, key=lambda r: abs(r - 500.0))
    reqs = streams[rate_ser]
    lib = _native.load()
    speed = 1.33333
    stream = torch.cuda.current_stream()
    ws_p = {}
    for gid, ns in prims.items():
        csr = centrality._primal_csr(ns)
        _, _, s5 = pair_distances_betas_time(speed, distances=[5000])
        ws_p[gid] = centrality._workspace(ns, csr, 0, 4, speed, s5[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n_ser = 0
    n_req_ser = 0
    for _, q in reqs:
        if time.perf_counter() - t0 > args.serial_seconds:
            break
        n_ser += len(q.sources)
        n_req_ser += 1
        d, b, s = pair_distances_betas_time(speed, distances=q.distances)
        if q.mode == "shortest":
            ns = prims[q.graph]
            csr = centrality._primal_csr(ns)
            g = csr.struct(speed)
            ws = ws_p[q.graph]
            nb = csr.n_bound
            fn = lib.cs_centrality_shortest
            rows = 7
        else:
            ns = duals[q.graph]
            csr = dual.dual_csr(ns)
            g = csr.struct(speed)
            ws = dws
            nb = csr.n_bound
            fn = lib.cs_centrality_simplest
            rows = 4
        src_t = torch.tensor(q.sources, dtype=torch.int32, device=dev)
        wt_t = torch.zeros(nb, dtype=torch.float32, device=dev)
        el_t = torch.zeros(nb, dtype=torch.uint8, device=dev)
        wt_t[src_t.long()] = 1.0
        el_t[src_t.long()] = 1
        out = torch.zeros((rows, len(d), nb), dtype=torch.float64, device=dev)
        reach = torch.zeros(len(d), dtype=torch.int32, device=dev)
        qq = centrality._make_query(d, b, s, speed, float(centrality.TIE_EPSILON), True, True, True, src_t, wt_t,
                                    el_t)
        _native.check(fn(C.byref(g), C.byref(qq), C.byref(ws.plan), ws.ptr, ws.nbytes,
                         _native.Outputs(out.data_ptr(), reach.data_ptr()), stream.cuda_stream), "serial plain call")
    torch.cuda.synchronize()
    t_ser = time.perf_counter() - t0
    at500 = next(x for x in sweep if x["rate_req_s"] == rate_ser)
    line = {
        "metric": SERVE_METRIC,
        "value": at500["sources_per_s"],
        "unit": "sources/s",
        "n_gpus": 1,
        "steps": len(rates),
        "warmup": len(warm),
        "ms_per_step": None,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded jittered lattices and their duals, Poisson request streams)",
        "config": {"workload": "serve6_50k_1200k", "graph_nodes": [ns.node_count() for ns in prims.values()],
                   "dual_nodes": [ns.node_count() for ns in duals.values()], "seconds_per_rate": args.serve_seconds,
                   "latency": "arrival to result rows complete on the device", **st},
        "sweep": sweep,
        "serial_plain": {"rate_req_s": rate_ser, "requests": n_req_ser, "of": len(reqs),
                         "sources_per_s": n_ser / t_ser, "seconds": t_ser},
        "served_over_serial_sources_per_s": at500["sources_per_s"] / (n_ser / t_ser),
        "p99_ms_le_1k_sources_at_rate": {str(x["rate_req_s"]): x["le_1k_sources"].get("p99_ms") for x in sweep},
        "setup_s": {"graphs": round(t_build, 1), "server": round(t_setup, 1)},
        "clocks": clk,
    }
    return line


def run_c3(args):
    """The curved-lattice configuration (250x250 jittered lattice, 30% of streets curved): simplest-path
    centrality on its dual (124,500 dual nodes) and segment centrality on the primal, thresholds
    [500, 1000, 2000] m, through the public API; wall clock around each call with the device
    synchronised, inputs resident after the warm-up calls.  Parity of both paths is in the tests."""
    import torch

    from cityseer_gb300 import _native, synth

    p, dists = synth.lattice_config("c3", side=args.side)
    t0 = time.perf_counter()
    nsd = synth.dual_structure(p)
    ns = synth.primal_structure(p)
    t_build = time.perf_counter() - t0
    n_seg = sum(1 for v in ns.node_indices() if ns.is_node_live(v))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t)
        return float(np.mean(ts))

    clocks = ClockSampler(0)
    clocks.start()
    t_simp = timed(lambda: nsd.centrality_simplest(distances=dists))
    over, inexact = C.c_int64(), C.c_int64()
    _native.load().cs_last_retries(C.byref(over), C.byref(inexact))
    # per-phase SM cycles of the last simplest-path call (summed over warps) and its replay rounds
    ph = (C.c_int64 * 16)()
    _native.load().cs_last_phase_cycles(ph, 16)
    tot = max(1, sum(ph[:7]))
    names = ("search", "sort", "replay", "node_best_closeness", "backward", "reset", "exact_search")
    dual_phases = {k: round(ph[i] / tot, 4) for i, k in enumerate(names)}
    rounds = ph[7] / max(1, nsd.node_count())
    t_seg = timed(lambda: ns.segment_centrality(distances=dists))
    clk = clocks.stop()
    line = {
        "metric": "sources/s, 250x250 curved lattice, d<=2 km: simplest-path centrality on the dual "
                  "(segment centrality on the primal beside it)",
        "value": nsd.node_count() / t_simp,
        "unit": "sources/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_simp * 1000.0,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded curved jittered lattice and its dual, see cityseer_gb300/synth.py)",
        "config": {"workload": "c3_curved250", "dual_nodes": nsd.node_count(), "primal_nodes": ns.node_count(),
                   "distances": dists, "timing": "wall clock per public-API call, device synchronised"},
        "segment": {"value": n_seg / t_seg, "unit": "sources/s", "ms_per_step": t_seg * 1000.0},
        "simplest_sources_redone_exactly": int(inexact.value),
        "simplest_phase_share": dual_phases,
        "simplest_replay_rounds_per_source": round(rounds, 3),
        "setup_s": round(t_build, 1),
        "clocks": clk,
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--side", type=int, default=None, help="lattice side override (small runs only)")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "batch", "serve"],
                    help="c2: the 202,500-node lattice (default); c3: the curved lattice, simplest paths "
                         "on its dual and segments on the primal; batch: the 96-graph batched form; "
                         "serve: the served form")
    ap.add_argument("--serve-sizes", default="50000,100000,200000,400000,800000,1200000")
    ap.add_argument("--serve-rates", default="20,100,500,2000")
    ap.add_argument("--serve-seconds", type=float, default=3.0)
    ap.add_argument("--serial-seconds", type=float, default=60.0)
    ap.add_argument("--graphs", type=int, default=96)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--no-extra", action="store_true",
                    help="default workload only: skip the batched, served and curved-dual legs")
    ap.add_argument("--extra-graphs", type=int, default=48, help="graphs of the batched leg in the default line")
    args = ap.parse_args()
    if args.workload == "batch" and args.impl != "reference":
        print(json.dumps(run_batch(args)), flush=True)
    elif args.workload == "serve" and args.impl != "reference":
        print(json.dumps(run_serve(args)), flush=True)
    elif args.workload == "c3" and args.impl != "reference":
        print(json.dumps(run_c3(args)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
