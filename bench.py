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

    from cityseer_gb300 import common

    d, b, s = common.pair_distances_betas_time(1.33333, distances=dists)
    og = oracle.OracleGraph(ns)
    nthreads = nthreads or (os.cpu_count() or 1)
    plan = oracle.all_sources_plan(ns)
    allsrc = plan["sources"]

    def run(count):
        idx = np.linspace(0, len(allsrc) - 1, count).astype(np.int64)
        pl = dict(plan)
        pl["sources"] = allsrc[idx]
        t0 = time.perf_counter()
        oracle.centrality_shortest(og, d, b, s, plan=pl, nthreads=nthreads)
        return time.perf_counter() - t0

    probe = max(nthreads * 2, 32)
    tp = run(probe)
    count = int(min(n_total, max(probe, probe * target_seconds / max(tp, 1e-6))))
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


def traffic_ratio():
    """DRAM bytes per algorithmic byte of primal_kernel, from the committed ncu summary."""
    p = ROOT / "profiles" / "primal_kernel_lattice160_shortest.md"
    try:
        for line in p.read_text().splitlines():
            if line.startswith("traffic_per_alg_byte:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def flush_l2(buf):
    buf.add_(1.0)


def run_reference(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return
    ns, dists = build_workload(args.side)
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
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "nodes": n, "distances": dists},
        "cpu_baseline": {k: times[-1][k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    t_max = step_s
    if ws > 1:
        tt = torch.tensor([step_s], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_max = float(tt.item())
    n_src = len(sp.process)
    value = ws * n_src / t_max
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
        "traffic_note": "DRAM bytes per launch scaled from the 160x160 ncu capture "
                        "(profiles/primal_kernel_lattice160_shortest.md) by algorithmic bytes",
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
    e2e_v = ws * n_src / float(np.mean(e2e_times)) if e2e_times else None
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
        "dtype": "f32",
        "data": "synthetic (seeded jittered lattice, see cityseer_gb300/synth.py)",
        "config": {
            "workload": WORKLOAD,
            "nodes": n_nodes,
            "directed_edges": int(csr.m),
            "distances": d,
            "sources_per_step": n_src,
            "l2": "flushed between timed steps (256 MB write)",
            "parallelism": f"replicas x{ws}",
            "slots": int(wsp.plan.n_slots),
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
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(ns, dists, n_nodes, args.cpu_seconds).items()
                                if k != "seconds"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


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
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
