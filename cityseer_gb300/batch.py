"""Batched persistent form: many graphs, thresholds and modes in one persistent launch.

Every (job, source) pair is an item of one device queue that the warps of a single persistent
launch (`batch_kernel`) drain.  Small and large graphs share the GPU, so there is no per-graph
launch tail and no per-graph host synchronisation.  The whole enqueue (resets, launch, threshold
prefixes) is CUDA-graph capturable: `Batch.capture()` records it once, `Batch.replay()` re-runs it.
The schedule -- band width per job and the register budget -- comes from `autotune`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native, autotune, centrality
from .centrality import CentralitySegmentResult, CentralityShortestResult, prepare_source_sampling
from .common import WALKING_SPEED, pair_distances_betas_time

MODES = {"shortest": 0, "segment": 1}


class Batch:
    """jobs: sequence of dicts with keys ns, mode ('shortest' | 'segment'), distances, and optional
    speed_m_s, tolerance, compute_closeness, compute_betweenness, source_indices."""

    def __init__(self, jobs, cap: int = 0, max_slots: int = 0, tune: bool = False, fuse: bool = False):
        """fuse: a shortest-path job and a segment job on the same graph, thresholds, flags and
        sources become one job of mode 3 (one search per source feeds both).  Off by default: on
        the 96-graph workload the fused job ran slower than the two jobs apart, since the fused
        per-source code (both accumulations) misses the instruction caches more than it saves in
        searches.  Jobs run grouped by mode, one launch of that mode's kernel per group."""
        self.lib = _native.load()
        self.jobs = []
        structs = [_native.BatchJob() for _ in jobs]
        variants = []
        max_reach = 1
        for j, spec in enumerate(jobs):
            ns = spec["ns"]
            mode = MODES[spec.get("mode", "shortest")]
            speed = float(spec.get("speed_m_s", WALKING_SPEED))
            d, b, s = pair_distances_betas_time(speed, distances=spec["distances"])
            if len(d) > _native.MAX_K:
                raise ValueError("a batch job takes at most 16 thresholds")
            csr = centrality._primal_csr(ns)
            if mode == 1 and csr.has_missing_reverse:
                raise ValueError("Edge not found")
            dev = csr.device
            if mode == 0:
                sp = prepare_source_sampling(ns, None, None, None, spec.get("source_indices"))
                proc = sp.process
                wt, el = sp.src_wt, sp.eligible
            else:
                a = ns.arrays()
                idx = ns._node_index_array()
                proc = idx[a["live"][idx] == 1].astype(np.int32)
                wt = np.zeros(max(csr.n_bound, 1), np.float32)
                el = np.zeros(max(csr.n_bound, 1), np.uint8)
                sp = None
            tuned = autotune.lookup(ns, csr, spec.get("mode", "shortest"), d, s, speed) if not tune else \
                autotune.tune(ns, spec.get("mode", "shortest"), spec["distances"], speed)
            variants.append(tuned["variant"])
            max_reach = max(max_reach, centrality.estimate_reach(ns, csr, speed, max(s)))
            nrows = 7 if mode == 0 else 4
            out = torch.zeros((nrows, len(d), csr.n_bound), dtype=torch.float64, device=dev)
            closeness = bool(spec.get("compute_closeness", True))
            betweenness = bool(spec.get("compute_betweenness", True))
            bucket = torch.zeros((3, len(d), csr.n_bound), dtype=torch.float64, device=dev) \
                if (mode == 0 and closeness) else None
            keep = [torch.from_numpy(np.ascontiguousarray(proc)).to(dev), torch.from_numpy(wt).to(dev),
                    torch.from_numpy(el).to(dev)]
            jb = structs[j]
            jb.g = csr.struct(speed)
            jb.mode = mode
            jb.k = len(d)
            for i, (dd, bb, ss) in enumerate(zip(d, b, s)):
                jb.distances[i] = dd
                jb.betas[i] = bb
                jb.seconds[i] = ss
            jb.speed_m_s = speed
            jb.tolerance = centrality.validate_tolerance(spec.get("tolerance"))
            jb.delta_seconds = tuned["delta"]
            jb.compute_closeness = int(closeness)
            jb.compute_betweenness = int(betweenness)
            jb.n_sources = len(proc)
            jb.sources = keep[0].data_ptr() if len(proc) else None
            jb.src_wt = keep[1].data_ptr()
            jb.eligible = keep[2].data_ptr()
            jb.out = out.data_ptr()
            jb.bucket = bucket.data_ptr() if bucket is not None else None
            self.jobs.append(dict(ns=ns, csr=csr, mode=mode, d=d, out=out, bucket=bucket, keep=keep, sp=sp,
                                  closeness=closeness, betweenness=betweenness, proc=np.asarray(proc),
                                  speed=speed, tol=jb.tolerance))
        # fusion: pair each segment job with a matching shortest-path job
        table = []
        used = set()
        if fuse:
            short = {}
            for j, jb in enumerate(self.jobs):
                if jb["mode"] == 0:
                    short.setdefault(self._fuse_key(jb), []).append(j)
            for j, jb in enumerate(self.jobs):
                if jb["mode"] != 1:
                    continue
                for cand in short.get(self._fuse_key(jb), []):
                    if cand in used or not np.array_equal(self.jobs[cand]["proc"], jb["proc"]):
                        continue
                    st = structs[cand]
                    st.mode = 3
                    st.out2 = jb["out"].data_ptr()
                    used.update((cand, j))
                    jb["fused_with"] = cand
                    break
        for j, st in enumerate(structs):
            if j in used and self.jobs[j]["mode"] == 1:
                continue
            table.append(st)
        table.sort(key=lambda st: {0: 0, 1: 1, 3: 2}[st.mode])  # one launch per mode group
        self.n_fused = sum(1 for jb in self.jobs if "fused_with" in jb)
        self.table = (_native.BatchJob * len(table))(*table)
        n = C.c_int64()
        _native.check(self.lib.cs_batch_prepare(self.table, len(table), C.byref(n)), "cs_batch_prepare")
        self.n_items = n.value
        dev = self.jobs[0]["csr"].device
        raw = bytes(memoryview(self.table).cast("B"))
        self.table_dev = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(dev)
        plan = _native.Plan()
        plan.variant = max(set(variants), key=variants.count)
        if cap <= 0:
            cap = int(max(1024, -(-int(max_reach * 1.3) // 256) * 256))
        _native.check(self.lib.cs_batch_plan(self.table, len(self.table), cap, max_slots,
                                             centrality._mem_budget(dev), C.byref(plan)), "cs_batch_plan")
        self.plan = plan
        from .device import Workspace

        self.ws = Workspace(plan, plan.n_bound, dev)
        self.graph = None

    @staticmethod
    def _fuse_key(jb):
        return (id(jb["ns"]), tuple(jb["d"]), jb["speed"], jb["tol"], jb["closeness"], jb["betweenness"])

    def run(self, async_: bool = False, stream=None) -> None:
        """Enqueues the whole batch; outputs must be zero (fresh Batch, or zero_outputs())."""
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        rc = self.lib.cs_batch_run(self.table, self.table_dev.data_ptr(), len(self.table), C.byref(self.plan),
                                   self.ws.ptr, self.ws.nbytes, _native.CS_BATCH_ASYNC if async_ else 0, st)
        if rc != _native.CS_OK:
            self.ws.init(st)
            for jb in self.jobs:
                if jb["bucket"] is not None:
                    jb["bucket"].zero_()
        _native.check(rc, "cs_batch_run")

    def zero_outputs(self) -> None:
        for jb in self.jobs:
            jb["out"].zero_()

    def capture(self) -> None:
        """Records zero-outputs + the batch launch as one CUDA graph."""
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                self.zero_outputs()
                self.run(async_=True, stream=side.cuda_stream)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = g

    def replay(self, check: bool = True) -> None:
        """Re-runs the captured batch.  With check, reads the status word afterwards and, when a
        source overflowed its slot's capacity (the captured form cannot retry in-call), re-runs the
        batch synchronously, which retries those sources at full capacity."""
        self.graph.replay()
        if check:
            overflowed, _ = self.status()
            if overflowed > 0:
                self.ws.init()
                self.zero_outputs()
                self.run()

    def status(self) -> tuple[int, int]:
        """(overflowed items, sources done) of the last launch; synchronises."""
        a, b = C.c_int64(), C.c_int64()
        _native.check(self.lib.cs_batch_status(self.ws.ptr, C.byref(a), C.byref(b),
                                               torch.cuda.current_stream().cuda_stream), "cs_batch_status")
        return a.value, b.value

    def results(self):
        """Each job's result object, as its plain call returns it, except that the batched launch does
        not count reachability_totals (left empty) for jobs with source subsets."""
        out = []
        for jb in self.jobs:
            ns = jb["ns"]
            data = jb["out"].cpu().numpy()
            if jb["mode"] == 0:
                sp = jb["sp"]
                if jb["betweenness"] and sp.is_source_indexed and sp.n_sources > 0:
                    sc = sp.n_live / sp.n_sources
                    if sc != 1.0:
                        idx = ns._node_index_array()
                        data[5][:, idx] *= sc
                        data[6][:, idx] *= sc
                res = CentralityShortestResult(jb["d"], ns.node_keys_py(), ns._node_index_array(), data)
                if sp.is_source_indexed:
                    res.sampled_source_count = sp.sampled_count
            else:
                res = CentralitySegmentResult(jb["d"], ns.node_keys_py(), ns._node_index_array(), data)
            out.append(res)
        return out
