"""Served form: continuous batching of centrality and isochrone queries over device-resident graphs.

A `Server` keeps every graph's CSR (primal, and dual for simplest-path queries) in HBM.  Clients
`submit()` queries from any thread; one serving thread runs the loop:

  admit   pending queries enter in arrival order while their device state (accumulator rows,
          threshold buckets, source weights) fits the HBM budget;
  fold    admitted queries are cut into chunks of sources and folded into waves: each wave is ONE
          persistent batch launch whose job table holds a chunk of every query in it, each with its
          own graph, thresholds and outputs.  Shortest-path and segment queries share the primal
          waves (cs_batch_run); simplest-path queries share the dual waves (cs_dual_batch_run);
  overlap two waves of each kind are in flight at once, on their own streams and workspaces, so the
          next wave's blocks start on SMs as the current wave's tail drains, and a query that
          arrives while waves run joins the next wave (it never waits for a whole queue to empty);
  retire  a finished wave's chunks are credited to their queries; sources that overflowed their
          slot's capacity (or, for simplest paths, whose replay disagreed with the search) are run
          again at once as a synchronous batch, which redoes them at growing capacities and with
          the exact heap search; a query whose sources are all done is complete.

Small queries go first within a wave (then by age; queries waiting longer than `age_ms` jump
ahead), and large ones fill the rest of each wave's source budget, so a 1-source query never waits
behind an 8192-source one.  A query is in at most one wave at a time, so its rows and buckets have
one writer.  Isochrone (tree) queries run on a side thread and stream of their own.

Semantics of a query equal the plain call with `source_indices=sources` (source-indexed sums,
betweenness scaled by n_live / n_sources on the host), so a query's result is the same whether it
ran alone or in a mix, up to float summation order.
"""
from __future__ import annotations

import ctypes as C
import queue
import threading
import time
from dataclasses import dataclass
from typing import Sequence

import numpy as np
import torch

from . import _native, autotune, centrality, dual
from .centrality import TIE_EPSILON, CentralitySegmentResult, CentralityShortestResult, CentralitySimplestResult
from .common import WALKING_SPEED, pair_distances_betas_time

PRIMAL_MODES = {"shortest": 0, "segment": 1}
WAVE_MODES = ("shortest", "segment", "simplest")


@dataclass
class Query:
    graph: int
    sources: Sequence[int]
    distances: Sequence[int]
    mode: str = "shortest"          # shortest | segment | simplest (dual graph) | isochrone
    compute_closeness: bool = True
    compute_betweenness: bool = True


class Ticket:
    """Handle of a submitted query: completion, timings and the result."""

    def __init__(self, qid: int, query: Query, t_arrival: float):
        self.id = qid
        self.query = query
        self.kind = "dual" if query.mode == "simplest" else "primal"
        self.t_arrival = t_arrival
        self.t_admit: float | None = None
        self.t_done: float | None = None
        self.error: BaseException | None = None
        self._ev = threading.Event()
        self.rows: torch.Tensor | None = None     # [M][K][node_bound] f64 on the device
        self.tree = None                           # isochrone: (counts, nodes, agg_seconds, preds)
        # wave state
        self.total = 0
        self.next_off = 0
        self.done_sources = 0
        self.in_flight = False
        self.cancelled = False
        self.nbytes = 0
        self._keep: list = []
        self._job = None
        self._src_host: np.ndarray | None = None
        self._meta: dict = {}

    @property
    def done(self) -> bool:
        return self._ev.is_set()

    def wait(self, timeout: float | None = None) -> bool:
        return self._ev.wait(timeout)

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.t_arrival

    def _finish(self, err: BaseException | None = None):
        self.t_done = time.perf_counter()
        self.error = err
        self._ev.set()

    def result(self, timeout: float | None = None):
        """The result object of the plain call (host copies of the rows)."""
        if not self._ev.wait(timeout):
            raise TimeoutError(f"query {self.id} not done")
        if self.error is not None:
            raise self.error
        m = self._meta
        if self.query.mode == "isochrone":
            return self.tree
        data = self.rows.cpu().numpy()
        ns = m["ns"]
        idx = np.asarray(ns.node_indices(), np.int64)
        if self.query.compute_betweenness and m["n_sources"] > 0:
            sc = m["n_live"] / m["n_sources"]
            if sc != 1.0:
                for r in m["betw_rows"]:
                    data[r][:, idx] *= sc
        cls = {"shortest": CentralityShortestResult, "segment": CentralitySegmentResult,
               "simplest": CentralitySimplestResult}[self.query.mode]
        res = cls(m["d"], ns.node_keys_py(), ns.node_indices(), data)
        if self.query.mode != "segment":
            res.sampled_source_count = m["n_sources"]
        return res

    def release(self) -> None:
        """Drops the device rows (the server frees their budget when it next admits)."""
        self.rows = None
        self._keep = []


class _PinnedRing:
    """Pinned host staging for source lists: one host->device copy per query without pinning or
    synchronising per query.  A region is reused only after the copy that read it has completed."""

    def __init__(self, n_int32: int = 1 << 24):
        self.buf = torch.empty(n_int32, dtype=torch.int32).pin_memory()
        self.np = self.buf.numpy()
        self.n = n_int32
        self.head = 0
        self.pending: list = []   # (start, end, event)

    def stage(self, src: np.ndarray, dev: torch.device, stream) -> torch.Tensor:
        n = len(src)
        out = torch.empty(n, dtype=torch.int32, device=dev)
        if n == 0:
            return out
        if n > self.n:
            return torch.from_numpy(src.astype(np.int32)).to(dev)
        if self.head + n > self.n:
            self.head = 0
        lo, hi = self.head, self.head + n
        keep = []
        for a, b, ev in self.pending:
            if ev.query():
                continue  # that copy is done: its region is free
            if a < hi and lo < b:
                ev.synchronize()
            else:
                keep.append((a, b, ev))
        self.np[lo:hi] = src
        out.copy_(self.buf[lo:hi], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(stream)
        keep.append((lo, hi, ev))
        self.pending = keep
        self.head = hi
        return out


class _Lane:
    def __init__(self, dev: torch.device, max_jobs: int, job_bytes: int, priority: int = 0):
        self.stream = torch.cuda.Stream(device=dev, priority=priority)
        self.ws = None
        self.table_host = torch.empty(max_jobs * job_bytes, dtype=torch.uint8).pin_memory()
        self.table_dev = torch.empty(max_jobs * job_bytes, dtype=torch.uint8, device=dev)
        self.table = None
        self.event = torch.cuda.Event(enable_timing=True)
        self.start = torch.cuda.Event(enable_timing=True)
        self.chunks: list = []
        self.idle = True
        self.rerun = None        # helper thread re-running a wave's listed items
        self.rerun_error = None


class _Kind:
    """Wave machinery of one search kind: 'primal' (shortest and segment jobs, cs_batch_*) or
    'dual' (simplest-path jobs, cs_dual_batch_*)."""

    def __init__(self, name: str, lib, job_cls, plan, ws_factory, dev, max_jobs: int):
        self.name = name
        self.job_cls = job_cls
        self.job_bytes = C.sizeof(job_cls)
        self.plan = plan
        if name == "primal":
            self.prepare, self.run, self.failed = lib.cs_batch_prepare, lib.cs_batch_run, lib.cs_batch_failed
        else:
            self.prepare, self.run, self.failed = (lib.cs_dual_batch_prepare, lib.cs_dual_batch_run,
                                                   lib.cs_dual_batch_failed)
        self.lanes = []
        for _ in range(2):
            # shortest-path waves take freed SM slots ahead of the (longer) simplest-path waves
            lane = _Lane(dev, max_jobs, self.job_bytes, priority=-1 if name == "primal" else 0)
            lane.ws = ws_factory(lane.stream.cuda_stream)
            self.lanes.append(lane)
        self.wave_cost = float(plan.n_slots)
        self.waves = 0
        self.items = 0
        self.jobs = 0
        self.gpu_ms: list[float] = []


class Server:
    """Continuous-batching server over device-resident graphs.

    graphs: {graph id: primal NetworkStructure}; duals: {graph id: dual NetworkStructure} for
    simplest-path queries.  max_distance / max_thresholds bound the queries the slot geometry is
    planned for.  wave_cost is the source budget of one wave in units of a max-distance source
    (default: one per search slot).  primal_hbm_frac / dual_hbm_frac: the share of the free HBM at
    start that each of the two primal / dual lanes' workspaces may take; dual_slots caps the dual
    lanes' slots."""

    def __init__(self, graphs: dict, duals: dict | None = None, *, speed_m_s: float = WALKING_SPEED,
                 max_distance: int = 5000, max_thresholds: int = 4, hbm_budget_bytes: int | None = None,
                 wave_cost: float | None = None, max_jobs_per_wave: int = 512, age_ms: float = 100.0,
                 keep_results: bool = True, dual_slots: int = 608, cap: int = 0, max_slots: int = 0,
                 primal_hbm_frac: float = 0.12, dual_hbm_frac: float = 0.17):
        if not torch.cuda.is_available():
            raise RuntimeError("the served form needs a CUDA device")
        self.lib = _native.load()
        self.device = torch.device("cuda", torch.cuda.current_device())
        dev = self.device
        self.speed = float(speed_m_s)
        self.max_k = int(max_thresholds)
        self.keep_results = keep_results
        self.age = age_ms / 1000.0
        self.graphs = dict(graphs)
        self.duals = dict(duals or {})
        self.max_jobs = int(max_jobs_per_wave)
        _, _, secs = pair_distances_betas_time(self.speed, distances=[int(max_distance)])
        self.max_seconds = int(secs[0])
        self.max_distance = int(max_distance)
        # ---- resident graphs (primal and dual): CSR, per-speed structs, host metadata
        self.csr = {g: centrality._primal_csr(ns) for g, ns in self.graphs.items()}
        self.gstruct = {g: c.struct(self.speed) for g, c in self.csr.items()}
        self.dcsr = {g: dual.dual_csr(ns) for g, ns in self.duals.items()}
        self.dstruct = {g: c.struct(self.speed) for g, c in self.dcsr.items()}
        self.meta = {("primal", g): self._graph_meta(ns, self.csr[g].n_bound) for g, ns in self.graphs.items()}
        self.meta.update({("dual", g): self._graph_meta(ns, self.dcsr[g].n_bound) for g, ns in self.duals.items()})
        self.zeros_w = {g: torch.zeros(max(1, c.n_bound), dtype=torch.float32, device=dev)
                        for g, c in self.csr.items()}
        self.zeros_e = {g: torch.zeros(max(1, c.n_bound), dtype=torch.uint8, device=dev)
                        for g, c in self.csr.items()}
        self.tuned = {}
        self.kinds: dict[str, _Kind] = {}
        # workspace budgets from the free HBM at start: about a quarter for the two primal lanes,
        # a third for the two dual lanes (the dual's per-slot scratch is 3x the primal's per node),
        # and half of what is left for the queries' rows
        free0, _ = torch.cuda.mem_get_info(dev)
        from .device import Workspace

        if self.graphs:
            reach = max(centrality.estimate_reach(ns, self.csr[g], self.speed, self.max_seconds)
                        for g, ns in self.graphs.items())
            self.cap = int(cap) if cap > 0 else int(max(1024, -(-int(reach * 1.3) // 256) * 256))
            dummy = (_native.BatchJob * len(self.graphs))()
            for i, g in enumerate(self.graphs):
                dummy[i].g = self.gstruct[g]
                dummy[i].mode = 0
                dummy[i].k = self.max_k
                dummy[i].speed_m_s = self.speed
                dummy[i].out = 1
                dummy[i].compute_closeness = 0
            plan = _native.Plan()
            _native.check(self.lib.cs_batch_plan(dummy, len(self.graphs), self.cap, max_slots,
                                                 int(free0 * primal_hbm_frac),
                                                 C.byref(plan)), "cs_batch_plan")
            self.kinds["primal"] = _Kind("primal", self.lib, _native.BatchJob, plan,
                                         lambda st, pl=plan: Workspace(pl, pl.n_bound, dev, stream=st), dev,
                                         self.max_jobs)
        else:
            self.cap = 0
        if self.duals:
            dcap = int(cap) if cap > 0 else max(dual.estimate_states(ns, self.speed, self.max_seconds)
                                                for ns in self.duals.values())
            djobs = (_native.DualBatchJob * len(self.duals))()
            for i, g in enumerate(self.duals):
                djobs[i].g = self.dstruct[g]
                djobs[i].k = self.max_k
                djobs[i].out = 1
                djobs[i].compute_closeness = 0
            dplan = _native.Plan()
            slots = min(dual_slots, max_slots) if max_slots > 0 else dual_slots
            _native.check(self.lib.cs_dual_batch_plan(djobs, len(self.duals), dcap, slots, int(free0 * dual_hbm_frac),
                                                      C.byref(dplan)), "cs_dual_batch_plan")
            self.kinds["dual"] = _Kind("dual", self.lib, _native.DualBatchJob, dplan,
                                       lambda st, pl=dplan: dual.DualWorkspace(pl, pl.n_bound, dev, stream=st), dev,
                                       self.max_jobs)
        if wave_cost:
            for kd in self.kinds.values():
                kd.wave_cost = float(wave_cost)
        self.side_stream = torch.cuda.Stream(device=dev)
        torch.cuda.synchronize()
        free, _ = torch.cuda.mem_get_info(dev)
        self.budget = int(hbm_budget_bytes) if hbm_budget_bytes else int(free * 0.5)
        self.in_use = 0
        # ---- queues and threads
        self._pending: list[Ticket] = []
        self._active: list[Ticket] = []
        self._staging = 0
        self._holding: list[Ticket] = []       # done, rows still on the device
        self._side_q: queue.Queue = queue.Queue()
        self._lock = threading.Lock()
        self._cv = threading.Condition(self._lock)
        self._next_id = 0
        self._stop = False
        self._threads: list[threading.Thread] = []
        # admission work (zero fills, source plan) goes ahead of pending wave blocks
        self.admit_stream = torch.cuda.Stream(device=dev, priority=-2)
        self.ring = _PinnedRing()
        self.admit_event = None
        self.host_s = {"admit": 0.0, "launch": 0.0, "retire": 0.0}

    def _graph_meta(self, ns, nb: int) -> dict:
        a = ns.arrays()
        idx = np.asarray(ns.node_indices(), np.int64)
        return dict(ns=ns, nb=nb, exists=a["node_exists"].astype(bool), n_live=int(a["live"][idx].sum()),
                    weight=torch.from_numpy(np.ascontiguousarray(a["weight"][:nb], dtype=np.float32)).to(self.device))

    # ------------------------------------------------------------------ client side
    def submit(self, q: Query, t_arrival: float | None = None) -> Ticket:
        if q.mode not in WAVE_MODES and q.mode != "isochrone":
            raise ValueError(f"unknown query mode {q.mode!r}")
        graphs = self.duals if q.mode == "simplest" else self.graphs
        if q.graph not in graphs:
            raise ValueError(f"graph {q.graph} is not resident for {q.mode} queries")
        if len(q.distances) < 1 or len(q.distances) > self.max_k:
            raise ValueError(f"a query takes 1 to {self.max_k} thresholds")
        if max(q.distances) > self.max_distance and q.mode in WAVE_MODES:
            raise ValueError(f"thresholds above {self.max_distance} m exceed the planned capacity")
        with self._cv:
            t = Ticket(self._next_id, q, time.perf_counter() if t_arrival is None else t_arrival)
            self._next_id += 1
            if q.mode in WAVE_MODES:
                self._pending.append(t)
                self._cv.notify_all()
            else:
                self._side_q.put(t)
        return t

    def start(self) -> "Server":
        self._stop = False
        self._threads = [threading.Thread(target=self._loop, name="cs-serve", daemon=True),
                         threading.Thread(target=self._side_loop, name="cs-serve-side", daemon=True)]
        for th in self._threads:
            th.start()
        return self

    def stop(self, drain: bool = True) -> None:
        if drain:
            self.drain()
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        self._side_q.put(None)
        for th in self._threads:
            th.join()
        self._threads = []

    def _lanes(self):
        return [ln for kd in self.kinds.values() for ln in kd.lanes]

    def drain(self, timeout: float | None = None) -> None:
        t0 = time.perf_counter()
        while True:
            with self._lock:
                busy = bool(self._pending or self._active or self._staging) or \
                    any(not ln.idle for ln in self._lanes())
            if not busy and self._side_q.unfinished_tasks == 0:
                return
            if timeout is not None and time.perf_counter() - t0 > timeout:
                raise TimeoutError("server did not drain")
            time.sleep(0.0005)

    def cancel(self) -> int:
        """Drops the queries not yet admitted and stops the admitted ones at their next chunk
        boundary; all of them finish with an error.  Returns how many were dropped before
        admission."""
        err = RuntimeError("query cancelled")
        with self._lock:
            dropped = self._pending[:]
            self._pending.clear()
            for t in self._active:
                t.cancelled = True
        side = []
        while True:
            try:
                t = self._side_q.get_nowait()
            except queue.Empty:
                break
            if t is None:
                self._side_q.put(None)
                self._side_q.task_done()
                break
            side.append(t)
            self._side_q.task_done()
        for t in dropped + side:
            t._finish(err)
        return len(dropped) + len(side)

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    # ------------------------------------------------------------------ serving loop
    def _loop(self):
        try:
            torch.cuda.set_device(self.device)
            while True:
                with self._cv:
                    if self._stop and not self._pending and not self._active and not self._staging and \
                            all(ln.idle for ln in self._lanes()):
                        return
                t0 = time.perf_counter()
                progressed = self._retire()
                t1 = time.perf_counter()
                progressed |= self._admit()
                t2 = time.perf_counter()
                for kd in self.kinds.values():
                    for lane in kd.lanes:
                        if lane.idle and self._launch(kd, lane):
                            progressed = True
                t3 = time.perf_counter()
                if progressed:
                    self.host_s["retire"] += t1 - t0
                    self.host_s["admit"] += t2 - t1
                    self.host_s["launch"] += t3 - t2
                else:
                    with self._cv:
                        self._cv.wait(timeout=0.0002)
        except BaseException as e:  # fail every open query rather than hang the clients
            with self._lock:
                for t in self._pending + self._active:
                    t._finish(e)
                self._pending.clear()
                self._active.clear()
            for lane in self._lanes():
                lane.idle = True
            raise

    def _need_bytes(self, t: Ticket) -> int:
        q = t.query
        nb = self.meta[(t.kind, q.graph)]["nb"]
        k = len(q.distances)
        rows = {"shortest": 7, "segment": 4, "simplest": 4}[q.mode]
        buck = 3 * k * nb * 8 if (q.mode != "segment" and q.compute_closeness) else 0
        return rows * k * nb * 8 + buck + 5 * nb + 4 * len(q.sources)

    def _admit(self) -> bool:
        with self._lock:
            # queries whose rows the client released give their budget back
            keep = []
            for t in self._holding:
                if t.rows is None:
                    self.in_use -= t.nbytes
                else:
                    keep.append(t)
            self._holding = keep
            take = []
            while self._pending:
                t = self._pending[0]
                if t.kind not in self.kinds:
                    self._pending.pop(0)
                    t._finish(ValueError(f"no resident graphs for {t.query.mode} queries"))
                    continue
                need = self._need_bytes(t)
                if self.in_use + need > self.budget and (self.in_use > 0 or take):
                    break
                self._pending.pop(0)
                self.in_use += need
                t.nbytes = need
                take.append(t)
            self._staging += len(take)  # admitted, not yet active: drain() must still wait for them
        if not take:
            return False
        with torch.cuda.stream(self.admit_stream):
            for t in take:
                try:
                    self._setup(t)
                except BaseException as e:
                    with self._lock:
                        self.in_use -= t.nbytes
                        self._staging -= 1
                    t._finish(e)
                    continue
                t.t_admit = time.perf_counter()
                with self._lock:
                    self._active.append(t)
                    self._staging -= 1
        self.admit_event = torch.cuda.Event()
        self.admit_event.record(self.admit_stream)
        return True

    def _setup(self, t: Ticket) -> None:
        q = t.query
        g = q.graph
        m = self.meta[(t.kind, g)]
        ns, nb = m["ns"], m["nb"]
        closeness, betweenness = bool(q.compute_closeness), bool(q.compute_betweenness)
        if not closeness and not betweenness:
            raise ValueError(
                "Either or both closeness and betweenness flags is required, but both parameters are False.")
        d, b, s = pair_distances_betas_time(self.speed, distances=list(q.distances))
        src = np.asarray(q.sources, np.int64).reshape(-1)
        exists = m["exists"]
        if len(src):
            bad = (src < 0) | (src >= nb)
            bad |= ~exists[np.clip(src, 0, nb - 1)]
            if bad.any():
                raise ValueError(f"node index {int(src[bad][0])} does not exist in the graph")
        dev = self.device
        # no host synchronisation here: persistent waves hold every SM, so a blocking call would
        # wait for the running wave to drain
        src_t = self.ring.stage(src.astype(np.int32), dev, self.admit_stream)
        if q.mode == "segment":
            wt_t, el_t = self.zeros_w[g], self.zeros_e[g]
        else:
            # source-indexed plan (prepare_source_sampling with source_indices), built on the device
            wt_t = torch.empty(nb, dtype=torch.float32, device=dev)
            el_t = torch.empty(nb, dtype=torch.uint8, device=dev)
            _native.check(self.lib.cs_source_weights(src_t.data_ptr() if len(src) else None, len(src),
                                                     m["weight"].data_ptr(), nb, wt_t.data_ptr(), el_t.data_ptr(),
                                                     self.admit_stream.cuda_stream), "cs_source_weights")
        rows = {"shortest": 7, "segment": 4, "simplest": 4}[q.mode]
        out = torch.zeros((rows, len(d), nb), dtype=torch.float64, device=dev)
        bucket = torch.zeros((3, len(d), nb), dtype=torch.float64, device=dev) \
            if (q.mode != "segment" and closeness) else None
        if t.kind == "primal":
            tkey = (g, q.mode, int(max(s)), len(d))
            tuned = self.tuned.get(tkey)
            if tuned is None:
                tuned = self.tuned[tkey] = autotune.lookup(ns, self.csr[g], q.mode, d, s, self.speed)
            jb = _native.BatchJob()
            jb.g = self.gstruct[g]
            jb.mode = PRIMAL_MODES[q.mode]
            jb.k = len(d)
            for i, (dd, bb, ss) in enumerate(zip(d, b, s)):
                jb.distances[i] = dd
                jb.betas[i] = bb
                jb.seconds[i] = ss
            jb.speed_m_s = self.speed
            jb.delta_seconds = tuned["delta"]
            betw_rows = (5, 6) if q.mode == "shortest" else (3,)
        else:
            jb = _native.DualBatchJob()
            jb.g = self.dstruct[g]
            jb.k = len(d)
            for i, ss in enumerate(s):
                jb.seconds[i] = ss
            jb.angular_scaling_unit = 180.0
            jb.farness_scaling_offset = 1.0
            betw_rows = (3,)
        jb.tolerance = float(TIE_EPSILON)
        jb.compute_closeness = int(closeness)
        jb.compute_betweenness = int(betweenness)
        jb.src_wt = wt_t.data_ptr()
        jb.eligible = el_t.data_ptr()
        jb.out = out.data_ptr()
        jb.bucket = bucket.data_ptr() if bucket is not None else None
        t._job = jb
        t._keep = [src_t, wt_t, el_t, bucket]
        t._src_host = src.astype(np.int32)
        t.rows = out
        t.total = len(src)
        t.next_off = 0
        t.done_sources = 0
        t._meta = dict(ns=ns, d=d, n_sources=len(src), n_live=m["n_live"], betw_rows=betw_rows,
                       cost=max(0.02, (max(d) / self.max_distance) ** 2))

    def _launch(self, kd: _Kind, lane: _Lane) -> bool:
        now = time.perf_counter()
        with self._lock:
            cand = [t for t in self._active if t.kind == kd.name and not t.in_flight and t.next_off < t.total
                    and not t.cancelled]
        if not cand:
            return False
        cand.sort(key=lambda t: (0 if now - t.t_arrival > self.age else 1, t.total - t.next_off, t.t_arrival))
        budget = kd.wave_cost
        chunks = []
        for t in cand:
            if budget <= 0 or len(chunks) >= self.max_jobs:
                break
            c = t._meta["cost"]
            n = min(t.total - t.next_off, max(1, int(budget / c)))
            chunks.append((t, t.next_off, n))
            budget -= n * c
        if kd.name == "primal":
            chunks.sort(key=lambda c: c[0]._job.mode)  # one launch per mode group
        table = (kd.job_cls * len(chunks))()
        for j, (t, off, n) in enumerate(chunks):
            C.memmove(C.byref(table[j]), C.byref(t._job), kd.job_bytes)
            table[j].sources = t._keep[0].data_ptr() + 4 * off
            table[j].n_sources = n
        n_items = C.c_int64()
        _native.check(kd.prepare(table, len(chunks), C.byref(n_items)), "batch prepare")
        nbytes = len(chunks) * kd.job_bytes
        C.memmove(lane.table_host.data_ptr(), C.addressof(table), nbytes)
        if self.admit_event is not None:
            lane.stream.wait_event(self.admit_event)
        lane.start.record(lane.stream)
        with torch.cuda.stream(lane.stream):
            lane.table_dev[:nbytes].copy_(lane.table_host[:nbytes], non_blocking=True)
        rc = kd.run(table, lane.table_dev.data_ptr(), len(chunks), C.byref(kd.plan), lane.ws.ptr, lane.ws.nbytes,
                    _native.CS_BATCH_ASYNC, lane.stream.cuda_stream)
        _native.check(rc, "batch run")
        lane.event.record(lane.stream)
        for t, off, n in chunks:
            t.in_flight = True
            t.next_off = off + n
        lane.table = table
        lane.chunks = chunks
        lane.idle = False
        kd.waves += 1
        kd.items += int(n_items.value)
        kd.jobs += len(chunks)
        return True

    def _retire(self) -> bool:
        progressed = False
        for kd in self.kinds.values():
            for lane in kd.lanes:
                if lane.idle or lane.rerun is not None or not lane.event.query():
                    continue
                kd.gpu_ms.append(lane.start.elapsed_time(lane.event))
                nf = C.c_int64()
                fails = np.zeros(1 << 16, np.int32)
                _native.check(kd.failed(lane.ws.ptr, C.byref(kd.plan), fails.ctypes.data_as(C.POINTER(C.c_int32)),
                                        len(fails), C.byref(nf), lane.stream.cuda_stream), "batch failed list")
                if nf.value > 0:
                    # the listed items run again synchronously on this lane, in a helper thread so
                    # that the loop keeps serving the other lanes; the lane's chunks complete after
                    items = fails[: nf.value] if nf.value <= len(fails) else None
                    lane.rerun = threading.Thread(target=self._rerun_guarded, args=(kd, lane, items), daemon=True)
                    lane.rerun.start()
                    progressed = True
                    continue
                self._finish_lane(lane)
                progressed = True
            for lane in kd.lanes:
                if lane.rerun is not None and not lane.rerun.is_alive():
                    lane.rerun = None
                    err, lane.rerun_error = lane.rerun_error, None
                    if err is not None:
                        raise err
                    self._finish_lane(lane)
                    progressed = True
        # queries without sources complete at admission; cancelled ones leave when not in a wave
        with self._lock:
            empty = [t for t in self._active if t.total == 0 and not t.cancelled]
            gone = [t for t in self._active if t.cancelled and not t.in_flight]
            for t in empty + gone:
                self._active.remove(t)
        for t in empty:
            self._complete(t)
        for t in gone:
            t._keep = []
            t.rows = None
            with self._lock:
                self.in_use -= t.nbytes
            t._finish(RuntimeError("query cancelled"))
        return progressed or bool(empty) or bool(gone)

    def _rerun_guarded(self, kd: _Kind, lane: _Lane, items) -> None:
        try:
            torch.cuda.set_device(self.device)
            self._rerun_failed(kd, lane, items)
        except BaseException as e:
            lane.rerun_error = e

    def _finish_lane(self, lane: _Lane) -> None:
        """Credits a completed wave's chunks to their queries and frees the lane."""
        done = []
        with self._lock:
            for t, off, n in lane.chunks:
                t.done_sources += n
                t.in_flight = False
                if t.done_sources >= t.total:
                    done.append(t)
            for t in done:
                self._active.remove(t)
        for t in done:
            self._complete(t)
        lane.chunks = []
        lane.table = None
        lane.idle = True

    def _complete(self, t: Ticket) -> None:
        t._keep = []
        if self.keep_results:
            with self._lock:
                self._holding.append(t)
        else:
            t.rows = None
            with self._lock:
                self.in_use -= t.nbytes
        t._finish()

    def _rerun_failed(self, kd: _Kind, lane: _Lane, items) -> None:
        """Runs a wave's listed items again as a synchronous batch (overflows at growing
        capacities; disagreeing simplest-path replays with the exact heap search)."""
        if items is None:
            raise _native.NativeError(_native.CS_ERR_CAPACITY, "too many listed sources in one wave")
        table = lane.table
        begins = np.array([table[j].item_begin for j in range(len(lane.chunks))], np.int64)
        per_job: dict[int, list[int]] = {}
        for it in items.tolist():
            j = int(np.searchsorted(begins, it, side="right") - 1)
            per_job.setdefault(j, []).append(it - int(begins[j]))
        jobs = []
        keep = []
        for j, locs in per_job.items():
            t, off, n = lane.chunks[j]
            srcs = t._src_host[off:off + n][np.asarray(sorted(locs), np.int64)]
            st = torch.from_numpy(srcs.astype(np.int32)).to(self.device)
            keep.append(st)
            jb = kd.job_cls()
            C.memmove(C.byref(jb), C.byref(t._job), kd.job_bytes)
            jb.sources = st.data_ptr()
            jb.n_sources = len(srcs)
            jobs.append(jb)
        rt = (kd.job_cls * len(jobs))(*jobs)
        n_items = C.c_int64()
        _native.check(kd.prepare(rt, len(jobs), C.byref(n_items)), "batch prepare")
        raw = torch.frombuffer(bytearray(bytes(memoryview(rt).cast("B"))), dtype=torch.uint8)
        dev_tab = raw.to(self.device)
        torch.cuda.current_stream(self.device).synchronize()
        lane.stream.synchronize()
        rc = kd.run(rt, dev_tab.data_ptr(), len(jobs), C.byref(kd.plan), lane.ws.ptr, lane.ws.nbytes, 0,
                    lane.stream.cuda_stream)
        # the call returns with its closeness-prefix launch still queued on the lane's stream; that
        # kernel reads this job table and writes the queries' rows, which the caller frees as the
        # queries complete: wait for it before the table, the source lists or the rows can go
        lane.stream.synchronize()
        del keep, dev_tab
        if rc != _native.CS_OK:
            lane.ws.init(lane.stream.cuda_stream)
        _native.check(rc, "batch run (listed items)")

    # ------------------------------------------------------------------ side path (trees)
    def _side_loop(self):
        torch.cuda.set_device(self.device)
        while True:
            t = self._side_q.get()
            if t is None:
                self._side_q.task_done()
                return
            try:
                t.t_admit = time.perf_counter()
                with torch.cuda.stream(self.side_stream):
                    self._run_isochrone(t)
                t._finish()
            except BaseException as e:
                t._finish(e)
            finally:
                self._side_q.task_done()

    def _run_isochrone(self, t: Ticket) -> None:
        q = t.query
        ns = self.graphs[q.graph]
        _, _, s = pair_distances_betas_time(self.speed, distances=[int(max(q.distances))])
        counts, nodes, agg, preds = centrality.tree_shortest_raw(ns, [int(x) for x in q.sources], int(s[0]),
                                                                 self.speed)
        t.tree = (counts, nodes, agg, preds)
        t._meta = dict(ns=ns, d=list(q.distances), n_sources=len(q.sources), n_live=0, betw_rows=())

    # ------------------------------------------------------------------ stats
    def stats(self) -> dict:
        out = {"host_s": {k: round(v, 3) for k, v in self.host_s.items()}, "hbm_budget": self.budget,
               "in_use": self.in_use, "cap": self.cap}
        for name, kd in self.kinds.items():
            w = np.asarray(kd.gpu_ms) if kd.gpu_ms else np.zeros(1)
            out[name] = {"waves": kd.waves, "items": kd.items, "jobs": kd.jobs, "slots": int(kd.plan.n_slots),
                         "cap": int(kd.plan.cap), "wave_gpu_ms_mean": float(w.mean()),
                         "wave_gpu_ms_p99": float(np.percentile(w, 99))}
        out["waves"] = sum(kd.waves for kd in self.kinds.values())
        return out


def latency_summary(tickets: Sequence[Ticket], max_sources: int | None = None) -> dict:
    """p50 / p99 / max latency in ms over completed tickets (optionally only small queries)."""
    lat = [t.latency for t in tickets if t.latency is not None and
           (max_sources is None or len(t.query.sources) <= max_sources)]
    if not lat:
        return {"n": 0}
    a = np.asarray(lat) * 1000.0
    return {"n": len(a), "p50_ms": float(np.percentile(a, 50)), "p99_ms": float(np.percentile(a, 99)),
            "max_ms": float(a.max())}
