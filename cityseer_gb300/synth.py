"""Seeded synthetic street networks for tests and benchmarks.

Jittered lattices built the way the reference's ingest would see them
(pysrc/cityseer/tools/io.py:1018-1210): every undirected street becomes two directed edges with the
same edge_idx, lengths are the f64 polyline length cast to f32 (rust/src/graph.rs:774) and
angle_sum is the cumulative turn of the polyline (rust/src/graph.rs:367-379, 857).

Workloads (node counts / thresholds are those of the benchmark configurations):
  lattice_config("c1")  40x40 at 100 m, jitter +-20 m, 15% of streets dropped, d = 500/1000/2000
  lattice_config("c2")  450x450 at 80 m, jitter +-15 m, 10% dropped, 5% of nodes with a diagonal
                        shortcut of length euclid * U(1.0, 1.3), d = 500/1000/2000/5000
  lattice_config("c3")  250x250 at 80 m, jitter +-15 m, 30% of streets curved (3 sub-segments with
                        +-25 degree bearing offsets); the simplest-path workload runs on its dual
Streets are dropped only where the lattice stays connected (a random spanning tree is protected).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .graph import NetworkStructure


@dataclass
class Primal:
    x: np.ndarray                     # f64 [n]
    y: np.ndarray                     # f64 [n]
    u: np.ndarray                     # int [m] undirected street endpoints
    v: np.ndarray
    length: np.ndarray                # f32 [m]
    angle_sum: np.ndarray             # f32 [m]
    geoms: list = field(default_factory=list)  # per street: None (straight) or (k,2) interior vertices
    stretched: np.ndarray | None = None


def _uf_find(parent, a):
    root = a
    while parent[root] != root:
        root = parent[root]
    while parent[a] != root:
        parent[a], a = root, parent[a]
    return root


def _spanning_protect(n, u, v, rng) -> np.ndarray:
    parent = np.arange(n)
    keep = np.zeros(len(u), bool)
    for e in rng.permutation(len(u)):
        a, b = _uf_find(parent, int(u[e])), _uf_find(parent, int(v[e]))
        if a != b:
            parent[a] = b
            keep[e] = True
    return keep


def _turn(ax, ay, bx, by, cx, cy):
    """|turn| in degrees at b for polyline a-b-c (rust/src/graph.rs:336-346), vectorised f64."""
    a1 = np.degrees(np.arctan2(ay - by, ax - bx))
    a2 = np.degrees(np.arctan2(by - cy, bx - cx))
    d = a2 - a1 + 180.0
    r = np.fmod(d, 360.0)
    r = np.where(r < 0, r + 360.0, r)
    out = np.abs(r - 180.0)
    same = ((ax == bx) & (ay == by)) | ((bx == cx) & (by == cy))
    return np.where(same, 0.0, out)


def lattice(side: int, spacing: float, jitter: float, drop: float, seed: int, diag_frac: float = 0.0,
            diag_stretch=(1.0, 1.3), curved_frac: float = 0.0, curve_deg: float = 25.0) -> Primal:
    rng = np.random.default_rng(seed)
    n = side * side
    ii, jj = np.divmod(np.arange(n), side)
    x = jj * spacing + rng.uniform(-jitter, jitter, n)
    y = ii * spacing + rng.uniform(-jitter, jitter, n)
    hu = (ii * side + jj)[jj < side - 1]
    vu = (ii * side + jj)[ii < side - 1]
    u = np.concatenate([hu, vu])
    v = np.concatenate([hu + 1, vu + side])
    keep = _spanning_protect(n, u, v, rng)
    cand = np.nonzero(~keep)[0]
    n_drop = min(len(cand), int(round(drop * len(u))))
    dropped = rng.choice(cand, size=n_drop, replace=False) if n_drop else np.zeros(0, np.int64)
    alive = np.ones(len(u), bool)
    alive[dropped] = False
    u, v = u[alive], v[alive]
    stretched = np.ones(len(u), np.float64)
    if diag_frac > 0:
        nd = int(round(diag_frac * n))
        who = rng.choice(n, size=nd, replace=False)
        wi, wj = np.divmod(who, side)
        di = rng.choice([-1, 1], size=nd)
        dj = rng.choice([-1, 1], size=nd)
        ok = (wi + di >= 0) & (wi + di < side) & (wj + dj >= 0) & (wj + dj < side)
        du = who[ok]
        dv = ((wi + di) * side + (wj + dj))[ok]
        u = np.concatenate([u, du])
        v = np.concatenate([v, dv])
        stretched = np.concatenate([stretched, rng.uniform(diag_stretch[0], diag_stretch[1], len(du))])
    m = len(u)
    geoms: list = [None] * m
    dx = x[v] - x[u]
    dy = y[v] - y[u]
    length64 = np.hypot(dx, dy) * stretched
    angle = np.zeros(m, np.float64)
    if curved_frac > 0:
        cur = np.nonzero(rng.random(m) < curved_frac)[0]
        b0 = np.arctan2(dy[cur], dx[cur])
        L = np.hypot(dx[cur], dy[cur])
        t1 = np.radians(rng.uniform(-curve_deg, curve_deg, len(cur)))
        t2 = np.radians(rng.uniform(-curve_deg, curve_deg, len(cur)))
        p1x = x[u[cur]] + (L / 3) * np.cos(b0 + t1)
        p1y = y[u[cur]] + (L / 3) * np.sin(b0 + t1)
        p2x = x[v[cur]] - (L / 3) * np.cos(b0 - t2)
        p2y = y[v[cur]] - (L / 3) * np.sin(b0 - t2)
        seg = (np.hypot(p1x - x[u[cur]], p1y - y[u[cur]]) + np.hypot(p2x - p1x, p2y - p1y)
               + np.hypot(x[v[cur]] - p2x, y[v[cur]] - p2y))
        length64[cur] = seg
        angle[cur] = (_turn(x[u[cur]], y[u[cur]], p1x, p1y, p2x, p2y)
                      + _turn(p1x, p1y, p2x, p2y, x[v[cur]], y[v[cur]]))
        for q, e in enumerate(cur):
            geoms[e] = np.array([[p1x[q], p1y[q]], [p2x[q], p2y[q]]])
    return Primal(x=x, y=y, u=u, v=v, length=length64.astype(np.float32), angle_sum=angle.astype(np.float32),
                  geoms=geoms, stretched=stretched)


def primal_structure(p: Primal, live: np.ndarray | None = None) -> NetworkStructure:
    """Two directed edges per street, inserted per start node in ascending order (as
    network_structure_from_nx iterates nodes then neighbours)."""
    m = len(p.u)
    src = np.concatenate([p.u, p.v])
    dst = np.concatenate([p.v, p.u])
    street = np.concatenate([np.arange(m), np.arange(m)])
    order = np.lexsort((street, src))
    src, dst, street = src[order], dst[order], street[order]
    length = p.length[street]
    # a curved street's angle_sum is the same read in either direction
    ang = p.angle_sum[street]
    return NetworkStructure.from_arrays(p.x, p.y, src, dst, length, edge_idx=np.zeros(len(src), np.int64),
                                        edge_angle_sum=ang, live=live)


def _half_polylines(p: Primal):
    """Per street: coordinates from each endpoint to the street's midpoint (by length)."""
    out_u, out_v, mids = [], [], []
    for e in range(len(p.u)):
        a = np.array([p.x[p.u[e]], p.y[p.u[e]]])
        b = np.array([p.x[p.v[e]], p.y[p.v[e]]])
        inner = p.geoms[e]
        pts = np.vstack([a, inner, b]) if inner is not None else np.vstack([a, b])
        seg = np.hypot(np.diff(pts[:, 0]), np.diff(pts[:, 1]))
        half = seg.sum() / 2.0
        cum = np.concatenate([[0.0], np.cumsum(seg)])
        k = int(np.searchsorted(cum, half, side="right") - 1)
        k = min(k, len(seg) - 1)
        frac = (half - cum[k]) / seg[k] if seg[k] > 0 else 0.0
        mid = pts[k] + (pts[k + 1] - pts[k]) * frac
        from_u = np.vstack([pts[: k + 1], mid])
        from_v = np.vstack([pts[k + 1:][::-1], mid])
        out_u.append(from_u)
        out_v.append(from_v)
        mids.append(mid)
    return out_u, out_v, np.array(mids)


def _dual_structure_straight(p: Primal) -> NetworkStructure:
    """dual_structure for lattices whose streets are all straight, vectorised: each dual edge a -> b
    through primal node n is the polyline mid_a -> n -> mid_b."""
    x, y = p.x, p.y
    ax, ay = x[p.u], y[p.u]
    bx, by = x[p.v], y[p.v]
    seg = np.hypot(bx - ax, by - ay)
    frac = np.where(seg > 0, (seg / 2.0) / np.where(seg > 0, seg, 1.0), 0.0)
    mx = ax + (bx - ax) * frac
    my = ay + (by - ay) * frac
    m = len(p.u)
    node_of = np.concatenate([p.u, p.v]).astype(np.int64)
    e_of = np.concatenate([np.arange(m), np.arange(m)]).astype(np.int64)
    order = np.lexsort((e_of, node_of))
    node_of, e_of = node_of[order], e_of[order]
    starts = np.flatnonzero(np.r_[True, node_of[1:] != node_of[:-1]])
    counts = np.diff(np.r_[starts, len(node_of)])
    pa, pb = [], []
    for i in range(int(counts.max()) if len(counts) else 0):
        for j in range(i + 1, int(counts.max())):
            sel = counts > j
            pa.append(starts[sel] + i)
            pb.append(starts[sel] + j)
    pa = np.concatenate(pa) if pa else np.zeros(0, np.int64)
    pb = np.concatenate(pb) if pb else np.zeros(0, np.int64)
    ea = np.concatenate([e_of[pa], e_of[pb]])
    eb = np.concatenate([e_of[pb], e_of[pa]])
    nd = np.concatenate([node_of[pa], node_of[pa]])
    nx_, ny_ = x[nd], y[nd]
    s0 = np.hypot(nx_ - mx[ea], ny_ - my[ea])
    s1 = np.hypot(mx[eb] - nx_, my[eb] - ny_)
    lens = (0.0 + s0) + s1
    angs = 0.0 + _turn(mx[ea], my[ea], nx_, ny_, mx[eb], my[eb])
    order = np.lexsort((nd, eb, ea))
    return NetworkStructure.from_arrays(
        mx, my, ea[order], eb[order], lens[order].astype(np.float32), edge_idx=np.zeros(len(ea), np.int64),
        edge_angle_sum=angs[order].astype(np.float32), edge_shared_key=[str(s) for s in nd[order]], is_dual=True)


def dual_structure(p: Primal) -> NetworkStructure:
    """The dual graph as nx_to_dual builds it (pysrc/cityseer/tools/graphs.py:1965-2149): one node
    per street at its midpoint, one undirected dual edge per pair of streets sharing a primal node,
    geometry = half street + half street welded at the shared node, shared_primal_node_key = that
    node.  Directed edges are inserted per dual node in ascending order of (neighbour, shared node)."""
    if all(g is None for g in p.geoms):
        return _dual_structure_straight(p)
    half_u, half_v, mids = _half_polylines(p)
    m = len(p.u)
    inc: dict[int, list[tuple[int, int]]] = {}
    for e in range(m):
        inc.setdefault(int(p.u[e]), []).append((e, 0))
        inc.setdefault(int(p.v[e]), []).append((e, 1))
    src, dst, lens, angs, shared = [], [], [], [], []
    for node, lst in inc.items():
        for a in range(len(lst)):
            for b in range(a + 1, len(lst)):
                e1, s1 = lst[a]
                e2, s2 = lst[b]
                h1 = half_u[e1] if s1 == 0 else half_v[e1]   # node -> mid1
                h2 = half_u[e2] if s2 == 0 else half_v[e2]   # node -> mid2
                for (ea, ha), (eb, hb) in (((e1, h1), (e2, h2)), ((e2, h2), (e1, h1))):
                    pts = np.vstack([ha[::-1], hb[1:]])    # mid_a -> node -> mid_b
                    seg = np.hypot(np.diff(pts[:, 0]), np.diff(pts[:, 1]))
                    ln = 0.0
                    for s_ in seg:
                        ln += float(s_)
                    an = 0.0
                    for q in range(1, len(pts) - 1):
                        an += float(_turn(pts[q - 1, 0], pts[q - 1, 1], pts[q, 0], pts[q, 1], pts[q + 1, 0],
                                          pts[q + 1, 1]))
                    src.append(ea)
                    dst.append(eb)
                    lens.append(ln)
                    angs.append(an)
                    shared.append(node)
    src = np.array(src, np.int64)
    dst = np.array(dst, np.int64)
    # parallel streets give two dual edges with the same ends: order those by the shared node
    order = np.lexsort((np.array(shared, np.int64), dst, src))
    return NetworkStructure.from_arrays(
        mids[:, 0], mids[:, 1], src[order], dst[order], np.array(lens)[order].astype(np.float32),
        edge_idx=np.zeros(len(src), np.int64), edge_angle_sum=np.array(angs)[order].astype(np.float32),
        edge_shared_key=[str(s) for s in np.array(shared)[order]], is_dual=True)


CONFIGS = {
    "c1": dict(side=40, spacing=100.0, jitter=20.0, drop=0.15, seed=1, distances=[500, 1000, 2000]),
    "c2": dict(side=450, spacing=80.0, jitter=15.0, drop=0.10, seed=2, diag_frac=0.05,
               distances=[500, 1000, 2000, 5000]),
    "c3": dict(side=250, spacing=80.0, jitter=15.0, drop=0.0, seed=3, curved_frac=0.30,
               distances=[500, 1000, 2000]),
}


def lattice_config(name: str, side: int | None = None):
    """(Primal, distances) for a named workload; `side` overrides the lattice size for small runs."""
    cfg = dict(CONFIGS[name])
    dists = cfg.pop("distances")
    if side is not None:
        cfg["side"] = side
    return lattice(**cfg), dists


BATCH_THRESHOLDS = (400, 800, 1200, 1600, 3200, 4800)


def batch_workload(n_graphs: int = 96, min_nodes: int = 2000, max_nodes: int = 150_000, seed: int = 4):
    """Mixed-size workload of the batched form: `n_graphs` lattices built like "c1" (100 m, jitter
    +-20 m, 15% of streets dropped), node counts log-uniform over [min_nodes, max_nodes] (side =
    round(sqrt(N))), each with its own seed and 2-4 thresholds drawn from BATCH_THRESHOLDS.
    Returns [(Primal, distances)]."""
    rng = np.random.default_rng(seed)
    out = []
    for g in range(n_graphs):
        n = float(np.exp(rng.uniform(np.log(min_nodes), np.log(max_nodes))))
        side = max(2, int(round(np.sqrt(n))))
        k = int(rng.integers(2, 5))
        dists = sorted(int(x) for x in rng.choice(BATCH_THRESHOLDS, size=k, replace=False))
        p = lattice(side=side, spacing=100.0, jitter=20.0, drop=0.15, seed=10_000 + seed * 1000 + g)
        out.append((p, dists))
    return out
