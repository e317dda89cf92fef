"""Data layers (rust/src/data.rs): assignment of data points to street nodes, pinned to the targets
of the reference's test_assign_to_network, and the oracle's aggregate_to_src_idx and accessibility
checked the way the reference's own tests check them (tests/rustalgos/test_data.py)."""
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, config
from cityseer_gb300.data import DataMap, composite_key
from cityseer_gb300.tools import graphs
from helpers import FIX, mock_graph, structure


def mock_points(g, length=50, seed=0):
    """mock_data_gdf (pysrc/cityseer/tools/mock.py:274-311): uniform points over the graph's extents
    from numpy's legacy seeded stream, the last five a cluster sharing data_id length - 5."""
    xs_n = [d["x"] for _, d in g.nodes(data=True)]
    ys_n = [d["y"] for _, d in g.nodes(data=True)]
    np.random.seed(seed=seed)
    xs = np.random.uniform(min(xs_n), max(xs_n), length)
    ys = np.random.uniform(min(ys_n), max(ys_n), length)
    data_id = np.arange(length)
    for i, loc in enumerate(range(length - 5, length)):
        data_id[loc] = length - 5
        xs[loc], ys[loc] = 700100 + i * 10, 5719100 + i * 10
    return xs, ys, data_id


def data_map(xs, ys, data_id=None):
    dm = DataMap()
    for uid, (x, y) in enumerate(zip(xs, ys)):
        dm.insert(int(uid), f"POINT ({float(x)!r} {float(y)!r})", None if data_id is None else int(data_id[uid]))
    return dm


def test_composite_keys_and_entries():
    dm = DataMap()
    dm.insert(3, "POINT (1.5 2)")
    dm.insert("a", "POINT (0 0)", 7)
    assert dm.entry_keys() == ["int:3", "str:a"] and composite_key(3.0) == "float:3.0"
    assert dm.get_entry("str:a").dedupe_key == "int:7" and dm.get_entry("int:3").dedupe_key == "int:3"
    assert dm.count() == 2 and not dm.is_empty()
    with pytest.raises(ValueError, match="Failed to parse WKT"):
        dm.insert(4, "LINESTRING (0 0, 1 1)")


@pytest.mark.parametrize("decompose", [False, True])
def test_assignment_matches_reference_targets(decompose):
    g = mock_graph()
    g.remove_edge("14", "15")
    g.remove_edge("15", "28")
    if decompose:
        g = graphs.nx_decompose(g, 50)
    ns = structure(g)[2]
    xs, ys, _ = mock_points(mock_graph(), seed=25)
    # override_coords (tests/rustalgos/test_data.py:274-281)
    for loc, (x, y) in ((18, (701200, 5719400)), (39, (700750, 5720025)), (26, (700400, 5719525))):
        xs[loc], ys[loc] = x, y
    dm = data_map(xs, ys)
    dm.assign_data_to_network(ns, max_assignment_dist=400, n_nearest_candidates=6)
    targets = FIX["data_assignment"]["decomp_targets" if decompose else "primal_targets"]
    assert sorted(dm.node_data_map) == sorted(int(k) for k in targets)
    nx_, ny_ = ns._x.view(), ns._y.view()
    for node, assigned in dm.node_data_map.items():
        assert sorted(k for k, _ in assigned) == sorted(targets[str(node)]), node
        for key, dist in assigned:
            e = dm.get_entry(key)
            assert abs(np.hypot(e.x - nx_[node], e.y - ny_[node]) - dist) < config.ATOL
    dm.assign_data_to_network(ns, max_assignment_dist=0, n_nearest_candidates=6)
    assert dm.node_data_map == {}


@pytest.mark.parametrize("dedupe", [False, True])
@pytest.mark.parametrize("max_dist", [250, 750])
def test_oracle_aggregation_against_trees(dedupe, max_dist):
    """aggregate_to_src_idx against a manual walk of the source's tree (as the reference's
    test_aggregate_to_src_idx): every reachable entry at network + assignment distance, the shadowed
    members of the clustered dedupe key replaced by the nearest one."""
    g = mock_graph()
    ns = structure(g)[2]
    xs, ys, did = mock_points(g)
    dm = data_map(xs, ys, did if dedupe else None)
    dm.assign_data_to_network(ns, 400, 6)
    t = dm._tables(ns)
    og = oracle.OracleGraph(ns)
    max_s = int(max_dist / config.SPEED_M_S)
    for src in ns.node_indices():
        got = oracle.aggregate(og, t, src, max_s, config.SPEED_M_S)
        vis, tree = oracle.tree_shortest(og, src, max_s, config.SPEED_M_S)
        manual = {}
        for v in vis:
            sec = tree["agg_seconds"][v]
            if not sec < np.float32(max_s):
                continue
            for key, dd in dm.node_data_map.get(int(v), []):
                tot = np.float32(sec * np.float32(config.SPEED_M_S)) + np.float32(dd)
                if tot <= np.float32(np.float32(max_s) * np.float32(config.SPEED_M_S)):
                    manual[key] = min(manual.get(key, np.inf), float(tot))
        reach = {t["keys"][e]: float(got[e]) for e in np.nonzero(~np.isnan(got))[0]}
        shadowed = {"int:45", "int:46", "int:47", "int:48"}
        for key, dist in manual.items():
            if dedupe and key in shadowed | {"int:49"}:
                continue
            assert reach[key] == pytest.approx(dist, abs=1e-3)
        if dedupe:
            group = [k for k in manual if k in shadowed | {"int:49"}]
            kept = [k for k in reach if k in shadowed | {"int:49"}]
            assert len(kept) == (1 if group else 0)
            if group:
                assert reach[kept[0]] == pytest.approx(min(manual[k] for k in group), abs=1e-3)
        assert set(reach) <= set(manual)


def test_oracle_accessibility_sums_the_aggregation():
    """accessibility's rows equal the per-source sums over aggregate_to_src_idx (the reference's
    test_accessibility), with four classes and a deduplicated cluster."""
    g = mock_graph()
    ns = structure(g)[2]
    xs, ys, did = mock_points(g, seed=13)
    rng = np.random.default_rng(13)
    classes = rng.choice(list("abcz"), len(xs))
    classes[-5:] = "z"
    dm = data_map(xs, ys, did)
    dm.assign_data_to_network(ns, 400, 6)
    keys = ["a", "b", "c", "z"]
    cls_of = {composite_key(i): keys.index(c) for i, c in enumerate(classes)}
    t = dm._tables(ns, cls_of)
    d, b, s = common.pair_distances_betas_time(config.SPEED_M_S, distances=[200, 400, 800, 1600])
    mcw = np.asarray(common.clip_wts_curve(d, b, 0), np.float32)
    og = oracle.OracleGraph(ns)
    u, w, n = oracle.accessibility(og, t, 4, d, b, mcw, max(s), config.SPEED_M_S)
    for src in ns.node_indices():
        got = oracle.aggregate(og, t, src, max(s), config.SPEED_M_S)
        for i, dist in enumerate(d):
            for c in range(4):
                sel = [e for e in np.nonzero(~np.isnan(got))[0] if t["entry_class"][e] == c and got[e] <= dist]
                assert u[c, i, src] == len(sel)
                wt = sum(float(np.float32(min(np.float32(np.exp(np.float32(-b[i]) * got[e])), mcw[i]) / mcw[i]))
                         for e in sel)
                assert w[c, i, src] == pytest.approx(wt, rel=1e-6, abs=1e-9)
                if dist == max(d):
                    want = min((float(got[e]) for e in sel), default=np.nan)
                    assert (np.isnan(n[c, src]) and np.isnan(want)) or n[c, src] == pytest.approx(want)
