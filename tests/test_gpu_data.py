"""GPU parity of the data layers (rust/src/data.rs) against the oracle: accessibility through
cs_accessibility (per class and threshold: counts bit-exact, clipped beta weights to 1e-6 relative,
nearest distances bit-exact), aggregate_to_src_idx over GPU trees, and angular accessibility on a
dual graph."""
import numpy as np
import pytest

import oracle
from cityseer_gb300 import common, config, synth
from cityseer_gb300.data import DataMap, composite_key
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph, structure

KEYS = ["a", "b", "c", "z"]


def _layer(xs, ys, groups, classes):
    dm = DataMap()
    for uid in range(len(xs)):
        dm.insert(int(uid), f"POINT ({float(xs[uid])!r} {float(ys[uid])!r})", int(groups[uid]))
    landuses = {int(uid): str(classes[uid]) for uid in range(len(xs))}
    return dm, landuses


def _check(ns, dm, landuses, dists, angular=False):
    res = dm.accessibility(ns, landuses, KEYS, distances=dists, angular=angular)
    d, b, s = common.pair_distances_betas_time(config.SPEED_M_S, distances=dists)
    mcw = np.asarray(common.clip_wts_curve(d, b, 0), np.float32)
    cls_of = {composite_key(k): KEYS.index(v) for k, v in landuses.items() if v in KEYS}
    t = dm._tables(ns, cls_of)
    u, w, n = oracle.accessibility(oracle.OracleGraph(ns), t, len(KEYS), d, b, mcw, max(s), config.SPEED_M_S,
                                   angular=angular)
    idx = np.asarray(ns.node_indices())
    for c, key in enumerate(KEYS):
        la = res.result[key]
        for i, dist in enumerate(d):
            np.testing.assert_array_equal(la.unweighted[dist], u[c, i][idx], err_msg=f"{key} unweighted {dist}")
            np.testing.assert_allclose(la.weighted[dist], w[c, i][idx], rtol=1e-6, atol=1e-12,
                                       err_msg=f"{key} weighted {dist}")
        np.testing.assert_array_equal(la.distance[max(d)], n[c][idx], err_msg=f"{key} nearest")
    return res


def _points(g, n, seed):
    xs_n = [v["x"] for _, v in g.nodes(data=True)]
    ys_n = [v["y"] for _, v in g.nodes(data=True)]
    rng = np.random.default_rng(seed)
    xs = rng.uniform(min(xs_n), max(xs_n), n)
    ys = rng.uniform(min(ys_n), max(ys_n), n)
    groups = np.arange(n)
    groups[-8:] = n - 8  # a cluster sharing one dedupe key
    classes = rng.choice(KEYS + ["q"], n)
    return xs, ys, groups, classes


@pytest.mark.gpu
def test_accessibility_mock_graph():
    g = mock_graph()
    ns = structure(g)[2]
    dm, lu = _layer(*_points(g, 60, 3))
    dm.assign_data_to_network(ns, 400, 6)
    _check(ns, dm, lu, [200, 400, 800, 1600])


@pytest.mark.gpu
def test_accessibility_lattice_with_dedupe_groups():
    p, _ = synth.lattice_config("c1", side=30)
    ns = synth.primal_structure(p)
    rng = np.random.default_rng(8)
    n = 3000
    xs = rng.uniform(p.x.min(), p.x.max(), n)
    ys = rng.uniform(p.y.min(), p.y.max(), n)
    groups = rng.integers(0, 1800, n)  # dedupe keys shared by up to a handful of entries
    classes = rng.choice(KEYS + ["q"], n)
    dm, lu = _layer(xs, ys, groups, classes)
    dm.assign_data_to_network(ns, 150, 6)
    assert sum(len(v) for v in dm.node_data_map.values()) > n
    _check(ns, dm, lu, [300, 700, 1500])


@pytest.mark.gpu
def test_aggregate_to_src_idx_and_angular():
    g = mock_graph()
    ns = structure(g)[2]
    xs, ys, groups, classes = _points(g, 50, 5)
    dm, lu = _layer(xs, ys, groups, classes)
    dm.assign_data_to_network(ns, 400, 6)
    t = dm._tables(ns)
    og = oracle.OracleGraph(ns)
    max_s = int(750 / config.SPEED_M_S)
    for src in ns.node_indices()[::5]:
        got = dm.aggregate_to_src_idx(src, ns, max_s, config.SPEED_M_S)
        ref = oracle.aggregate(og, t, src, max_s, config.SPEED_M_S)
        want = {t["keys"][e]: float(ref[e]) for e in np.nonzero(~np.isnan(ref))[0]}
        assert got == want, src
    with pytest.raises(ValueError, match="dual"):
        dm.aggregate_to_src_idx(ns.node_indices()[0], ns, max_s, config.SPEED_M_S, angular=True)
    nsd = io.network_structure_from_nx(graphs.nx_to_dual(g))[2]
    dmd, lud = _layer(xs, ys, groups, classes)
    dmd.assign_data_to_network(nsd, 400, 6)
    _check(nsd, dmd, lud, [400, 800], angular=True)


@pytest.mark.gpu
def test_compute_accessibilities_columns():
    from cityseer_gb300.metrics import layers

    g = mock_graph()
    ns = structure(g)[2]
    xs, ys, groups, classes = _points(g, 40, 11)
    data = {"geometry": list(zip(xs, ys)), "landuse": list(classes), "data_id": list(groups)}
    nodes, _ = layers.compute_accessibilities(data, "landuse", ["a", "z"], None, ns, max_netw_assign_dist=400,
                                              distances=[400, 800], data_id_col="data_id")
    dm, lu = _layer(xs, ys, groups, classes)
    dm.assign_data_to_network(ns, 400, 50)
    raw = dm.accessibility(ns, lu, ["a", "z"], distances=[400, 800])
    for key in ("a", "z"):
        for d in (400, 800):
            np.testing.assert_array_equal(nodes[f"cc_{key}_{d}_nw"], raw.result[key].unweighted[d])
            np.testing.assert_allclose(nodes[f"cc_{key}_{d}_wt"], raw.result[key].weighted[d], rtol=1e-12)
        np.testing.assert_array_equal(nodes[f"cc_{key}_nearest_max_800"], raw.result[key].distance[800])
