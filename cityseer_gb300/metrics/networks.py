"""cityseer.metrics.networks wrappers (pysrc/cityseer/metrics/networks.py:101-755).

Same signatures, defaults and output columns (cc_{metric}_{d}, `_ang` for simplest, cc_seg_* for
segment).  `nodes_gdf` may be a (Geo)DataFrame indexed by node key, or -- where pandas is not
installed -- a plain dict of columns; in that case the new columns are numpy arrays in
`network_structure.node_keys_py()` order, and the same dict is returned.
"""
from __future__ import annotations

import logging

import numpy as np

from .. import config, sampling
from ..common import pair_distances_betas_time

logger = logging.getLogger(__name__)

MIN_THRESH_WT = config.MIN_THRESH_WT
SPEED_M_S = config.SPEED_M_S


def _require_dual_for_angular(network_structure, context: str) -> None:
    if not network_structure.is_dual:
        raise ValueError(
            f"{context} requires a dual graph for angular analysis. "
            "Convert the graph with cityseer.tools.graphs.nx_to_dual(...) before ingesting it."
        )


def _write(nodes_gdf, keys, temp: dict[str, np.ndarray]):
    if hasattr(nodes_gdf, "loc") and hasattr(nodes_gdf, "index"):
        import pandas as pd

        df = pd.DataFrame(temp, index=keys)
        idx = nodes_gdf.index.intersection(keys)
        nodes_gdf.loc[idx, df.columns] = df.loc[idx, df.columns]
        return nodes_gdf
    if nodes_gdf is None:
        nodes_gdf = {}
    nodes_gdf.setdefault("index", list(keys))
    for k, v in temp.items():
        nodes_gdf[k] = np.asarray(v)
    return nodes_gdf


def _schedule(resolved, sample, epsilon):
    eps = epsilon if epsilon is not None else sampling.HOEFFDING_EPSILON
    full, sampled = [], []
    if not sample:
        return sorted(resolved), []
    logger.warning("Sampling is experimental: API and behaviour may change in future releases.")
    for d in sorted(resolved):
        p = sampling.compute_distance_p(d, epsilon=eps)
        if p >= 1.0:
            full.append(d)
        else:
            sampled.append((d, p))
    return full, sampled


def node_centrality_shortest(network_structure, nodes_gdf, distances=None, betas=None, minutes=None,
                             compute_closeness=True, compute_betweenness=True, min_threshold_wt=MIN_THRESH_WT,
                             speed_m_s=SPEED_M_S, tolerance=None, random_seed=None, sample=False, epsilon=None):
    resolved, _b, _s = pair_distances_betas_time(speed_m_s, distances, betas, minutes,
                                                 min_threshold_wt=min_threshold_wt)
    full, sampled = _schedule(resolved, sample, epsilon)
    results = {}
    if full:
        res = network_structure.centrality_shortest(
            distances=full, compute_closeness=compute_closeness, compute_betweenness=compute_betweenness,
            min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s, tolerance=tolerance, random_seed=random_seed)
        for d in full:
            results[d] = res
    for d, p in sampled:
        results[d] = network_structure.centrality_shortest(
            distances=[d], compute_closeness=compute_closeness, compute_betweenness=compute_betweenness,
            min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s, tolerance=tolerance, sample_probability=p,
            random_seed=random_seed)
    if not results:
        return nodes_gdf
    keys = next(iter(results.values())).node_keys_py
    temp = {}
    if compute_closeness:
        for measure, attr in (("beta", "node_beta"), ("cycles", "node_cycles"), ("density", "node_density"),
                              ("farness", "node_farness"), ("harmonic", "node_harmonic")):
            for d, res in results.items():
                temp[config.prep_gdf_key(measure, d)] = getattr(res, attr)[d]
        for d, res in results.items():
            with np.errstate(divide="ignore", invalid="ignore"):
                temp[config.prep_gdf_key("hillier", d)] = res.node_density[d] ** 2 / res.node_farness[d]
    if compute_betweenness:
        for measure, attr in (("betweenness", "node_betweenness"), ("betweenness_beta", "node_betweenness_beta")):
            for d, res in results.items():
                temp[config.prep_gdf_key(measure, d)] = getattr(res, attr)[d]
    return _write(nodes_gdf, keys, temp)


def node_centrality_simplest(network_structure, nodes_gdf, distances=None, betas=None, minutes=None,
                             compute_closeness=True, compute_betweenness=True, min_threshold_wt=MIN_THRESH_WT,
                             speed_m_s=SPEED_M_S, tolerance=None, angular_scaling_unit=90, farness_scaling_offset=1,
                             random_seed=None, sample=False, epsilon=None):
    _require_dual_for_angular(network_structure, "node_centrality_simplest")
    resolved, _b, _s = pair_distances_betas_time(speed_m_s, distances, betas, minutes,
                                                 min_threshold_wt=min_threshold_wt)
    full, sampled = _schedule(resolved, sample, epsilon)
    results = {}
    kw = dict(compute_closeness=compute_closeness, compute_betweenness=compute_betweenness,
              min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s, tolerance=tolerance,
              angular_scaling_unit=angular_scaling_unit, farness_scaling_offset=farness_scaling_offset,
              random_seed=random_seed)
    if full:
        res = network_structure.centrality_simplest(distances=full, **kw)
        for d in full:
            results[d] = res
    for d, p in sampled:
        results[d] = network_structure.centrality_simplest(distances=[d], sample_probability=p, **kw)
    if not results:
        return nodes_gdf
    keys = next(iter(results.values())).node_keys_py
    temp = {}
    if compute_closeness:
        for d, res in results.items():
            temp[config.prep_gdf_key("density", d, angular=True)] = res.node_density[d]
            temp[config.prep_gdf_key("harmonic", d, angular=True)] = res.node_harmonic[d]
            temp[config.prep_gdf_key("farness", d, angular=True)] = res.node_farness[d]
            with np.errstate(divide="ignore", invalid="ignore"):
                temp[config.prep_gdf_key("hillier", d, angular=True)] = res.node_density[d] ** 2 / res.node_farness[d]
    if compute_betweenness:
        for d, res in results.items():
            temp[config.prep_gdf_key("betweenness", d, angular=True)] = res.node_betweenness[d]
    return _write(nodes_gdf, keys, temp)


def segment_centrality(network_structure, nodes_gdf, distances=None, betas=None, minutes=None,
                       compute_closeness=True, compute_betweenness=True, min_threshold_wt=MIN_THRESH_WT,
                       speed_m_s=SPEED_M_S):
    res = network_structure.segment_centrality(distances=distances, betas=betas, minutes=minutes,
                                               compute_closeness=compute_closeness,
                                               compute_betweenness=compute_betweenness,
                                               min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s)
    dists, _b, _s = pair_distances_betas_time(speed_m_s, distances, betas, minutes, min_threshold_wt=min_threshold_wt)
    temp = {}
    if compute_closeness is True:
        for measure, attr in (("seg_density", "segment_density"), ("seg_harmonic", "segment_harmonic"),
                              ("seg_beta", "segment_beta")):
            for d in dists:
                temp[config.prep_gdf_key(measure, d)] = getattr(res, attr)[d]
    if compute_betweenness is True:
        for d in dists:
            temp[config.prep_gdf_key("seg_betweenness", d)] = res.segment_betweenness[d]
    return _write(nodes_gdf, res.node_keys_py, temp)


# convenience wrappers of the reference (networks.py, closeness / betweenness only)
def closeness_shortest(network_structure, nodes_gdf, **kw):
    return node_centrality_shortest(network_structure, nodes_gdf, compute_closeness=True, compute_betweenness=False,
                                    **kw)


def betweenness_shortest(network_structure, nodes_gdf, **kw):
    return node_centrality_shortest(network_structure, nodes_gdf, compute_closeness=False, compute_betweenness=True,
                                    **kw)


def closeness_simplest(network_structure, nodes_gdf, **kw):
    return node_centrality_simplest(network_structure, nodes_gdf, compute_closeness=True, compute_betweenness=False,
                                    **kw)


def betweenness_simplest(network_structure, nodes_gdf, **kw):
    return node_centrality_simplest(network_structure, nodes_gdf, compute_closeness=False, compute_betweenness=True,
                                    **kw)


def build_od_matrix(od_df, zones_gdf, network_structure, origin_col, destination_col, weight_col,
                    zone_id_col=None, max_snap_dist=500.0):
    """OdMatrix from OD flows and zones (pysrc/cityseer/metrics/networks.py:278-380): each zone's
    centroid snaps to the nearest network node (scipy KDTree); zones farther than max_snap_dist are
    left out, as are rows with a missing or non-positive weight or an unknown zone.  `zones_gdf` is a
    GeoDataFrame (polygon or point geometry, projected CRS) or, without geopandas, a dict with
    "x"/"y" centroid columns and the zone ids in `zone_id_col` (else "index").  `od_df` is anything
    indexable by column name (DataFrame or dict of columns).  Reprojection from EPSG:4326 is not
    restated: pass zones in the network's projected CRS."""
    from scipy.spatial import KDTree

    from ..centrality import OdMatrix

    if hasattr(zones_gdf, "geometry"):
        crs = getattr(zones_gdf, "crs", None)
        if crs is not None and crs.to_epsg() == 4326:
            raise ValueError("reproject the zones to the network's projected CRS first")
        geom_types = set(zones_gdf.geometry.geom_type)
        cents = zones_gdf.geometry.centroid if geom_types & {"Polygon", "MultiPolygon"} else zones_gdf.geometry
        coords = np.array([(g.x, g.y) for g in cents], np.float64)
        zone_ids = zones_gdf[zone_id_col].values if zone_id_col is not None else zones_gdf.index.values
    else:
        coords = np.column_stack([np.asarray(zones_gdf["x"], np.float64), np.asarray(zones_gdf["y"], np.float64)])
        zone_ids = list(zones_gdf[zone_id_col if zone_id_col is not None else "index"])
    tree = KDTree(np.asarray(network_structure.node_xys, np.float64))
    snap_d, snap_i = tree.query(coords)
    zone_to_node = {}
    n_excluded = 0
    for i, zid in enumerate(zone_ids):
        if snap_d[i] > max_snap_dist:
            n_excluded += 1
            continue
        zone_to_node[zid] = int(snap_i[i])
    if n_excluded:
        logger.warning(f"{n_excluded} zone centroids exceeded max_snap_dist={max_snap_dist}m and were excluded")
    origins, dests, weights = [], [], []
    for o_zone, d_zone, w in zip(list(od_df[origin_col]), list(od_df[destination_col]), list(od_df[weight_col])):
        if w is None or not np.isfinite(float(w)) or float(w) <= 0:
            continue
        if o_zone not in zone_to_node or d_zone not in zone_to_node:
            continue
        origins.append(zone_to_node[o_zone])
        dests.append(zone_to_node[d_zone])
        weights.append(float(w))
    logger.info(f"Built OD matrix: {len(origins)} pairs, {sum(weights):.0f} total trips")
    return OdMatrix(origins, dests, weights)


def betweenness_od(network_structure, nodes_gdf, od_matrix, distances=None, betas=None, minutes=None,
                   min_threshold_wt=MIN_THRESH_WT, speed_m_s=SPEED_M_S, tolerance=None):
    """OD-weighted shortest-path betweenness (pysrc/cityseer/metrics/networks.py:383-461): columns
    cc_betweenness_{d} and cc_betweenness_beta_{d}; no closeness."""
    res = network_structure.betweenness_od_shortest(
        od_matrix=od_matrix, distances=distances, betas=betas, minutes=minutes, min_threshold_wt=min_threshold_wt,
        speed_m_s=speed_m_s, tolerance=tolerance)
    temp = {}
    for measure, attr in (("betweenness", "node_betweenness"), ("betweenness_beta", "node_betweenness_beta")):
        rows = getattr(res, attr)
        for d in res.distances:
            temp[config.prep_gdf_key(measure, d)] = rows[d]
    return _write(nodes_gdf, res.node_keys_py, temp)
