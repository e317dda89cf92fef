"""cityseer.metrics.layers.compute_accessibilities (pysrc/cityseer/metrics/layers.py:104-283).

Same signature, defaults and output columns (cc_{key}_{d}_nw, cc_{key}_{d}_wt and
cc_{key}_nearest_max_{max d}, `_ang` for angular).  Without pandas, `data_gdf` is a dict of
columns: "geometry" (POINT WKT strings or (x, y) pairs), the land-use column, optionally the data id
column and "index" (the data keys; default 0..n-1); `nodes_gdf` is a dict of columns or None (the new
columns are numpy arrays in `network_structure.node_keys_py()` order).  With pandas, (Geo)DataFrames
work as in the reference.
"""
from __future__ import annotations

import numpy as np

from .. import config
from ..data import DataMap
from .networks import _write

MIN_THRESH_WT = config.MIN_THRESH_WT
SPEED_M_S = config.SPEED_M_S


def _wkt(g) -> str:
    if isinstance(g, str):
        return g
    if hasattr(g, "wkt"):
        return g.wkt
    x, y = g
    return f"POINT ({float(x)!r} {float(y)!r})"


def _columns(data_gdf, landuse_column_label: str, data_id_col: str | None):
    if hasattr(data_gdf, "columns") and hasattr(data_gdf, "index"):
        if landuse_column_label not in data_gdf.columns:
            raise ValueError("The specified landuse column name can't be found in the GeoDataFrame.")
        keys = list(data_gdf.index)
        geoms = list(data_gdf.geometry)
        lus = list(data_gdf[landuse_column_label])
        ids = list(data_gdf[data_id_col]) if data_id_col is not None else None
    else:
        if landuse_column_label not in data_gdf:
            raise ValueError("The specified landuse column name can't be found in the GeoDataFrame.")
        geoms = list(data_gdf["geometry"])
        keys = list(data_gdf.get("index", range(len(geoms))))
        lus = list(data_gdf[landuse_column_label])
        ids = list(data_gdf[data_id_col]) if data_id_col is not None else None
    return keys, geoms, lus, ids


def build_data_map(data_gdf, network_structure, max_netw_assign_dist: int = 100, data_id_col: str | None = None,
                   barriers_gdf=None, n_nearest_candidates: int = 50, landuse_column_label: str | None = None):
    """A DataMap of the data points, assigned to the network (layers.build_data_map)."""
    if barriers_gdf is not None:
        raise NotImplementedError("data assignment with barriers is not supported")
    keys, geoms, _, ids = _columns(data_gdf, landuse_column_label or "geometry", data_id_col)
    dm = DataMap()
    for i, (k, g) in enumerate(zip(keys, geoms)):
        dm.insert(k, _wkt(g), None if ids is None else ids[i])
    dm.assign_data_to_network(network_structure, max_netw_assign_dist, n_nearest_candidates)
    return dm


def compute_accessibilities(data_gdf, landuse_column_label: str, accessibility_keys: list[str], nodes_gdf,
                            network_structure, max_netw_assign_dist: int = 100, distances: list[int] | None = None,
                            betas: list[float] | None = None, minutes: list[float] | None = None,
                            data_id_col: str | None = None, barriers_gdf=None, angular: bool = False,
                            n_nearest_candidates: int = 50, spatial_tolerance: int = 0,
                            min_threshold_wt: float = MIN_THRESH_WT, speed_m_s: float = SPEED_M_S):
    """Land-use accessibilities per node: counts (nw), distance-weighted counts (wt) and the nearest
    distance within the largest threshold, written to nodes_gdf; returns (nodes_gdf, data_gdf)."""
    keys, geoms, lus, _ = _columns(data_gdf, landuse_column_label, data_id_col)
    dm = build_data_map(data_gdf, network_structure, max_netw_assign_dist, data_id_col, barriers_gdf,
                        n_nearest_candidates, landuse_column_label)
    landuses_map = dict(zip(keys, lus))
    res = dm.accessibility(network_structure, landuses_map, accessibility_keys, distances=distances, betas=betas,
                           minutes=minutes, angular=angular, spatial_tolerance=spatial_tolerance,
                           min_threshold_wt=min_threshold_wt, speed_m_s=speed_m_s)
    dists = config.log_thresholds(distances=distances, betas=betas, minutes=minutes, min_threshold_wt=min_threshold_wt,
                                  speed_m_s=speed_m_s)
    temp: dict[str, np.ndarray] = {}
    for key in accessibility_keys:
        acc = res.result[key]
        for d in dists:
            temp[config.prep_gdf_key(key, d, angular, weighted=False)] = acc.unweighted[d]
            temp[config.prep_gdf_key(key, d, angular, weighted=True)] = acc.weighted[d]
            if d == max(dists):
                temp[config.prep_gdf_key(f"{key}_nearest_max", d, angular)] = acc.distance[d]
    return _write(nodes_gdf, network_structure.node_keys_py(), temp), data_gdf
