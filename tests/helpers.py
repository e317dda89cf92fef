"""Shared test helpers: fixture graphs from the reference's own test data, comparisons."""
from __future__ import annotations

import json
from pathlib import Path

import networkx as nx
import numpy as np

from cityseer_gb300.tools import graphs, io

GOLDEN = Path(__file__).resolve().parent / "golden"
FIX = json.loads((GOLDEN / "reference_fixtures.json").read_text())

# float sums: summation order differs between the GPU (atomics) and the oracle
RTOL_SUM = 1e-5
ATOL_SUM = 1e-9


def nx_from_spec(spec) -> nx.MultiGraph:
    g = nx.MultiGraph()
    for k, x, y in spec["nodes"]:
        g.add_node(str(k), x=float(x), y=float(y))
    for a, b in spec["edges"]:
        g.add_edge(str(a), str(b))
    return graphs.nx_simple_geoms(g)


def mock_graph() -> nx.MultiGraph:
    return nx_from_spec(FIX["mock_graph"])


def diamond_graph() -> nx.MultiGraph:
    return nx_from_spec(FIX["conftest"]["diamond_graph"])


def structure(g):
    return io.network_structure_from_nx(g)


def assert_close_sums(got, want, rtol=RTOL_SUM, atol=ATOL_SUM, what=""):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    bad = ~np.isclose(got, want, rtol=rtol, atol=atol, equal_nan=True)
    if bad.any():
        i = np.argwhere(bad)[0]
        raise AssertionError(f"{what}: {bad.sum()} mismatches, first at {tuple(i)}: got {got[tuple(i)]!r} "
                             f"want {want[tuple(i)]!r}")
