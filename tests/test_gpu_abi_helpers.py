"""GPU: a direct C-ABI call built with cityseer_gb300.abi (what a binding in another package would do)
gives the rows the public API returns."""
import numpy as np
import pytest

from cityseer_gb300 import abi
from cityseer_gb300.tools import graphs, io
from helpers import mock_graph, structure

pytestmark = pytest.mark.gpu

SHORT = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
         "node_betweenness_beta")
SIMPLE = ("node_density", "node_farness", "node_harmonic", "node_betweenness")


def test_shortest_call_through_the_abi_helpers():
    ns = structure(mock_graph())[2]
    dists = [200, 500, 1200]
    call = abi.shortest_call(ns, dists)
    abi.check(abi.library().cs_centrality_shortest(*call.args()), "cs_centrality_shortest")
    # the library adds the bucketed closeness terms into the rows before it returns
    rows = call.out.cpu().numpy()
    res = ns.centrality_shortest(distances=dists)
    idx = np.asarray(ns.node_indices())
    for m, name in enumerate(SHORT):
        for i, d in enumerate(dists):
            np.testing.assert_allclose(rows[m, i][idx], getattr(res, name)[d], rtol=1e-12, atol=1e-12,
                                       err_msg=f"{name}[{d}]")
    assert all(int(x) > 0 for x in call.reach.cpu().numpy())  # reached (source, target) pairs per threshold


def test_simplest_call_through_the_abi_helpers():
    nsd = io.network_structure_from_nx(graphs.nx_to_dual(mock_graph()))[2]
    dists = [300, 900]
    call = abi.simplest_call(nsd, dists, source_indices=[0, 3, 7, 11])
    abi.check(abi.library().cs_centrality_simplest(*call.args()), "cs_centrality_simplest")
    rows = call.out.cpu().numpy()
    res = nsd.centrality_simplest(distances=dists, source_indices=[0, 3, 7, 11])
    idx = np.asarray(nsd.node_indices())
    n_live, n_src = len(idx), 4
    for m, name in enumerate(SIMPLE):
        for i, d in enumerate(dists):
            want = getattr(res, name)[d]
            got = rows[m, i][idx] * (n_live / n_src if name == "node_betweenness" else 1.0)  # the API's post-scale
            np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12, err_msg=f"{name}[{d}]")
