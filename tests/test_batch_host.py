"""The batched form's host side (job tables, mode groups, fusion pairing, result decoding) on the CPU:
every job of a Batch equals its plain call, with the C-ABI answered by the oracle-backed stand-in
(tests/standin.py).  The GPU batch tests check the kernels' side."""
import numpy as np
import pytest

import standin
from cityseer_gb300 import synth
from cityseer_gb300.batch import Batch
from cityseer_gb300.tools import io
from helpers import mock_graph

SHORT = ("node_density", "node_farness", "node_cycles", "node_harmonic", "node_beta", "node_betweenness",
         "node_betweenness_beta")
SEG = ("segment_density", "segment_harmonic", "segment_beta", "segment_betweenness")


@pytest.fixture
def stand_in(monkeypatch, tmp_path_factory):
    monkeypatch.setenv("CS_AUTOTUNE_CACHE", "/nonexistent/autotune.json")
    return standin.install(monkeypatch)


def _plain(spec):
    ns = spec["ns"]
    kw = dict(distances=spec["distances"], compute_closeness=spec.get("compute_closeness", True),
              compute_betweenness=spec.get("compute_betweenness", True))
    if spec["mode"] == "shortest":
        return ns.centrality_shortest(source_indices=spec.get("source_indices"), **kw), SHORT
    return ns.segment_centrality(**kw), SEG


@pytest.mark.parametrize("fuse", [False, True])
def test_batch_jobs_equal_plain_calls(stand_in, fuse):
    g1 = synth.primal_structure(synth.lattice_config("c1", side=8)[0])
    g2 = io.network_structure_from_nx(mock_graph())[2]
    stand_in(g1, g2)
    jobs = [dict(ns=g1, mode="shortest", distances=[300, 600]),
            dict(ns=g1, mode="segment", distances=[300, 600]),
            dict(ns=g2, mode="segment", distances=[200, 900, 1500]),
            dict(ns=g2, mode="shortest", distances=[200, 900, 1500], compute_closeness=False),
            dict(ns=g2, mode="shortest", distances=[400], source_indices=[0, 5, 9, 33])]
    b = Batch(jobs, fuse=fuse)
    assert b.n_fused == (1 if fuse else 0)  # one shortest + segment pair shares graph, thresholds and flags
    b.run()
    assert b.status() == (0, b.n_items)
    for spec, res in zip(jobs, b.results()):
        want, rows = _plain(spec)
        for name in rows:
            got, exp = getattr(res, name), getattr(want, name)
            for d in spec["distances"]:
                np.testing.assert_array_equal(got[d], exp[d], err_msg=f"{spec['mode']} {name}[{d}]")
