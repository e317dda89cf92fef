"""The synthetic workloads stand in for the benchmark configurations' networks; their shapes are
checked here against the configurations' stated sizes and recipes (node counts, streets, drop and
diagonal fractions, curvature, dual sizes, thresholds)."""

from cityseer_gb300 import synth


def test_c1_lattice_recipe():
    p, dists = synth.lattice_config("c1")
    assert len(p.x) == 40 * 40 and dists == [500, 1000, 2000]
    full = 2 * 40 * 39
    assert len(p.u) == full - int(round(0.15 * full))  # 15% of streets dropped
    ns = synth.primal_structure(p)
    assert ns.node_count() == 1600 and int(ns.arrays()["e_exists"].sum()) == 2 * len(p.u)


def test_c2_lattice_recipe():
    p, dists = synth.lattice_config("c2")
    n = 450 * 450
    assert len(p.x) == n and dists == [500, 1000, 2000, 5000]
    full = 2 * 450 * 449
    diag = len(p.u) - (full - int(round(0.10 * full)))
    assert 0.04 * n < diag <= 0.05 * n  # one diagonal for ~5% of nodes (fewer at the border)
    stretch = p.stretched[-diag:]
    assert stretch.min() >= 1.0 and stretch.max() <= 1.3
    assert 2 * len(p.u) == 747_568  # directed edges of the benchmark graph


def test_c3_curved_lattice_and_dual():
    p, dists = synth.lattice_config("c3", side=60)
    assert dists == [500, 1000, 2000]
    curved = sum(g is not None for g in p.geoms)
    assert abs(curved / len(p.u) - 0.30) < 0.03
    full = synth.lattice_config("c3")[0]
    assert len(full.u) == 2 * 250 * 249 == 124_500  # no drops: one dual node per street
    nsd = synth.dual_structure(p)
    assert nsd.is_dual and nsd.node_count() == len(p.u)


def test_batch_workload_shape():
    w = synth.batch_workload(n_graphs=12, seed=4)
    assert len(w) == 12
    for p, dists in w:
        assert 2000 * 0.9 <= len(p.x) <= 150_000 * 1.1
        assert 2 <= len(dists) <= 4 and dists == sorted(dists)
        assert set(dists) <= set(synth.BATCH_THRESHOLDS)
