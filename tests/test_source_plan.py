"""The vectorised source plan (centrality.prepare_source_sampling) against a per-source loop that
follows sample_source_weight (rust/src/centrality.rs:1107-1139) step by step."""
import numpy as np
import pytest

from cityseer_gb300 import synth
from cityseer_gb300.centrality import prepare_source_sampling
from cityseer_gb300.stdrng import StdRng


def _loop_plan(ns, prob, sw, seed, source_indices):
    nb = ns.node_bound()
    a = ns.arrays()
    idx = np.asarray(ns.node_indices(), np.int64)
    live = a["live"][:nb].astype(bool)
    weight = a["weight"][:nb]
    is_indexed = source_indices is not None
    sources = np.asarray(source_indices, np.int64) if is_indexed else idx
    eligible = np.zeros(nb, np.uint8)
    if is_indexed:
        eligible[sources] = 1
    else:
        eligible[idx[live[idx]]] = 1
    prob = None if prob is None else np.float32(prob)
    randoms = StdRng.seed_from_u64(seed).random_f32(nb) if (prob is not None and not is_indexed) else None
    if sw is not None:
        sw = np.asarray(sw, np.float32)
    src_wt = np.zeros(nb, np.float32)
    proc, count = [], 0
    for s in sources:
        if not eligible[s]:
            continue
        wt = weight[s]
        if is_indexed:
            if prob is not None:
                wt = np.float32(wt / prob)
            count += 1
        elif prob is not None:
            p = prob if sw is None else np.float32(prob * sw[s])
            if p <= 0.0 or randoms[s] >= p:
                continue
            count += 1
            wt = np.float32(wt / p)
        proc.append(s)
        src_wt[s] = wt
    return np.asarray(proc, np.int32), src_wt, count


@pytest.mark.parametrize("case", range(7))
def test_vectorised_plan_equals_the_loop(case):
    p, _ = synth.lattice_config("c1", side=30)
    ns = synth.primal_structure(p)
    nb = ns.node_bound()
    rng = np.random.default_rng(case)
    a = ns.arrays()
    for v in rng.choice(nb, 40, replace=False):
        ns.set_node_live(int(v), False)
    w = rng.uniform(0.5, 2.0, nb).astype(np.float32)
    ns._weight.view()[:] = w
    ns._touch()
    sw = rng.random(nb).astype(np.float32)
    sw[rng.random(nb) < 0.2] = 0.0
    subset = rng.choice(nb, 200).tolist()  # repeats allowed, as the reference allows
    prob, weights, seed, src = [
        (None, None, None, None), (0.4, None, 7, None), (1.0, sw, 3, None), (0.7, sw, 11, None),
        (None, None, None, subset), (0.5, None, None, subset), (0.05, None, 1, None)][case]
    sp = prepare_source_sampling(ns, prob, weights, seed, src)
    proc, src_wt, count = _loop_plan(ns, prob, weights, seed, src)
    np.testing.assert_array_equal(sp.process, proc)
    np.testing.assert_array_equal(sp.src_wt, src_wt)
    assert sp.sampled_count == count
