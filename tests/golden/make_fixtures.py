"""Extracts golden fixtures from the reference's own sources into tests/golden/*.json.

Reads (as text, with the ast module; nothing from the reference is imported or executed):
  pysrc/cityseer/tools/mock.py        mock_graph() node coordinates and edge list (57 nodes)
  tests/conftest.py                   diamond / box / parallel_segments fixture graphs
  tests/rustalgos/test_centrality.py  golden vectors asserted in test_local_centrality_all and the
                                      expected paths of test_shortest_path_trees
  tests/rustalgos/test_data.py        node -> data key targets of test_assign_to_network

Usage: python tests/golden/make_fixtures.py REFERENCE_ROOT   (the cityseer-api source tree)
"""
from __future__ import annotations

import ast
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _literal(node):
    return ast.literal_eval(node)


def mock_graph(ref: Path) -> dict:
    tree = ast.parse((ref / "pysrc/cityseer/tools/mock.py").read_text())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "mock_graph")
    nodes = edges = None
    for st in ast.walk(fn):
        if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name):
            if st.targets[0].id == "nodes":
                nodes = _literal(st.value)
            elif st.targets[0].id == "edges":
                edges = _literal(st.value)
    return {
        "source": "pysrc/cityseer/tools/mock.py:mock_graph",
        "nodes": [[k, d["x"], d["y"]] for k, d in nodes],
        "edges": [list(e) for e in edges],
    }


def conftest_graphs(ref: Path) -> dict:
    tree = ast.parse((ref / "tests/conftest.py").read_text())
    out = {}
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef):
            continue
        nodes = edges = None
        for st in ast.walk(fn):
            if isinstance(st, ast.Call) and isinstance(st.func, ast.Attribute):
                if st.func.attr == "add_nodes_from" and not isinstance(st.args[0], ast.Name):
                    nodes = _literal(st.args[0])
                elif st.func.attr == "add_edges_from" and not isinstance(st.args[0], ast.Name):
                    edges = _literal(st.args[0])
            if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name):
                if st.targets[0].id == "nodes":
                    nodes = _literal(st.value)
                elif st.targets[0].id == "edges":
                    edges = _literal(st.value)
        if nodes is not None and edges is not None:
            out[fn.name] = {
                "source": f"tests/conftest.py:{fn.name}",
                "nodes": [[str(k), float(d["x"]), float(d["y"])] for k, d in nodes],
                "edges": [[str(a), str(b)] for a, b in edges],
            }
    return out


def centrality_golden(ref: Path) -> dict:
    """np.allclose(<result>.<attr>[<dist>], [<values>], ...) assertions of test_local_centrality_all."""
    src = (ref / "tests/rustalgos/test_centrality.py").read_text()
    tree = ast.parse(src)
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "test_local_centrality_all")
    gold = []
    for st in ast.walk(fn):
        if not (isinstance(st, ast.Call) and isinstance(st.func, ast.Attribute) and st.func.attr == "allclose"):
            continue
        a0, a1 = st.args[0], st.args[1]
        if not (isinstance(a0, ast.Subscript) and isinstance(a0.value, ast.Attribute)):
            continue
        obj = a0.value.value.id
        attr = a0.value.attr
        dist = _literal(a0.slice)
        try:
            vals = _literal(a1)
        except ValueError:
            continue
        gold.append({"result": obj, "attr": attr, "distance": dist, "values": vals, "line": st.lineno})
    paths = []
    fn2 = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "test_shortest_path_trees")
    for st in ast.walk(fn2):
        if isinstance(st, ast.Assert) and isinstance(st.test, ast.Compare) and isinstance(st.test.comparators[0],
                                                                                           ast.List):
            try:
                paths.append({"line": st.lineno, "path": _literal(st.test.comparators[0])})
            except ValueError:
                pass
    return {"source": "tests/rustalgos/test_centrality.py", "local_centrality_all": gold, "dual_paths": paths}


def helper_graphs(ref: Path) -> dict:
    """Coordinates/edges of make_angular_plateau_graph and make_tolerance_drift_graph."""
    tree = ast.parse((ref / "tests/rustalgos/test_centrality.py").read_text())
    out = {}
    for fn in tree.body:
        if not (isinstance(fn, ast.FunctionDef) and fn.name in ("make_angular_plateau_graph",
                                                                  "make_tolerance_drift_graph")):
            continue
        coords = edges = None
        for st in ast.walk(fn):
            if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name) and st.targets[0].id == "coords":
                coords = _literal(st.value)
            if isinstance(st, ast.For) and isinstance(st.iter, ast.List):
                edges = _literal(st.iter)
        out[fn.name] = {
            "source": f"tests/rustalgos/test_centrality.py:{fn.name}",
            "nodes": [[k, float(x), float(y)] for k, (x, y) in coords.items()],
            "edges": [list(e) for e in edges],
        }
    return out


def data_assignment_targets(ref: Path) -> dict:
    """The node -> data keys targets asserted by test_assign_to_network
    (tests/rustalgos/test_data.py): primal_targets and decomp_targets (module-level dicts)."""
    tree = ast.parse((ref / "tests/rustalgos/test_data.py").read_text())
    out = {}
    for st in tree.body:
        if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name):
            name = st.targets[0].id
            if name in ("primal_targets", "decomp_targets"):
                out[name] = {str(k): v for k, v in _literal(st.value).items()}
    return out


def main(ref: Path) -> None:
    data = {
        "reference": "cityseer-api v4.24.0",
        "mock_graph": mock_graph(ref),
        "conftest": conftest_graphs(ref),
        "centrality": centrality_golden(ref),
        "helpers": helper_graphs(ref),
        "data_assignment": data_assignment_targets(ref),
    }
    (HERE / "reference_fixtures.json").write_text(json.dumps(data, indent=1))
    print("wrote", HERE / "reference_fixtures.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_fixtures.py <cityseer-api source root>")
    main(Path(sys.argv[1]))
