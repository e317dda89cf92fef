"""Simplest-path (angular) centrality on the dual graph -- device CSR and drivers."""
from __future__ import annotations


def run_simplest(ns, dists, bets, secs, speed, tol, asu, fso, closeness, betweenness, sp):
    raise NotImplementedError("simplest-path kernels are not built yet")


def tree_simplest(ns, sources, max_seconds, speed):
    raise NotImplementedError("simplest-path kernels are not built yet")
