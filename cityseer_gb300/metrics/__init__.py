"""Metric wrappers mirroring cityseer.metrics."""
