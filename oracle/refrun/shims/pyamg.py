"""Stub of pyamg (not installed here).  The SFC-multigrid path the oracle
runs (mg_opt_D = 2) never calls it; the reference only imports it and names
``pyamg.smoothed_aggregation_solver`` at import time (config.py:5, 137)."""


def smoothed_aggregation_solver(*args, **kwargs):
    raise RuntimeError("pyamg is not available; use the SFC multigrid (mg_opt_D=2)")


def air_solver(*args, **kwargs):
    raise RuntimeError("pyamg is not available")


def ruge_stuben_solver(*args, **kwargs):
    raise RuntimeError("pyamg is not available")
