"""Serving: resident meshes, HBM-footprint admission, continuous batching.

Each request's result must be the same alone and in the mix: a request is
solved once by a server that only has that request, and once inside a
stream of overlapping requests of several mesh sizes; the two solutions must
agree to 1e-12 relative (the slot computation is deterministic, so in
practice they are bitwise equal), and every solution must meet its FP64
residual tolerance.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import serving  # noqa: E402


def test_results_same_alone_and_in_mix():
    sizes = [3, 4, 5]
    srv = serving.SolveServer(sizes, hbm_budget=8e9)
    reqs = serving.make_requests(sizes, count=9, rate=200.0, seed=4, meshes=srv.meshes)
    mix = srv.run(reqs)
    assert len(mix) == 9
    # several requests were on the GPU at the same time
    overlaps = sum(1 for a in mix for b in mix if a.rid < b.rid and a.start < b.end and b.start < a.end)
    assert overlaps > 0
    srv.close()
    for r in mix:
        assert r.residual <= r.tol
    for rid in (0, 4, 8):
        alone_srv = serving.SolveServer(sizes, hbm_budget=8e9)
        req = reqs[rid]
        alone = alone_srv.run([serving.Request(req.rid, req.n, req.kappa, req.f, 0.0)])[0]
        alone_srv.close()
        x_mix = mix[rid].x
        d = np.abs(alone.x - x_mix).max() / np.abs(alone.x).max()
        assert d <= 1e-12, (rid, d)


def test_admission_respects_budget():
    """With a budget of one slot per mesh, requests of one size queue behind
    each other and the server creates no second slot."""
    srv = serving.SolveServer([4], hbm_budget=1.0)
    reqs = serving.make_requests([4], count=4, rate=1000.0, seed=1, meshes=srv.meshes)
    res = srv.run(reqs)
    assert len(srv.slots[4]) == 1
    assert all(r.residual <= r.tol for r in res)
    stats = serving.latency_stats(res)
    assert stats["p99_s"] >= stats["p50_s"] > 0
    srv.close()
