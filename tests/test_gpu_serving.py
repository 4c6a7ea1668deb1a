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


def test_native_queue_matches_direct_solves():
    """The library's request queue (dg_enqueue / dg_poll, two worker threads
    with a stream each) on two contexts with interleaved requests, some with
    a new kappa (the worker rebuilds the operator first): every result equals
    the same sequence of calls made directly on twin contexts (<= 1e-12
    relative, deterministic kernels), meets its tolerance, and requests on
    one context run in their order."""
    from dg_nn_public_gb300 import element, mesh, sfc
    from dg_nn_public_gb300.solver import DGSolver, SolverConfig

    def solver(m):
        s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                     element.p3_element(3))
        s.set_build_mode("affine")
        s.build_operator()
        return s

    meshes = [mesh.build_mesh("tet", n, seed=0) for n in (4, 5)]
    queued = [solver(m) for m in meshes]
    direct = [solver(m) for m in meshes]
    rng = np.random.default_rng(11)
    plan = []   # (context index, kappa or None, mode)
    for k in range(7):
        c = k % 2
        kap = np.exp(0.5 * rng.standard_normal(meshes[c].nele)) if k in (0, 1, 2, 5) else None
        plan.append((c, kap, "fp64" if k == 3 else "mixed"))
    # right-hand sides formed before the queue runs: a context with requests
    # in flight belongs to the queue
    rhs = []
    for c, kap, mode in plan:
        b = direct[c].rhs(torch.ones(direct[c].nonods, dtype=torch.float64, device="cuda:0"))
        rhs.append((b, 1e-10 * float(torch.linalg.norm(b))))
    xs = [torch.zeros_like(b) for b, _ in rhs]
    torch.cuda.synchronize()   # the workers' streams do not wait for this thread's stream
    q = serving.NativeQueue(nworkers=2)
    jobs = []
    for (c, kap, mode), (b, tol), x in zip(plan, rhs, xs):
        jobs.append((q.enqueue(queued[c], x, b, tol, mode=mode, kappa=kap), x, b, tol))
    outs = [q.wait(rid, timeout=120.0) for rid, _, _, _ in jobs]
    q.close()
    assert all(o is not None and o["status"] == 0 for o in outs), outs
    for (c, kap, mode), (rid, x, b, tol), o in zip(plan, jobs, outs):
        s = direct[c]
        if kap is not None:
            s.set_kappa(kap)
            s.build_operator()
        xd = torch.zeros_like(b)
        if mode == "mixed":
            s.solve_mixed(xd, b, tol)
        else:
            s.gmres(xd, b, tol)
        d = float(torch.abs(x - xd).max() / torch.abs(xd).max())
        assert d <= 1e-12, (rid, mode, d)
        assert o["res"] <= tol
    for s in queued + direct:
        s.close()
