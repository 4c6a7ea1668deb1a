"""Mixed-precision solve (FP32 inner FGMRES + FP32 multigrid inside FP64
refinement) against the FP64 path and the manufactured solution.

Both solves stop at ||b - A x|| <= 1e-10 ||b|| in FP64, so they are two
approximations of the same discrete solution; their difference is bounded
by the condition number times the tolerance.  The tests check the FP64
residual independently, the solution difference (<= 1e-7 relative, max-abs)
and that the discretisation error against the exact solution is unchanged.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import element, mesh, sfc  # noqa: E402
from dg_nn_public_gb300.solver import DGSolver, SolverConfig  # noqa: E402


def _setup(kind, n, smooth, kappa_sigma=0.0, seed=0):
    m = mesh.build_mesh(kind, n, seed=seed)
    order = sfc.hilbert_sfc_order(m.cg_coords)
    s = DGSolver(m, order, SolverConfig(pre_smooth_its=smooth, post_smooth_its=smooth),
                 element.p3_element(m.ndim))
    if kappa_sigma > 0:
        kap = np.exp(kappa_sigma * np.random.default_rng(seed).standard_normal(m.nele))
        s.set_kappa(kap)
    s.build_operator()
    X = m.x_ref_in
    u = np.prod([np.sin(np.pi * X[:, k]) for k in range(m.ndim)], axis=0).ravel()
    f = m.ndim * np.pi ** 2 * u
    return m, s, f, u


@pytest.mark.parametrize("kind,n,smooth", [("tet", 6, 2), ("tri", 16, 3), ("tet", 12, 2)])
def test_mixed_matches_fp64(kind, n, smooth):
    m, s, f, u = _setup(kind, n, smooth)
    b = s.rhs(torch.tensor(f, device="cuda:0"))
    tol = 1e-10 * float(torch.linalg.norm(b))
    x64 = torch.zeros_like(b)
    its64, res64 = s.gmres(x64, b, tol)
    xm = torch.zeros_like(b)
    its, res, outer = s.solve_mixed(xm, b, tol)
    assert res <= tol
    r = s.residual(xm, b)
    assert float(torch.linalg.norm(r)) <= tol * (1 + 1e-12)
    d = float(torch.abs(xm - x64).max() / torch.abs(x64).max())
    assert d < 1e-7, d
    e64 = float(torch.abs(x64.cpu() - torch.tensor(u)).max())
    em = float(torch.abs(xm.cpu() - torch.tensor(u)).max())
    assert abs(em - e64) <= 1e-6 * e64
    assert outer >= 1 and its >= 1


def test_mixed_variable_kappa_and_nonzero_guess():
    m, s, f, u = _setup("tet", 6, 2, kappa_sigma=1.0, seed=4)
    b = s.rhs(torch.tensor(f, device="cuda:0"))
    tol = 1e-10 * float(torch.linalg.norm(b))
    x64 = torch.zeros_like(b)
    s.gmres(x64, b, tol)
    x0 = torch.randn_like(b)
    its, res, outer = s.solve_mixed(x0, b, tol)
    assert res <= tol
    assert float(torch.abs(x0 - x64).max() / torch.abs(x64).max()) < 1e-7


def test_mixed_iteration_limit_reports_noconv():
    from dg_nn_public_gb300 import _capi
    m, s, f, u = _setup("tet", 4, 2)
    b = s.rhs(torch.tensor(f, device="cuda:0"))
    x = torch.zeros_like(b)
    with pytest.raises(_capi.DGError) as ei:
        s.solve_mixed(x, b, 1e-30, max_its=5, raise_noconv=True)
    assert ei.value.code == _capi.DG_ERR_NOCONV
    assert torch.isfinite(x).all()


@pytest.mark.parametrize("smoother,bf16,scaled,tol", [("jacobi3", False, "1", 1e-5), ("blockinv", False, "1", 1e-5),
                                                      ("blockinv", True, "0", 3e-2), ("blockinv", True, "1", 3e-2)])
def test_smooth_pc_matches_fp64_smoothing(smoother, bf16, scaled, tol, monkeypatch):
    """One preconditioner smoothing step (FP32 vectors; FP32 or BF16 blocks)
    against the same step in FP64: the three-sweep Jacobi map through
    dg_residual(do_smooth=1), or x + w A_ee^-1 (b - A x) with the FP64
    diagonal blocks from dg_get_bdiag.  With BF16 blocks the step runs on
    the unscaled blocks and smoother matrices, or (scaled = "1") as
    x + c - w x - sum_f S_f x_f with the scaled face blocks S_f = W A_f and
    c = W b.  Tolerance relative to max|x_out|."""
    monkeypatch.setenv("DG_SCALED_FACES", scaled)
    m, s, f, u = _setup("tet", 6, 2)
    w = 0.8
    s.set_mixed_options(smoother=smoother, smooth_w=w, precond_bf16=bf16)
    g = torch.Generator(device="cuda:0").manual_seed(3)
    x = torch.randn(s.nonods, dtype=torch.float64, device="cuda:0", generator=g)
    b = torch.randn(s.nonods, dtype=torch.float64, device="cuda:0", generator=g)
    if smoother == "jacobi3":
        ref = torch.empty_like(x)
        s.residual(x, b, x_out=ref, smooth=True)
    else:
        K, _ = s.bdiag()
        r = s.residual(x, b).view(m.nele, m.nloc, 1)
        ref = x + w * torch.linalg.solve(K.view(m.nele, m.nloc, m.nloc), r).view(-1)
    out = s.smooth_pc(x.float().contiguous(), b.float().contiguous())
    err = float(torch.abs(out.double() - ref).max() / torch.abs(ref).max())
    assert err < tol, err
    out2 = s.smooth_pc(x.float().contiguous(), b.float().contiguous())
    assert torch.equal(out, out2)


@pytest.mark.parametrize("n", [6, 7])
def test_bulk_copy_kernels_match_plain_loads(n, monkeypatch):
    """The persistent bulk-copy (TMA) kernels and the plain-load kernels run
    the same arithmetic in the same order: the preconditioner's smoothing
    step (BF16 and FP32 block copies), the whole FP32 preconditioner and the
    FP32 apply agree bit for bit (7^3 * 6 = 2058 tets leaves partial last
    groups of elements)."""
    outs = {}
    monkeypatch.setenv("DG_SHARED_FACES", "0")
    monkeypatch.setenv("DG_SCALED_FACES", "0")   # the plain-load kernels have no scaled form
    for tma in ("1", "0"):
        monkeypatch.setenv("DG_BF16_TMA", tma)
        monkeypatch.setenv("DG_F32_TMA", tma)
        m, s, f, u = _setup("tet", n, 2)
        g = torch.Generator(device="cuda:0").manual_seed(8)
        x = torch.randn(s.nonods, dtype=torch.float32, device="cuda:0", generator=g)
        b = torch.randn(s.nonods, dtype=torch.float32, device="cuda:0", generator=g)
        res = [s.smooth_pc(x, b), s.precond_f32(b), s.apply_f32(x)]
        s.set_mixed_options(precond_bf16=False)
        s.build_operator()
        res += [s.smooth_pc(x, b), s.precond_f32(b)]
        torch.cuda.synchronize()
        outs[tma] = res
    for a, c in zip(outs["1"], outs["0"]):
        assert torch.equal(a, c)


@pytest.mark.parametrize("n", [6, 7])
def test_shared_face_copies_match_five_block_copies(n, monkeypatch):
    """Each interior face block stored once (read transposed by the
    neighbour) against five stored blocks per element, both through the
    bulk-copy kernels.  The operator is symmetric to FP64 rounding, so the
    reduced-precision copies differ at most by one rounding step in a few
    entries: FP32 apply within 1e-6, BF16 smoothing step and FP32
    preconditioner within 1e-4 (relative to the max entry); the mixed solve
    reaches the same FP64 tolerance with the same solution to 1e-9."""
    outs = {}
    monkeypatch.setenv("DG_SCALED_FACES", "0")   # both forms on the unscaled blocks
    for sf in ("1", "0"):
        monkeypatch.setenv("DG_SHARED_FACES", sf)
        m, s, f, u = _setup("tet", n, 2, kappa_sigma=0.5, seed=2)
        g = torch.Generator(device="cuda:0").manual_seed(8)
        x = torch.randn(s.nonods, dtype=torch.float32, device="cuda:0", generator=g)
        b = torch.randn(s.nonods, dtype=torch.float32, device="cuda:0", generator=g)
        res = [s.apply_f32(x), s.smooth_pc(x, b), s.precond_f32(b)]
        bb = s.rhs(torch.tensor(f, device="cuda:0"))
        tol = 1e-10 * float(torch.linalg.norm(bb))
        xm = torch.zeros_like(bb)
        its, r, outer = s.solve_mixed(xm, bb, tol)
        assert r <= tol
        torch.cuda.synchronize()
        outs[sf] = res + [xm]
    for (a, c), t in zip(zip(outs["1"], outs["0"]), (1e-6, 1e-4, 1e-4, 1e-9)):
        err = float(torch.abs(a.double() - c.double()).max() / torch.abs(c.double()).max())
        assert err < t, (t, err)


@pytest.mark.parametrize("cond", ["0", "1"])
def test_chunk_graphs_match_direct_launches(cond, monkeypatch):
    """Chunk graphs against direct launches of the inner Arnoldi steps: the
    solution is bitwise the same.  With the device-side convergence test
    (cond = 1: Givens update per step, one conditional graph node per step)
    the graphs skip the steps after the test is met, direct launches run the
    whole chunk and stop at the same Krylov step, so the graph form runs no
    more steps."""
    outs = {}
    monkeypatch.setenv("DG_COND_GRAPH", cond)
    for ng in ("1", "0"):
        monkeypatch.setenv("DG_NO_GRAPH", ng)
        m, s, f, u = _setup("tet", 8, 2, kappa_sigma=0.5, seed=3)
        b = s.rhs(torch.tensor(f, device="cuda:0"))
        tol = 1e-10 * float(torch.linalg.norm(b))
        x = torch.zeros_like(b)
        its, res, outer = s.solve_mixed(x, b, tol)
        assert res <= tol
        torch.cuda.synchronize()
        outs[ng] = (x.cpu(), its)
    assert torch.equal(outs["0"][0], outs["1"][0])
    assert outs["0"][1] <= outs["1"][1]


@pytest.mark.parametrize("kind,n,fits", [("tet", 14, True), ("tet", 20, True), ("tet", 28, False),
                                         ("tri", 64, True)])
def test_cluster_vcycle_matches_launch_chain(kind, n, fits):
    """The SFC V-cycle legs as two thread-block-cluster launches (16 and 8
    CTAs) against the chain of per-sweep launches: the same operations in
    the same order, so the FP32 preconditioner agrees bit for bit; the mixed
    solve then takes the same iterations.  1 to 4 levels above the dense
    coarse level (3,375 to 24,389 P1 vertices); where a CTA's share of the
    levels does not fit in its shared memory the chain runs (chosen 0)."""
    m = mesh.build_mesh(kind, n, seed=1)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                 element.p3_element(m.ndim))
    s.set_kappa(np.exp(0.5 * np.random.default_rng(5).standard_normal(m.nele)))
    s.build_operator()
    g = torch.Generator(device="cuda:0").manual_seed(3)
    b = torch.randn(s.nonods, dtype=torch.float32, device="cuda:0", generator=g)
    assert s.set_vcycle_cluster(0) == -1          # before the first mixed build
    z_chain = s.precond_f32(b).clone()
    outs = {}
    for cs in (16, 8, -1):
        chosen = s.set_vcycle_cluster(cs)
        assert chosen in ((cs, 0) if cs > 0 else (16, 8, 0)), (cs, chosen)
        if cs == -1:
            assert (chosen > 0) == fits, chosen
        outs[cs] = s.precond_f32(b).clone()
        again = s.precond_f32(b)
        assert torch.equal(outs[cs], again)
    torch.cuda.synchronize()
    for cs, z in outs.items():
        assert torch.equal(z, z_chain), cs
    X = m.x_ref_in
    u = np.prod([np.sin(np.pi * X[:, k]) for k in range(m.ndim)], axis=0).ravel()
    bb = s.rhs(torch.tensor(m.ndim * np.pi ** 2 * u, device="cuda:0"))
    tol = 1e-10 * float(torch.linalg.norm(bb))
    res = {}
    for cs in (0, -1):
        s.set_vcycle_cluster(cs)
        x = torch.zeros_like(bb)
        its, r, outer = s.solve_mixed(x, bb, tol)
        assert r <= tol
        res[cs] = (its, outer, x)
    assert res[0][:2] == res[-1][:2]
    assert torch.equal(res[0][2], res[-1][2])
    s.close()


@pytest.mark.parametrize("kind,n", [("tet", 14), ("tet", 20), ("tri", 64)])
def test_blocked_fp32_dense_inverse(kind, n, monkeypatch):
    """The dense coarse inverse of the mixed preconditioner by the blocked
    FP32 Gauss-Jordan against the one-pivot FP64 form (DG_DENSE_FP64=1):
    the FP32 preconditioner outputs agree to 1e-4 of their max entry and
    the mixed solves reach the same tolerance within two inner iterations of
    each other (a rounding-level change of the preconditioner can move the
    predicted stop of a refinement step by one step)."""
    outs, its = {}, {}
    for fp64 in ("0", "1"):
        monkeypatch.setenv("DG_DENSE_FP64", fp64)
        m = mesh.build_mesh(kind, n, seed=1)
        s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                     element.p3_element(m.ndim))
        s.set_kappa(np.exp(0.5 * np.random.default_rng(5).standard_normal(m.nele)))
        s.build_operator()
        g = torch.Generator(device="cuda:0").manual_seed(3)
        b = torch.randn(s.nonods, dtype=torch.float32, device="cuda:0", generator=g)
        outs[fp64] = s.precond_f32(b).clone()
        X = m.x_ref_in
        u = np.prod([np.sin(np.pi * X[:, k]) for k in range(m.ndim)], axis=0).ravel()
        bb = s.rhs(torch.tensor(m.ndim * np.pi ** 2 * u, device="cuda:0"))
        tol = 1e-10 * float(torch.linalg.norm(bb))
        x = torch.zeros_like(bb)
        it, r, outer = s.solve_mixed(x, bb, tol)
        assert r <= tol
        its[fp64] = it
        s.close()
    err = float(torch.abs(outs["0"] - outs["1"]).max() / torch.abs(outs["1"]).max())
    print("%s n=%d: blocked FP32 vs FP64 dense inverse: preconditioner %.2e, its %s" % (kind, n, err, its))
    assert err < 1e-4, err
    assert abs(its["0"] - its["1"]) <= 2, its


@pytest.mark.parametrize("kind,n", [("tet", 6), ("tet", 8)])
def test_scaled_face_smoothing_solve(kind, n, monkeypatch):
    """The mixed solve with the preconditioner's smoothing steps on the
    scaled face blocks (S_ef = W_e A_ef, c = W b: the self block is w I)
    against the same solve on the unscaled blocks: both meet the FP64
    residual tolerance, the solutions agree within 1e-7 and the scaled form
    needs at most 10% more inner iterations."""
    res = {}
    for scaled in ("0", "1"):
        monkeypatch.setenv("DG_SCALED_FACES", scaled)
        m, s, f, u = _setup(kind, n, 2)
        b = s.rhs(torch.tensor(f, device="cuda:0"))
        tol = 1e-10 * float(torch.linalg.norm(b))
        x = torch.zeros_like(b)
        its, r, outer = s.solve_mixed(x, b, tol)
        assert r <= tol
        res[scaled] = (its, x.clone())
    (i0, x0), (i1, x1) = res["0"], res["1"]
    assert float(torch.abs(x1 - x0).max() / torch.abs(x0).max()) < 1e-7
    print("mixed solve scaled vs unscaled: its %d / %d" % (i0, i1))
    assert i1 <= i0 + max(2, 0.1 * i0), (i0, i1)
