"""Kernel variants of the batched BF16 smoothing step on 64 RHS-interleaved
right-hand sides, through dg_smooth_pc_batched and the batched solve.

Variant 0 (CUDA cores, FP32 x) is the reference here; the tensor-core
variants (mma.sync tiles, mma.sync bulk-copy, tcgen05 with tensor-memory
accumulators) split x into BF16 high + low parts, so they agree with it to
the ~16 bits x keeps: max-abs difference <= 1e-4 of max |X_out| (a layout
error gives O(1)).  The batched solve with the tcgen05 kernel must meet every
FP64 tolerance and agree with the single-RHS solve within 1e-7, and the
autotuner must time every variant and keep the fastest.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import element, mesh, sfc  # noqa: E402
from dg_nn_public_gb300.solver import DGSolver, SolverConfig  # noqa: E402

KERNELS = DGSolver.BATCHED_KERNELS


@pytest.fixture(scope="module")
def tet5():
    m = mesh.build_mesh("tet", 5, seed=4)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                 element.p3_element(3))
    s.set_kappa(np.exp(0.5 * np.random.default_rng(3).standard_normal(m.nele)))
    s.build_operator()
    yield m, s
    s.close()


def _rel(a, b):
    return float(torch.abs(a - b).max() / torch.abs(b).max())


@pytest.mark.parametrize("zero_guess", [False, True])
def test_smoothing_kernels_agree(tet5, zero_guess):
    m, s = tet5
    g = torch.Generator(device="cuda:0").manual_seed(9)
    X = torch.randn(s.nonods * 64, dtype=torch.float32, device="cuda:0", generator=g)
    B = torch.randn(s.nonods * 64, dtype=torch.float32, device="cuda:0", generator=g)
    outs = {}
    for k in KERNELS:
        s.set_batched_kernel(k)
        outs[k] = s.smooth_pc_batched(None if zero_guess else X, B).clone()
        again = s.smooth_pc_batched(None if zero_guess else X, B)
        assert torch.equal(outs[k], again), k          # deterministic
    torch.cuda.synchronize()
    for k in KERNELS[1:]:
        err = _rel(outs[k], outs["cuda_cores"])
        print("batched smoothing %s vs cuda_cores (zero guess %s): %.3e" % (k, zero_guess, err))
        assert err < 1e-4, (k, err)
    s.set_batched_kernel("auto")


def test_batched_apply_matches_single_rhs(tet5):
    """Y = A X for 64 interleaved RHS equals 64 single-RHS FP32 applies."""
    m, s = tet5
    g = torch.Generator(device="cuda:0").manual_seed(2)
    X = torch.randn(s.nonods, 64, dtype=torch.float32, device="cuda:0", generator=g)
    Y = s.apply_batched(X.reshape(-1).contiguous()).reshape(s.nonods, 64)
    for q in (0, 17, 63):
        y1 = s.apply_f32(X[:, q].contiguous())
        assert _rel(Y[:, q], y1) < 1e-6, q


def _modes(m, nrhs, seed):
    rng = np.random.default_rng(seed)
    X = m.x_ref_in
    F = np.zeros((nrhs, m.nele * m.nloc))
    for q in range(nrhs):
        f = np.zeros((m.nele, m.nloc))
        for _ in range(8):
            k = rng.integers(1, 5, size=3)
            a = rng.standard_normal()
            f += a * np.pi ** 2 * float((k ** 2).sum()) * np.prod(
                [np.sin(k[d] * np.pi * X[:, d]) for d in range(3)], axis=0)
        F[q] = f.reshape(-1)
    return F


@pytest.mark.parametrize("kernel", ["tcgen05_bulk", "tcgen05_split", "tcgen05_ws"])
def test_batched_solve_with_tcgen05_kernel(kernel):
    """The kernel pinned before the first batched solve (the autotuner does
    not run): for the split form the preconditioner keeps its iterates in
    the operand layout from the first smoothing step to the last."""
    m = mesh.build_mesh("tet", 6, seed=1)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                 element.p3_element(3))
    s.build_operator()
    s.set_batched_kernel(kernel)
    nrhs = 12
    F = _modes(m, nrhs, seed=5)
    Bm = torch.stack([s.rhs(torch.tensor(F[q], device="cuda:0")) for q in range(nrhs)]).contiguous()
    tol = 1e-10 * torch.linalg.norm(Bm, dim=1).cpu().numpy()
    X = torch.zeros_like(Bm)
    its, res = s.solve_mixed_batched(X, Bm, tol, raise_noconv=True)
    assert (res <= tol).all()
    for q in range(nrhs):
        r = s.residual(X[q].contiguous(), Bm[q].contiguous())
        assert float(torch.linalg.norm(r)) <= tol[q] * (1 + 1e-9)
    for q in (0, nrhs - 1):
        x1 = torch.zeros_like(Bm[q])
        s.solve_mixed(x1, Bm[q].contiguous(), float(tol[q]))
        d = float(torch.abs(X[q] - x1).max() / torch.abs(x1).max())
        assert d < 1e-7, (q, d)
    print("%s batched solve: its" % kernel, its.tolist())
    s.close()


def test_autotuner_times_every_variant():
    m = mesh.build_mesh("tet", 4, seed=2)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                 element.p3_element(3))
    s.build_operator()
    s.set_batched_kernel("auto")
    Bm = torch.stack([s.rhs(torch.ones(s.nonods, dtype=torch.float64, device="cuda:0"))] * 2).contiguous()
    X = torch.zeros_like(Bm)
    s.solve_mixed_batched(X, Bm, 1e-8 * torch.linalg.norm(Bm, dim=1).cpu().numpy())
    chosen, us = s.batched_tuning()
    print("batched autotuner:", chosen, us)
    assert set(us) == set(KERNELS)
    assert us[chosen] == min(us.values())
    s.close()


@pytest.mark.parametrize("kernel", ["mma_sync4", "tcgen05_ws"])
def test_batched_step_graphs_match_direct_launches(kernel):
    """Each inner Arnoldi step of the batched solve is replayed as one CUDA
    graph (captured at its first use): the solve must give the same
    iterates as direct launches, count the same kernels, and capture again
    when the smoothing kernel changes between solves."""
    from dg_nn_public_gb300 import _capi
    m = mesh.build_mesh("tet", 5, seed=3)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                 element.p3_element(3))
    s.build_operator()
    nrhs = 6
    F = _modes(m, nrhs, seed=8)
    Bm = torch.stack([s.rhs(torch.tensor(F[q], device="cuda:0")) for q in range(nrhs)]).contiguous()
    tol = 1e-10 * torch.linalg.norm(Bm, dim=1).cpu().numpy()

    def run(graph, k):
        s.set_launch_options(use_graph=graph)
        s.set_batched_kernel(k)
        X = torch.zeros_like(Bm)
        torch.cuda.synchronize()
        l0 = _capi.launch_count()
        its, res = s.solve_mixed_batched(X, Bm, tol, raise_noconv=True)
        torch.cuda.synchronize()
        return X, its, _capi.launch_count() - l0

    other = "cuda_cores"
    run(False, kernel)                    # first solve: builds the mixed operator copies
    Xd, itd, nd = run(False, kernel)
    Xg, itg, ng = run(True, kernel)       # captures
    Xr, itr, nr = run(True, kernel)       # replays
    Xo, ito, _ = run(True, other)         # new kernel: captured again
    Xod, itod, _ = run(False, other)
    print("%s: its %s, kernels direct %d / graph %d / replay %d" % (kernel, itd.tolist(), nd, ng, nr))
    assert itg.tolist() == itd.tolist() and itr.tolist() == itd.tolist()
    assert nd == ng == nr
    for Xa in (Xg, Xr):
        assert float(torch.abs(Xa - Xd).max() / torch.abs(Xd).max()) < 1e-12
    assert ito.tolist() == itod.tolist()
    assert float(torch.abs(Xo - Xod).max() / torch.abs(Xod).max()) < 1e-12
    s.set_launch_options(use_graph=True)
    s.close()


def test_scaled_batched_step_matches_single_rhs(tet5):
    """The batched smoothing step on the scaled face blocks (X + C - w X -
    sum_f S_f X_f, tensor cores with x split into BF16 hi + lo) against the
    single-RHS step on the same blocks (FP32 x, CUDA cores), column by
    column: the split keeps ~16 bits of x, so max-abs <= 1e-4 of max |y|."""
    m, s = tet5
    assert s.info()["scaled_faces"] == 1
    g = torch.Generator(device="cuda:0").manual_seed(12)
    X = torch.randn(s.nonods, 64, dtype=torch.float32, device="cuda:0", generator=g)
    C = torch.randn(s.nonods, 64, dtype=torch.float32, device="cuda:0", generator=g)
    Y = s.smooth_scaled_batched(X.reshape(-1).contiguous(), C.reshape(-1).contiguous()).reshape(s.nonods, 64)
    again = s.smooth_scaled_batched(X.reshape(-1).contiguous(), C.reshape(-1).contiguous()).reshape(s.nonods, 64)
    assert torch.equal(Y, again)
    for q in (0, 31, 63):
        y1 = s.smooth_scaled(X[:, q].contiguous(), C[:, q].contiguous())
        err = _rel(Y[:, q], y1)
        print("scaled batched step vs single RHS, column %d: %.3e" % (q, err))
        assert err < 1e-4, (q, err)


def test_batched_solve_scaled_faces_on_off(monkeypatch):
    """The batched solve with its smoothing steps on the scaled face blocks
    and on the unscaled blocks (DG_SCALED_FACES=0): both meet every FP64
    tolerance, their solutions agree within 1e-7 and the scaled form needs
    at most 10% more iterations (with the default 5-step Chebyshev smoothing
    it needs fewer: 27 against 33 here)."""
    m = mesh.build_mesh("tet", 6, seed=2)
    F = _modes(m, 8, seed=7)
    out = {}
    for scaled in ("0", "1"):
        monkeypatch.setenv("DG_SCALED_FACES", scaled)
        s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                     element.p3_element(3))
        s.build_operator()
        s.set_batched_kernel("mma_sync4")
        assert s.info()["scaled_faces"] == int(scaled)
        Bm = torch.stack([s.rhs(torch.tensor(F[q], device="cuda:0")) for q in range(len(F))]).contiguous()
        tol = 1e-10 * torch.linalg.norm(Bm, dim=1).cpu().numpy()
        X = torch.zeros_like(Bm)
        its, res = s.solve_mixed_batched(X, Bm, tol, raise_noconv=True)
        assert (res <= tol).all()
        out[scaled] = (int(max(its)), X.clone())
        s.close()
    (i0, x0), (i1, x1) = out["0"], out["1"]
    d = float(torch.abs(x1 - x0).max() / torch.abs(x0).max())
    print("batched solve scaled vs unscaled: its %d / %d, max rel diff %.3e" % (i0, i1, d))
    assert d < 1e-7
    assert i1 <= i0 + max(2, 0.1 * i0)
