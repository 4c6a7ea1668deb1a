"""Batched mixed-precision solve (dg_solve_mixed_batched): several right-hand
sides in lockstep on one operator, against the single-RHS mixed solve and
the FP64 residual.

Every RHS must reach ||b_q - A x_q|| <= 1e-10 ||b_q|| in FP64 (checked here
independently with dg_residual), and its solution must agree with the
single-RHS solve of the same system to 1e-7 relative (two approximations of
the same discrete solution, each within the tolerance).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import element, mesh, sfc  # noqa: E402
from dg_nn_public_gb300.solver import DGSolver, SolverConfig  # noqa: E402


def _modes(m, nrhs, seed):
    """f = sum of 8 Fourier modes (integer wavenumbers 1..4, N(0,1) amplitudes)."""
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


@pytest.mark.parametrize("n,nrhs", [(6, 5), (5, 64)])
def test_batched_matches_single(n, nrhs):
    m = mesh.build_mesh("tet", n, seed=1)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                 element.p3_element(3))
    s.build_operator()
    F = _modes(m, nrhs, seed=n)
    Bm = torch.stack([s.rhs(torch.tensor(F[q], device="cuda:0")) for q in range(nrhs)]).contiguous()
    tol = 1e-10 * torch.linalg.norm(Bm, dim=1).cpu().numpy()
    X = torch.zeros_like(Bm)
    its, res = s.solve_mixed_batched(X, Bm, tol, raise_noconv=True)
    assert (res <= tol).all()
    for q in range(nrhs):
        r = s.residual(X[q].contiguous(), Bm[q].contiguous())
        assert float(torch.linalg.norm(r)) <= tol[q] * (1 + 1e-9)
    for q in list(range(min(nrhs, 3))) + [nrhs - 1]:
        x1 = torch.zeros_like(Bm[q])
        s.solve_mixed(x1, Bm[q].contiguous(), float(tol[q]))
        d = float(torch.abs(X[q] - x1).max() / torch.abs(x1).max())
        assert d < 1e-7, (q, d)
    assert its.max() > 0


def test_batched_nonzero_guess_and_converged_rhs():
    """A RHS whose initial guess already solves it stays untouched (0 its);
    the others converge."""
    m = mesh.build_mesh("tet", 5, seed=3)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                 element.p3_element(3))
    s.build_operator()
    F = _modes(m, 3, seed=9)
    Bm = torch.stack([s.rhs(torch.tensor(F[q], device="cuda:0")) for q in range(3)]).contiguous()
    tol = 1e-10 * torch.linalg.norm(Bm, dim=1).cpu().numpy()
    x1 = torch.zeros_like(Bm[1])
    s.solve_mixed(x1, Bm[1].contiguous(), float(tol[1]) * 1e-2)
    X = torch.zeros_like(Bm)
    X[1] = x1
    X1_before = X[1].clone()
    its, res = s.solve_mixed_batched(X, Bm, tol, raise_noconv=True)
    assert its[1] == 0 and torch.equal(X[1], X1_before)
    assert its[0] > 0 and its[2] > 0 and (res <= tol).all()


@pytest.mark.parametrize("variant", [("DG_BATCHED_TMA", "1"), ("DG_BATCHED_WARPS", "8")])
def test_smoothing_kernel_forms_agree(monkeypatch, variant):
    """The persistent bulk-copy form and the 8-warp form of the batched
    tensor-core smoothing kernel do the same arithmetic as the default
    (one CTA of 4 warps per element): the whole batched solve is bitwise
    identical with any of them."""
    out = {}
    for tma in ("1", "0"):
        if tma == "1":
            monkeypatch.setenv(*variant)
        else:
            monkeypatch.delenv(variant[0], raising=False)
        m = mesh.build_mesh("tet", 5, seed=2)
        s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(pre_smooth_its=2, post_smooth_its=2),
                     element.p3_element(3))
        s.build_operator()
        F = _modes(m, 6, seed=3)
        Bm = torch.stack([s.rhs(torch.tensor(F[q], device="cuda:0")) for q in range(6)]).contiguous()
        tol = 1e-10 * torch.linalg.norm(Bm, dim=1).cpu().numpy()
        X = torch.zeros_like(Bm)
        its, res = s.solve_mixed_batched(X, Bm, tol, raise_noconv=True)
        out[tma] = (X, its)
    assert torch.equal(out["1"][0], out["0"][0])
    assert (out["1"][1] == out["0"][1]).all()
