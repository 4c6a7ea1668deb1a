"""dg_residual_norm_noalloc, the allocation-free residual norm, against the
existing dg_residual entry point, called through the C ABI.

r must agree with dg_residual's r to 1e-14 of max|r| (the same per-thread
FP64 summation order, so it is normally bit-identical) and ||r||_2 with the
FP64 norm of that r to 1e-12 relative (only the order of the sum of squares
differs).  Two calls in a row must both pass and agree bit for bit: the
reduction order is fixed and nothing in the static scratch has to start at
zero.  The file sorts last so that it also runs after the other GPU tests
have used the library in the same process.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import element, mesh, sfc  # noqa: E402
from dg_nn_public_gb300._capi import DG_OK  # noqa: E402
from dg_nn_public_gb300.solver import DGSolver, SolverConfig  # noqa: E402


def _solver(kind, n, seed=0, kappa_sigma=0.0):
    m = mesh.build_mesh(kind, n, seed=seed)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(), element.p3_element(m.ndim))
    if kappa_sigma > 0:
        s.set_kappa(np.exp(kappa_sigma * np.random.default_rng(seed).standard_normal(m.nele)))
    s.build_operator()
    return m, s


def _call(s, x, b, r, norm_out):
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = s._lib.dg_residual_norm_noalloc(s._ctx, x.data_ptr(), None if b is None else b.data_ptr(),
                                         None if r is None else r.data_ptr(), norm_out.data_ptr(), stream)
    if rc != DG_OK:
        raise AssertionError("dg_residual_norm_noalloc returned %d: %s" % (rc, s._lib.dg_last_error(s._ctx)))


@pytest.mark.parametrize("kind,n,kappa_sigma", [("tet", 6, 0.0), ("tet", 8, 1.0), ("tri", 24, 0.0)])
def test_noalloc_residual_norm_matches_dg_residual(kind, n, kappa_sigma):
    m, s = _solver(kind, n, seed=2, kappa_sigma=kappa_sigma)
    g = torch.Generator(device="cuda:0").manual_seed(11)
    x = torch.randn(s.nonods, dtype=torch.float64, device="cuda:0", generator=g)
    b = torch.randn(s.nonods, dtype=torch.float64, device="cuda:0", generator=g)
    r_ref = s.residual(x, b)                       # existing entry point dg_residual
    nrm_ref = float(torch.linalg.norm(r_ref))
    scale = float(torch.abs(r_ref).max())
    outs = []
    for _ in range(2):                             # two calls in a row
        r = torch.full_like(x, float("nan"))
        nrm = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda:0")
        _call(s, x, b, r, nrm)
        torch.cuda.synchronize()
        assert float(torch.abs(r - r_ref).max()) <= 1e-14 * scale
        assert abs(float(nrm) - nrm_ref) <= 1e-12 * nrm_ref, (float(nrm), nrm_ref)
        outs.append((r.clone(), nrm.clone()))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])


def test_noalloc_norm_only_and_zero_rhs():
    m, s = _solver("tet", 6, seed=5)
    g = torch.Generator(device="cuda:0").manual_seed(4)
    x = torch.randn(s.nonods, dtype=torch.float64, device="cuda:0", generator=g)
    y = s.apply(x)                                 # A x, so b = NULL gives ||A x||
    nrm_ref = float(torch.linalg.norm(y))
    for _ in range(2):
        nrm = torch.zeros(1, dtype=torch.float64, device="cuda:0")
        _call(s, x, None, None, nrm)
        torch.cuda.synchronize()
        assert abs(float(nrm) - nrm_ref) <= 1e-12 * nrm_ref
    # the Python wrapper over the same entry point
    nrm = s.residual_norm_noalloc(x)
    assert abs(float(nrm) - nrm_ref) <= 1e-12 * nrm_ref


def test_noalloc_rejects_null_and_unbuilt():
    m = mesh.build_mesh("tet", 3, seed=1)
    s = DGSolver(m, sfc.hilbert_sfc_order(m.cg_coords), SolverConfig(), element.p3_element(3))
    x = torch.zeros(s.nonods, dtype=torch.float64, device="cuda:0")
    nrm = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert s._lib.dg_residual_norm_noalloc(s._ctx, x.data_ptr(), None, None, None, stream) != DG_OK
    assert s._lib.dg_residual_norm_noalloc(s._ctx, x.data_ptr(), None, None, nrm.data_ptr(), stream) != DG_OK
    assert b"not built" in s._lib.dg_last_error(s._ctx)


def test_noalloc_size_limit(monkeypatch):
    """A mesh that needs more partial sums than the scratch holds is rejected
    with DG_ERR_ARG and a message naming the limit; at the limit it runs.
    The limit is lowered for the test through DG_NOALLOC_MAX_PARTIALS, which
    can only tighten it (4^3 Kuhn cells = 384 tets = 48 CTAs of 8)."""
    from dg_nn_public_gb300._capi import DG_ERR_ARG
    m, s = _solver("tet", 4, seed=3)
    need = (m.nele + 7) // 8
    x = torch.randn(s.nonods, dtype=torch.float64, device="cuda:0")
    y = s.apply(x)
    nrm = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    monkeypatch.setenv("DG_NOALLOC_MAX_PARTIALS", str(need - 1))
    rc = s._lib.dg_residual_norm_noalloc(s._ctx, x.data_ptr(), None, None, nrm.data_ptr(), stream)
    assert rc == DG_ERR_ARG
    assert b"partial sums" in s._lib.dg_last_error(s._ctx)
    monkeypatch.setenv("DG_NOALLOC_MAX_PARTIALS", str(need))
    _call(s, x, None, None, nrm)
    torch.cuda.synchronize()
    ref = float(torch.linalg.norm(y))
    assert abs(float(nrm) - ref) <= 1e-12 * ref
    # a larger value does not raise the limit above the static array
    monkeypatch.setenv("DG_NOALLOC_MAX_PARTIALS", str(10 ** 9))
    _call(s, x, None, None, nrm)
