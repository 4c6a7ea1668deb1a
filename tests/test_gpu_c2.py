"""The 3D benchmark solve (48,000 P3 tets, 960,000 DOFs) against the reference's own run.

The reference solved this exact mesh and right-hand side on CPU in FP64
(tests/golden/make_golden.py, c2_summary); the GPU path must take the same
number of GMRES iterations and reproduce the solution within 1e-12 relative
(max-abs over the sampled entries; both Arnoldi orthogonalisations, the
error printed), the operator apply within 1e-12.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import element, mesh, sfc  # noqa: E402
from dg_nn_public_gb300.solver import DGSolver, SolverConfig  # noqa: E402
from golden_util import harness_vectors, load, rel  # noqa: E402


@pytest.fixture(scope="module")
def c2():
    d, meta = load("tet20_c2_summary")
    m = mesh.build_mesh("tet", 20, seed=0)
    order = sfc.hilbert_sfc_order(m.cg_coords)
    s = DGSolver(m, order, SolverConfig(pre_smooth_its=2, post_smooth_its=2), element.p3_element(3))
    s.build_operator()
    return d, meta, m, s


def test_c2_apply_and_rar(c2):
    d, meta, m, s = c2
    x, b, _, _ = harness_vectors(m)
    r = s.residual(torch.tensor(x, device="cuda:0"), torch.tensor(b, device="cuda:0")).cpu().numpy()
    assert rel(r[::97], d["apply_r_sub"]) < 1e-12
    assert rel(s.rar_values().cpu().numpy()[::7], d["rar_sub"]) < 1e-12
    assert int(s.info()["ncolor"]) == int(d["ncolor"])


@pytest.mark.parametrize("ortho", ["cgs2", "mgs"])
def test_c2_solve_matches_reference(c2, ortho):
    d, meta, m, s = c2
    X = m.x_ref_in
    f = 3 * np.pi ** 2 * np.prod([np.sin(np.pi * X[:, k]) for k in range(3)], axis=0).ravel()
    b = s.rhs(torch.tensor(f, device="cuda:0"))
    assert abs(float(torch.linalg.norm(b)) - float(d["rhs_norm"])) <= 1e-12 * float(d["rhs_norm"])
    tol = 1e-10 * float(d["rhs_norm"])
    x = torch.zeros_like(b)
    s.set_gmres_ortho(ortho)
    try:
        its, res = s.gmres(x, b, tol)
    finally:
        s.set_gmres_ortho("cgs2")
    xn = x.cpu().numpy()
    err = rel(xn[::97], d["x_sub"])
    print("c2 GMRES solution vs reference: ortho %s its %d max-abs rel err %.3e (sampled every 97th)" % (ortho, its, err))
    assert its == int(d["its"])
    assert res <= tol
    assert err < 1e-12, (ortho, err)
    assert abs(np.linalg.norm(xn) - float(d["x_norm"])) <= 1e-12 * float(d["x_norm"])
    u = np.prod([np.sin(np.pi * X[:, k]) for k in range(3)], axis=0).ravel()
    # solutions agreeing to 1e-12 relative move the nodal error by <= ~1e-12
    assert abs(np.abs(xn - u).max() - float(d["linferr"])) <= 1e-11
