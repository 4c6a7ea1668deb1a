"""Meshes of uneven size in one operator on the GPU (MultiMeshSolver).

Two jittered Kuhn meshes (n = 6 and n = 8, 1,296 + 3,072 tets) with their own
log-normal kappa (harmonic face kappa): the union apply equals each mesh's
own apply bit for bit (same per-element arithmetic), and the joint mixed
and FP64 solves meet every mesh's own FP64 tolerance and agree with the
separate solves of each mesh within 1e-7 relative.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import element, mesh, sfc  # noqa: E402
from dg_nn_public_gb300.multimesh import MultiMeshSolver  # noqa: E402
from dg_nn_public_gb300.solver import DGSolver, SolverConfig  # noqa: E402


@pytest.fixture(scope="module")
def pair():
    ms = [mesh.build_mesh("tet", 6, seed=1), mesh.build_mesh("tet", 8, seed=2)]
    orders = [sfc.hilbert_sfc_order(m.cg_coords) for m in ms]
    rng = np.random.default_rng(7)
    kaps = [np.exp(0.5 * rng.standard_normal(m.nele)) for m in ms]
    fs = []
    for m in ms:
        X = m.x_ref_in
        fs.append((3 * np.pi ** 2 * np.prod([np.sin(np.pi * X[:, d]) for d in range(3)], axis=0)).ravel())
    cfg = SolverConfig(pre_smooth_its=2, post_smooth_its=2)
    mm = MultiMeshSolver(ms, orders, cfg, kappas=kaps, face_kappa="harmonic")
    singles = []
    for m, o, k in zip(ms, orders, kaps):
        s = DGSolver(m, o, cfg, element.p3_element(3))
        s.set_build_mode("affine")
        s.set_kappa(k)
        s.set_face_kappa("harmonic")
        s.build_operator()
        singles.append(s)
    yield ms, fs, mm, singles
    mm.close()
    for s in singles:
        s.close()


def test_union_apply_equals_each_mesh(pair):
    ms, fs, mm, singles = pair
    x = torch.randn(mm.solver.nonods, dtype=torch.float64, device="cuda:0")
    y = mm.solver.apply(x)
    for s, xs, ys in zip(singles, mm.split(x), mm.split(y)):
        assert torch.equal(s.apply(xs.contiguous()), ys)


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_joint_solve_matches_separate_solves(pair, mode):
    ms, fs, mm, singles = pair
    xs, its, res, tols = mm.solve(fs, rtol=1e-10, mode=mode)
    assert (res <= tols).all(), (res, tols)
    for s, f, xj, tol in zip(singles, fs, xs, tols):
        b = s.rhs(torch.tensor(f, device="cuda:0"))
        x1 = torch.zeros_like(b)
        if mode == "mixed":
            s.solve_mixed(x1, b, float(tol))
        else:
            s.gmres(x1, b, float(tol))
        d = float(torch.abs(xj - x1).max() / torch.abs(x1).max())
        print("joint %s solve vs separate: its %d, rel diff %.3e" % (mode, its, d))
        assert d < 1e-7
