"""Direct Galerkin P1CG assembly (per-block products P^T A_b P summed over
fixed contribution lists) against the colour-probe assembly of the
reference (z06/volume_mf_diff.py:1696-1754) on the GPU.

The same mesh is built twice, with DG_RAP_DIRECT=0 (one operator apply per
colour of the distance-2 colouring) and DG_RAP_DIRECT=1 (block_galerkin_kernel
+ rap_gather_kernel); the P1CG values must agree within 1e-12 relative
(max-abs), on the golden cases also with the reference's own RARvalues, with
and without a log-normal per-element kappa, and at the 3D benchmark size
against the reference's sampled values.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import element, mesh, sfc  # noqa: E402
from dg_nn_public_gb300.solver import DGSolver, SolverConfig  # noqa: E402
from golden_util import SMALL_CASES, load, rebuild, rel  # noqa: E402

TOL = 1e-12


def _rar(monkeypatch, m, order, el, cfg, direct, kappa=None, face_kappa="mean"):
    monkeypatch.setenv("DG_RAP_DIRECT", "1" if direct else "0")
    s = DGSolver(m, order, cfg, el)
    try:
        if kappa is not None:
            s.set_kappa(kappa)
            s.set_face_kappa(face_kappa)
        s.build_operator()
        return s.rar_values().cpu().numpy(), s.info()
    finally:
        s.close()


@pytest.mark.parametrize("name", list(SMALL_CASES) + ["tri32_c1"])
def test_direct_rar_equals_probes_and_reference(name, monkeypatch):
    d, meta = load(name)
    g, m, el, order = rebuild(meta)
    opts = meta["opts"]
    cfg = SolverConfig(eta_e=opts.get("eta_e", 90.0), pre_smooth_its=opts.get("pre_smooth_its", 3),
                       post_smooth_its=opts.get("post_smooth_its", 3))
    probe, _ = _rar(monkeypatch, m, order, el, cfg, False)
    direct, _ = _rar(monkeypatch, m, order, el, cfg, True)
    e_pd, e_ref = rel(direct, probe), rel(direct, d["RARvalues"])
    print("direct P1CG values %s: vs probes %.3e, vs reference %.3e" % (name, e_pd, e_ref))
    assert e_pd < TOL and e_ref < TOL


@pytest.mark.parametrize("kind,n,face_kappa", [("tet", 4, "mean"), ("tet", 5, "harmonic"), ("tri", 8, "mean")])
def test_direct_rar_with_kappa(kind, n, face_kappa, monkeypatch):
    m = mesh.build_mesh(kind, n, seed=2)
    order = sfc.hilbert_sfc_order(m.cg_coords)
    el = element.p3_element(m.ndim)
    kap = np.exp(np.random.default_rng(4).standard_normal(m.nele))
    probe, _ = _rar(monkeypatch, m, order, el, SolverConfig(), False, kap, face_kappa)
    direct, _ = _rar(monkeypatch, m, order, el, SolverConfig(), True, kap, face_kappa)
    err = rel(direct, probe)
    print("direct P1CG values %s n=%d kappa (%s faces): vs probes %.3e" % (kind, n, face_kappa, err))
    assert err < TOL


def test_direct_rar_c2(monkeypatch):
    d, meta = load("tet20_c2_summary")
    m = mesh.build_mesh("tet", 20, seed=0)
    order = sfc.hilbert_sfc_order(m.cg_coords)
    el = element.p3_element(3)
    cfg = SolverConfig(pre_smooth_its=2, post_smooth_its=2)
    direct, _ = _rar(monkeypatch, m, order, el, cfg, True)
    probe, _ = _rar(monkeypatch, m, order, el, cfg, False)
    e_pd, e_ref = rel(direct, probe), rel(direct[::7], d["rar_sub"])
    print("direct P1CG values c2: vs probes %.3e, vs reference (sampled) %.3e" % (e_pd, e_ref))
    assert e_pd < TOL and e_ref < TOL
