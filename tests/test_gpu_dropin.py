"""The reference-compatible modules (volume_mf_diff & co.) against the golden vectors.

These call the functions with the reference's names and argument
conventions, the way the reference's driver (z06/main.py:202-206) does.
"""
import types

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from dg_nn_public_gb300 import get_bdiag_diag as gbd  # noqa: E402
from dg_nn_public_gb300 import multigrid_linearelastic as mg  # noqa: E402
from dg_nn_public_gb300 import state  # noqa: E402
from dg_nn_public_gb300 import volume_mf_diff as vmd  # noqa: E402
from golden_util import load, rebuild, rel  # noqa: E402

DEV = "cuda:0"


def T(a):
    return torch.tensor(np.asarray(a, dtype=np.float64).ravel(), device=DEV)


@pytest.fixture(scope="module", params=["tet3_v22", "tri3_sinh"])
def bound(request):
    d, meta = load(request.param)
    g, m, el, order = rebuild(meta)
    opts = meta["opts"]
    state.config.pre_smooth_its = opts.get("pre_smooth_its", 3)
    state.config.post_smooth_its = opts.get("post_smooth_its", 3)
    state.config.eta_e = 90.0
    state.config.gmres_its = opts.get("gmres_its", 400)
    state.bind(m, order, el)
    yield d, meta, m
    state.config.pre_smooth_its = 3
    state.config.post_smooth_its = 3


def test_bdiag_and_residual(bound):
    d, meta, m = bound
    gbd.get_bdiag_diag()
    assert rel(state.sf_nd_nb.bdiagK.cpu().numpy(), d["bdiagK"]) < 1e-12
    r0 = torch.zeros(m.nele * m.nloc, dtype=torch.float64, device=DEV)
    x = T(d["apply_x"])
    r, _ = vmd.get_residual_or_smooth(r0, x, T(d["apply_b"]), do_smooth=False)
    assert rel(r.cpu().numpy(), d["apply_r"]) < 1e-12
    r0.zero_()
    r, xs = vmd.get_residual_or_smooth(r0, x, T(d["apply_b"]), do_smooth=True)
    assert rel(xs.cpu().numpy(), d["smooth_x"]) < 1e-12
    # x_rhs given as the integer 0 (as the reference's Arnoldi loop does)
    r0 = torch.zeros_like(r0)
    r, _ = vmd.get_residual_or_smooth(r0, T(d["apply_x"]), 0, do_smooth=False)
    ax = -r.cpu().numpy()
    assert rel(d["apply_b"] - ax, d["apply_r"]) < 1e-12


def test_precond_vcycle_rar(bound):
    d, meta, m = bound
    xd = torch.zeros(m.nele * m.nloc, dtype=torch.float64, device=DEV)
    out = vmd._um_left_precond(xd, T(d["pc_r"]))
    assert rel(out.cpu().numpy(), d["pc_x"]) < 1e-12
    assert rel(vmd._calc_RAR_mf_color().cpu().numpy(), d["RARvalues"]) < 1e-12
    sfc, variables, nlevel, npl = mg.mg_on_P1CG_prep()
    assert nlevel == int(d["nlevel"]) and list(npl) == list(d["nodes_per_level"])
    e = mg.mg_on_P1CG(T(d["mg_r"]), variables, nlevel, npl, m.cg_nonods)
    assert rel(e.cpu().numpy(), d["mg_e"]) < 1e-12


def test_solve_for_diff_device_and_host(bound):
    d, meta, m = bound
    state.config.linear_solver = "gmres-mg"
    state.config.tol = 1e-10 * float(np.linalg.norm(d["rhs"]))
    x = torch.zeros(m.nele * m.nloc, dtype=torch.float64, device=DEV)
    ub = [T(d["g"]).view(m.nele, m.nloc)]
    x = vmd.solve_for_diff(x, T(d["f"]), ub, None)
    assert state.sf_nd_nb.its == int(d["its"])
    err = rel(x.cpu().numpy(), d["x_solution"])
    xh = torch.zeros(m.nele * m.nloc, dtype=torch.float64)
    xh = vmd.solve_for_diff(xh, torch.tensor(d["f"]).reshape(-1), [torch.tensor(d["g"])], None)
    err_h = rel(xh.numpy(), d["x_solution"])
    print("solve_for_diff vs reference: device %.3e host %.3e (max-abs rel)" % (err, err_h))
    assert err < 1e-12 and err_h < 1e-12, (err, err_h)
    l2, linf = vmd.get_l2_error(x, T(d["u_exact"]))
    assert abs(l2 - float(d["l2err"])) <= 1e-8 * float(d["l2err"])


def test_cg_and_mg_solvers_match_oracle(bound):
    """Fixed iteration counts of the CG and stand-alone MG solvers against the
    oracle's restatement of the same iterations."""
    from dg_nn_public_gb300 import element
    from oracle.dg_oracle import OracleDG
    d, meta, m = bound
    s = state.solver()
    O = OracleDG(m, s.el, element.drst_duv(m.ndim), pre_smooth_its=state.config.pre_smooth_its,
                 post_smooth_its=state.config.post_smooth_its)
    ctx = O.setup(state.sf_nd_nb.sfc_data_Um.space_filling_curve_numbering)
    saved = state.config.gmres_its
    state.config.gmres_its = 8
    try:
        for fn, ofn in ((vmd._cg_mg_solver, O.cg_mg), (vmd._mg_solver, O.mg_solve)):
            b = T(d["rhs"])
            x = torch.zeros_like(b)
            x, its = fn(x, b, 0.0)
            xo, its_o = ofn(d["rhs"], ctx, 0.0, 8)
            assert its == its_o == 8
            err = rel(x.cpu().numpy(), xo)
            print("%s vs oracle after 8 iterations: max-abs rel %.3e" % (fn.__name__, err))
            assert err < 1e-12, (fn.__name__, err)
    finally:
        state.config.gmres_its = saved


def test_bind_from_reference_objects(bound):
    """Bind from FuncSpace-like objects carrying the reference's attribute names."""
    d, meta, m = bound
    s0 = state.solver()
    el = s0.el
    elem = types.SimpleNamespace(ndim=m.ndim, n=torch.tensor(el.n), nlx=torch.tensor(el.nlx),
                                 weight=torch.tensor(el.weight), sn=torch.tensor(el.sn),
                                 snlx=torch.tensor(el.snlx), sweight=torch.tensor(el.sweight),
                                 gi_align=torch.tensor(el.gi_align))
    fs = types.SimpleNamespace(element=elem, x_ref_in=torch.tensor(m.x_ref_in), nbf=torch.tensor(m.nbf),
                               alnmt=torch.tensor(m.alnmt), glb_bcface_type=torch.tensor(m.glb_bcface_type),
                               cg_ndglno=m.cg_ndglno.reshape(-1))
    sfc_num = state.sf_nd_nb.sfc_data_Um.space_filling_curve_numbering
    state.bind_reference_funcspace(fs, sfc_num)
    r0 = torch.zeros(m.nele * m.nloc, dtype=torch.float64, device=DEV)
    r, _ = vmd.get_residual_or_smooth(r0, T(d["apply_x"]), T(d["apply_b"]))
    assert rel(r.cpu().numpy(), d["apply_r"]) < 1e-12


def test_reference_structures_checked_and_levels_returned(bound):
    """_calc_RAR_mf_color accepts the reference's own P1CG structures (golden
    fina / cola / whichc / ncolor) and refuses altered ones; mg_on_P1CG_prep
    returns the SFC levels in the reference's format with the reference's
    values; mg_on_P1CG refuses level data other than the bound operator's."""
    import scipy.sparse as sp
    d, meta, m = bound
    rar = vmd._calc_RAR_mf_color(whichc=d["whichc"], ncolor=int(d["ncolor"]), fina=d["fina"], cola=d["cola"],
                                 ncola=int(d["cola"].size))
    assert rel(rar.cpu().numpy(), d["RARvalues"]) < 1e-12
    bad = d["cola"].copy()
    bad[[0, 1]] = bad[[1, 0]]
    with pytest.raises(ValueError):
        vmd._calc_RAR_mf_color(fina=d["fina"], cola=bad)
    with pytest.raises(ValueError):
        vmd._calc_RAR_mf_color(ncolor=int(d["ncolor"]) + 1)
    sfc, variables, nlevel, npl = mg.mg_on_P1CG_prep()
    assert nlevel == int(d["nlevel"]) and list(npl) == list(d["nodes_per_level"])
    for lev in range(nlevel - 1):
        A, diag, n = variables[lev]
        assert n == npl[lev]
        assert np.array_equal(A.crow_indices().numpy(), d["lev%d_crow" % lev])
        assert np.array_equal(A.col_indices().numpy(), d["lev%d_col" % lev])
        assert rel(A.values().numpy(), d["lev%d_val" % lev]) < 1e-12
        assert rel(diag.numpy().ravel(), d["lev%d_diag" % lev]) < 1e-12
    assert isinstance(variables[-1][0], sp.csr_matrix) and variables[-1][2] == npl[-1]
    e = mg.mg_on_P1CG(T(d["mg_r"]), variables, nlevel, npl, m.cg_nonods)
    assert rel(e.cpu().numpy(), d["mg_e"]) < 1e-12
    A0, dg0, n0 = variables[0]
    altered = [(torch.sparse_csr_tensor(A0.crow_indices(), A0.col_indices(), A0.values() * 2.0, size=A0.shape),
                dg0, n0)] + list(variables[1:])
    with pytest.raises(ValueError):
        mg.mg_on_P1CG(T(d["mg_r"]), altered, nlevel, npl, m.cg_nonods)
    with pytest.raises(ValueError):
        mg.mg_on_P1CG(T(d["mg_r"]), variables, nlevel + 1, npl, m.cg_nonods)
