"""Pin the CPU oracle and the mesh/element setup to the reference's own outputs.

The golden vectors come from running the reference's z06 Python on CPU
(tests/golden/make_golden.py).  Integer arrays must match exactly; floating
point stages within a few units of roundoff of the FP64 reference.
"""
import os

import numpy as np
import pytest

from dg_nn_public_gb300 import element
from oracle.dg_oracle import OracleDG, upsample_index
from golden_util import SMALL_CASES, load, rebuild, rel

FP_TOL = 5e-13      # relative (max-abs) tolerance for single FP64 stages
SOL_TOL = 1e-11     # relative tolerance on the GMRES solution


@pytest.fixture(scope="module", params=SMALL_CASES)
def case(request):
    d, meta = load(request.param)
    g, m, el, order = rebuild(meta)
    opts = meta["opts"]
    O = OracleDG(m, el, element.drst_duv(m.ndim), eta_e=opts.get("eta_e", 90.0),
                 pre_smooth_its=opts.get("pre_smooth_its", 3),
                 post_smooth_its=opts.get("post_smooth_its", 3))
    return d, meta, m, el, order, O


def test_mesh_ingest_bit_exact(case):
    d, meta, m, el, order, O = case
    assert np.array_equal(m.x_ref_in, d["x_ref_in"])
    assert np.array_equal(m.nbf, d["nbf"])
    assert np.array_equal(m.alnmt, d["alnmt"])
    assert np.array_equal(m.glb_bcface_type, d["glb_bcface_type"])
    assert np.array_equal(m.cg_ndglno, d["cg_ndglno"])
    assert np.array_equal(np.asarray(m.bc_node_list), d["bc_node_list"])
    assert np.array_equal(order, d["sfc"])


def test_element_tables(case):
    d, meta, m, el, order, O = case
    for k in ("n", "nlx", "weight", "sn", "snlx", "sweight"):
        a, b = getattr(el, k), d["el_" + k]
        assert a.shape == b.shape
        assert np.abs(a - b).max() < 1e-13, k
    assert np.array_equal(el.gi_align, d["el_gi_align"])


def test_operator_stages(case):
    d, meta, m, el, order, O = case
    assert rel(O.residual(d["apply_x"], d["apply_b"]), d["apply_r"]) < FP_TOL
    K, dK = O.bdiag()
    assert rel(K, d["bdiagK"]) < FP_TOL
    assert rel(dK, d["diagK"]) < FP_TOL
    rs, xs = O.smooth(d["apply_x"], d["apply_b"], K, dK)
    assert rel(rs, d["smooth_r"]) < FP_TOL
    assert rel(xs, d["smooth_x"]) < FP_TOL
    assert rel(O.rhs(d["f"], d["g"]), d["rhs"]) < FP_TOL


def test_p1cg_structures_exact(case):
    d, meta, m, el, order, O = case
    pc = O.p1cg()
    assert np.array_equal(pc["fina"], d["fina"])
    assert np.array_equal(pc["cola"], d["cola"])
    assert np.array_equal(pc["whichc"], d["whichc"])
    assert pc["ncolor"] == int(d["ncolor"])
    # I_cf rows: the DG copies of each vertex with weight 1/#copies
    crow, col, val = d["I_cf_crow"], d["I_cf_col"], d["I_cf_val"]
    p1 = m.p1cg.ravel()
    for i in range(m.cg_nonods):
        cols = np.sort(col[crow[i]:crow[i + 1]])
        assert np.array_equal(cols, np.nonzero(p1 == i)[0])
        assert np.allclose(val[crow[i]:crow[i + 1]], 1.0 / cols.size, rtol=0, atol=1e-16)


def test_sfc_hierarchy_and_vcycle(case):
    d, meta, m, el, order, O = case
    ctx = O.setup(order)
    assert rel(ctx["rar"], d["RARvalues"]) < FP_TOL
    assert ctx["nlevel"] == int(d["nlevel"])
    assert list(ctx["sizes"]) == list(d["nodes_per_level"])
    for lev in range(ctx["nlevel"] - 1):
        A, dg = ctx["levels"][lev]
        assert np.array_equal(A.indptr, d["lev%d_crow" % lev])
        assert np.array_equal(A.indices, d["lev%d_col" % lev])
        assert rel(A.data, d["lev%d_val" % lev]) < FP_TOL
        assert rel(dg, d["lev%d_diag" % lev]) < FP_TOL
    assert rel(O.mg_on_p1cg(d["mg_r"], ctx["levels"], ctx["sizes"]), d["mg_e"]) < FP_TOL
    assert rel(O.precond(d["pc_r"], ctx), d["pc_x"]) < FP_TOL


def test_gmres_solution(case):
    d, meta, m, el, order, O = case
    ctx = O.setup(order)
    opts = meta["opts"]
    tol = opts.get("rtol", 1e-10) * np.linalg.norm(d["rhs"])
    x, its, hist = O.gmres(d["rhs"], ctx, tol, m=opts.get("gmres_m", 30),
                           max_its=opts.get("gmres_its", 400))
    assert its == int(d["its"])
    assert rel(x, d["x_solution"]) < SOL_TOL
    l2, linf = O.l2_error(x, d["u_exact"])
    assert abs(l2 - float(d["l2err"])) <= 1e-10 * abs(float(d["l2err"]))


def test_upsample_index_matches_torch():
    torch = pytest.importorskip("torch")
    for nf in list(range(2, 80)) + [1157, 2315, 4631, 9261, 68921, 137841]:
        nc = (nf - 1) // 2 + 1
        up = torch.nn.Upsample(scale_factor=nf / nc)
        src = torch.arange(nc, dtype=torch.float64).view(1, 1, -1)
        got = up(src).view(-1).numpy().astype(np.int64)
        assert np.array_equal(got, upsample_index(nf, nc)), nf


def test_face_kappa_coercivity_under_a_kappa_jump():
    """kappa = 1 except one neighbour of an interior element at 1000: with the
    reference's arithmetic face mean, that face's consistency terms carry
    kappa ~ 500 against the element's volume term of 1, and its diagonal
    block is indefinite; the harmonic face mean (weighted-average SIP) keeps
    every diagonal block positive definite (smallest/largest eigenvalue
    ~0.056) and the operator symmetric."""
    from dg_nn_public_gb300 import element, mesh
    from oracle.dg_oracle import OracleDG
    m = mesh.build_mesh("tet", 3, seed=0)
    nbf = np.asarray(m.nbf).reshape(m.nele, 4)
    t = np.asarray(m.glb_bcface_type).reshape(m.nele, 4)
    e = [k for k in range(m.nele) if (t[k] < 0).all()][0]
    kappa = np.ones(m.nele)
    kappa[int(nbf[e, 0]) // 4] = 1000.0
    el = element.p3_element(3)
    lo = {}
    for mode in ("mean", "harmonic"):
        O = OracleDG(m, el, element.drst_duv(3), kappa=kappa, face_kappa=mode)
        K = O.bdiag()[0]
        ev = np.linalg.eigvalsh(K[e])
        lo[mode] = ev[0] / ev[-1]
        if mode == "harmonic":
            assert all(np.linalg.eigvalsh(K[k])[0] > 0 for k in range(m.nele))
            rng = np.random.default_rng(0)
            x, y = rng.standard_normal((2, m.nele * m.nloc))
            xAy, yAx = x @ O.apply_Ax(y).reshape(-1), y @ O.apply_Ax(x).reshape(-1)
            assert abs(xAy - yAx) <= 1e-12 * abs(xAy)
    assert lo["mean"] < 0 < 0.05 < lo["harmonic"], lo


def test_vtk_node_order_matches_reference_tables():
    """The VTK permutation derived from the barycentric node tables equals
    the reference's hand-written tables (fixture extracted from its source)."""
    import os
    from dg_nn_public_gb300.output import vtk_node_order
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "vtk_node_order.npz"))
    assert (vtk_node_order(3) == d["tet"]).all()
    assert (vtk_node_order(2) == d["tri"]).all()


def test_write_vtu_roundtrip(tmp_path):
    """The VTU lists every DG node once, cells in VTK order, and the field."""
    import xml.etree.ElementTree as ET
    from dg_nn_public_gb300 import mesh
    from dg_nn_public_gb300.output import write_vtu, vtk_node_order
    m = mesh.build_mesh("tet", 2, seed=0)
    u = np.arange(m.nele * m.nloc, dtype=np.float64)
    p = write_vtu(str(tmp_path / "u.vtu"), m.x_ref_in, {"u": u})
    root = ET.parse(p).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == m.nele * 20 and int(piece.get("NumberOfCells")) == m.nele
    conn = np.array(piece.find("Cells/DataArray[@Name='connectivity']").text.split(), dtype=np.int64)
    assert (conn.reshape(m.nele, 20)[1] == 20 + vtk_node_order(3)).all()
    vals = np.array(piece.find("PointData/DataArray[@Name='u']").text.split(), dtype=np.float64)
    assert np.array_equal(vals, u)


@pytest.mark.parametrize("kind,n", [("tet", 2), ("tri", 4)])
def test_colour_probe_rar_equals_galerkin_product(kind, n):
    """The colour-probe P1CG operator (one apply per colour of a distance-2
    colouring) is the Galerkin product I_cf A I_fc entry for entry: a
    direct assembly from the element blocks has to reproduce exactly these
    values (up to summation order).  Dense products on a small jittered mesh
    with log-normal kappa."""
    from dg_nn_public_gb300 import mesh
    m = mesh.build_mesh(kind, n, seed=3)
    el = element.p3_element(m.ndim)
    kap = np.exp(0.6 * np.random.default_rng(2).standard_normal(m.nele))
    O = OracleDG(m, el, element.drst_duv(m.ndim), eta_e=90.0, kappa=kap)
    pc = O.p1cg()
    probe = O.rar(pc)
    ndg, ncg = m.nele * m.nloc, m.cg_nonods
    eye_dg, eye_cg = np.eye(ndg), np.eye(ncg)
    A = np.stack([O.apply_Ax(eye_dg[i]).ravel() for i in range(ndg)], axis=1)
    P = np.stack([O.prolong_from_cg(eye_cg[j], pc).ravel() for j in range(ncg)], axis=1)
    R = np.stack([O.restrict_to_cg(eye_dg[i], pc) for i in range(ndg)], axis=1)
    G = R @ A @ P
    rows = np.repeat(np.arange(ncg), np.diff(pc["fina"]))
    direct = G[rows, pc["cola"]]
    assert np.abs(direct - probe).max() <= 1e-12 * np.abs(probe).max()
    # and nothing of the product lies outside the P1CG sparsity
    mask = np.zeros((ncg, ncg), dtype=bool)
    mask[rows, pc["cola"]] = True
    assert np.abs(G[~mask]).max(initial=0.0) <= 1e-12 * np.abs(probe).max()


def test_kappa_convention_matches_reference_varprop():
    """The per-element diffusivity convention (kappa_e in the volume term,
    (kappa_e + kappa_nb)/2 on the three interior-face terms, kappa_e on
    boundary faces) against the reference's own variable-property residual
    (z05-ns/volume_mf_um_diff_varprop.py:347-395, run by
    oracle/refrun/run_varprop.py on the tet3_v22 mesh arrays with log-normal
    kappa, sigma 1).  The reference solves for a 3-component field whose
    operator is the scalar one times the identity, so every component must
    equal the scalar residual."""
    d, meta = load("tet3_v22")
    g, m, el, order = rebuild(meta)
    v = np.load(os.path.join(os.path.dirname(__file__), "golden", "varprop_tet3.npz"))
    O = OracleDG(m, el, element.drst_duv(3), eta_e=float(v["eta_e"]), kappa=v["kappa"], face_kappa="mean")
    for k in range(3):
        r = O.residual(v["x"][:, :, k].ravel(), v["b"][:, :, k].ravel())
        assert rel(r, v["r"][:, :, k]) < FP_TOL, k
