"""Union of meshes of uneven size (dg_nn_public_gb300.multimesh) on the CPU:
the union operator is block diagonal -- the CPU oracle's residual of the
union equals the per-mesh residuals stacked, with per-mesh kappa -- and the
union's face, vertex and curve numbering stays consistent."""
import numpy as np

from dg_nn_public_gb300 import element, mesh, sfc
from dg_nn_public_gb300.multimesh import union_mesh
from oracle.dg_oracle import OracleDG


def test_union_operator_is_block_diagonal():
    ms = [mesh.build_mesh("tet", 2, seed=1), mesh.build_mesh("tet", 3, seed=2)]
    orders = [sfc.hilbert_sfc_order(m.cg_coords) for m in ms]
    u, order, segs = union_mesh(ms, orders)
    assert u.nele == sum(m.nele for m in ms) and u.cg_nonods == sum(m.cg_nonods for m in ms)
    assert np.array_equal(np.sort(order.ravel()), np.arange(1, u.cg_nonods + 1))
    # every interior face points into its own mesh
    nbf = u.nbf.reshape(u.nele, 4)
    for sg in segs:
        f = nbf[sg.e0:sg.e1]
        f = f[f >= 0] // 4
        assert ((f >= sg.e0) & (f < sg.e1)).all()
    rng = np.random.default_rng(0)
    kap = [np.exp(0.5 * rng.standard_normal(m.nele)) for m in ms]
    el = element.p3_element(3)
    Ou = OracleDG(u, el, element.drst_duv(3), kappa=np.concatenate(kap), face_kappa="harmonic")
    x = rng.standard_normal(u.nele * 20)
    b = rng.standard_normal(u.nele * 20)
    ru = Ou.residual(x, b).ravel()
    for m, k, sg in zip(ms, kap, segs):
        O = OracleDG(m, el, element.drst_duv(3), kappa=k, face_kappa="harmonic")
        r = O.residual(x[sg.d0:sg.d1], b[sg.d0:sg.d1]).ravel()
        assert np.array_equal(ru[sg.d0:sg.d1], r)
