"""The 2D benchmark mesh (32x32x2 P3 triangles, 20,480 DOFs) against the reference.

Integer arrays are compared through SHA-256 digests of the reference's
arrays; floating-point stages against the stored reference vectors.
"""
import numpy as np
import pytest

from dg_nn_public_gb300 import element
from oracle.dg_oracle import OracleDG
from golden_util import harness_vectors, load, rebuild, rel



def _digest(a):
    import hashlib
    a = np.ascontiguousarray(a)
    h = hashlib.sha256()
    h.update(str(a.dtype.str).encode())
    h.update(str(a.shape).encode())
    h.update(a.tobytes())
    return h.hexdigest()


@pytest.fixture(scope="module")
def c1():
    d, meta = load("tri32_c1")
    g, m, el, order = rebuild(meta)
    O = OracleDG(m, el, element.drst_duv(m.ndim))
    return d, meta, m, el, order, O


def test_c1_integer_arrays(c1):
    d, meta, m, el, order, O = c1
    dig = meta["digests"]
    assert _digest(m.x_ref_in) == dig["x_ref_in"]
    assert _digest(m.nbf) == dig["nbf"]
    assert _digest(m.alnmt) == dig["alnmt"]
    assert _digest(m.glb_bcface_type) == dig["glb_bcface_type"]
    assert _digest(order) == dig["sfc"]
    pc = O.p1cg()
    assert _digest(pc["fina"].astype(np.int32)) == dig["fina"]
    assert _digest(pc["cola"].astype(np.int32)) == dig["cola"]
    assert _digest(pc["whichc"]) == dig["whichc"]


def test_c1_stages(c1):
    d, meta, m, el, order, O = c1
    x, b, r_cg, rp = harness_vectors(m)
    assert rel(O.residual(x, b), d["apply_r"]) < 5e-13
    ctx = O.setup(order)
    assert rel(ctx["rar"], d["RARvalues"]) < 5e-13
    assert rel(O.mg_on_p1cg(r_cg, ctx["levels"], ctx["sizes"]), d["mg_e"]) < 5e-13
    assert rel(O.precond(rp, ctx), d["pc_x"]) < 5e-13


@pytest.mark.slow
def test_c1_gmres(c1):
    d, meta, m, el, order, O = c1
    ctx = O.setup(order)
    xr = np.asarray(m.x_ref_in)
    f = 2 * np.pi ** 2 * np.sin(np.pi * xr[:, 0]) * np.sin(np.pi * xr[:, 1])
    bvec = O.rhs(f, np.zeros_like(f))
    assert rel(bvec, d["rhs"]) < 5e-13
    x, its, hist = O.gmres(bvec, ctx, 1e-10 * np.linalg.norm(bvec))
    assert its == int(d["its"])
    assert rel(x, d["x_solution"]) < 1e-11
