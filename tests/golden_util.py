"""Helpers shared by the tests: load a golden case and rebuild its inputs."""
import json
import os

import numpy as np

from dg_nn_public_gb300 import element, mesh, sfc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SMALL_CASES = ("tri3_sinh", "tri4_sin", "tet2_sin", "tet3_v22")


def load(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    meta = json.loads(str(d.pop("meta_json")))
    return d, meta


def rebuild(meta):
    """Mesh, element tables and SFC ordering exactly as the generator made them."""
    if meta["kind"] == "tri":
        g = mesh.unit_square_tri_mesh(meta["n"], seed=meta.get("seed", 0))
    else:
        g = mesh.unit_cube_kuhn_mesh(meta["n"], seed=meta.get("seed", 0))
    m = mesh.ingest(g)
    el = element.p3_element(m.ndim)
    order = sfc.hilbert_sfc_order(m.cg_coords)
    return g, m, el, order


def harness_vectors(m, seed=1234):
    """The random vectors the reference harness drew, in its order."""
    rng = np.random.default_rng(seed)
    nonods = m.nele * m.nloc
    x = rng.standard_normal(nonods)
    b = rng.standard_normal(nonods)
    r_cg = rng.standard_normal(m.cg_nonods)
    rp = rng.standard_normal(nonods)
    return x, b, r_cg, rp


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
