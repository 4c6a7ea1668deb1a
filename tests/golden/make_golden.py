"""Generate the golden vectors the oracle and the CUDA path are pinned to.

Run in a checkout next to the reference (it executes the reference's own
z06 Python on CPU through ``oracle/refrun``; $DG_REFERENCE_DIR names the
reference checkout):

    DG_REFERENCE_DIR=/path/to/reference python tests/golden/make_golden.py [case ...]

``varprop_tet3`` runs the reference's variable-property residual
(z05-ns/volume_mf_um_diff_varprop.py) on the mesh arrays and element tables
of the ``tet3_v22`` golden case (oracle/refrun/run_varprop.py).

Each case builds a synthetic mesh with this package's generator, writes it
as a Gmsh v2 file plus the SFC ordering the reference reads from its cache,
runs the reference in a subprocess and stores a compressed ``.npz`` here.
Small meshes keep every intermediate; the 2D benchmark mesh keeps hashes of
its integer arrays and the vectors that are not reproducible from a seed.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from dg_nn_public_gb300 import mesh as dgmesh  # noqa: E402
from dg_nn_public_gb300 import sfc as dgsfc  # noqa: E402

# name: (kind, n, options)
CASES = {
    "tri3_sinh": ("tri", 3, dict(problem="sinh2d", gmres_its=90)),
    "tri4_sin": ("tri", 4, dict(problem="sin", gmres_its=90)),
    "tet2_sin": ("tet", 2, dict(problem="sin", gmres_its=90)),
    "tet3_v22": ("tet", 3, dict(problem="sin", pre_smooth_its=2, post_smooth_its=2, gmres_its=120)),
    "tri32_c1": ("tri", 32, dict(problem="sin", gmres_its=400, full=False)),
    # the 3D benchmark mesh: about 40 minutes of reference CPU time
    "tet20_c2_summary": ("tet", 20, dict(problem="sin", pre_smooth_its=2, post_smooth_its=2, gmres_its=400,
                                         apply_reps=4, summary=True)),
}

FULL_KEYS_SKIP = ()
REDUCED_KEEP = ("apply_r", "smooth_x", "rhs", "RARvalues", "mg_e", "pc_x", "x_solution", "its",
                "res_hist", "l2err", "linferr", "ncolor", "nlevel", "nodes_per_level",
                "t_apply", "t_solve", "t_rar", "t_mesh_setup", "t_rhs", "t_precond", "threads")
HASHED = ("x_ref_in", "nbf", "alnmt", "glb_bcface_type", "fina", "cola", "whichc", "sfc")


def array_digest(a) -> str:
    a = np.ascontiguousarray(a)
    h = hashlib.sha256()
    h.update(str(a.dtype.str).encode())
    h.update(str(a.shape).encode())
    h.update(a.tobytes())
    return h.hexdigest()


VARPROP = {"varprop_tet3": ("tet3_v22", 21)}


def run_varprop_case(name: str) -> str:
    """Per-element kappa residual of the reference's z05 varprop module."""
    src, seed = VARPROP[name]
    out = os.path.join(HERE, name + ".npz")
    subprocess.run([sys.executable, "-m", "oracle.refrun.run_varprop", os.path.join(HERE, src + ".npz"), out,
                    str(seed)], cwd=REPO, check=True)
    return out


def run_case(name: str) -> str:
    """Run the reference on one case and store its golden file."""
    if name in VARPROP:
        return run_varprop_case(name)
    kind, n, opts = CASES[name]
    opts = dict(opts)
    full = opts.pop("full", True)
    summary = opts.pop("summary", False)
    g = dgmesh.unit_square_tri_mesh(n) if kind == "tri" else dgmesh.unit_cube_kuhn_mesh(n)
    m = dgmesh.ingest(g)
    order = dgsfc.hilbert_sfc_order(m.cg_coords)
    work = tempfile.mkdtemp(prefix="golden_")
    mp = os.path.join(work, "mesh.msh")
    dgmesh.write_gmsh22(mp, g)
    sp = os.path.join(work, "sfc.npy")
    np.save(sp, order)
    op = os.path.join(work, "opts.json")
    with open(op, "w") as fh:
        json.dump(opts, fh)
    raw = os.path.join(work, "out.npz")
    subprocess.run([sys.executable, "-m", "oracle.refrun.run_reference", mp, sp, raw, op],
                   cwd=REPO, check=True, stdout=subprocess.DEVNULL)
    if summary:
        return c2_summary(raw, name)
    d = dict(np.load(raw))
    meta = dict(kind=kind, n=n, seed=0, opts=opts, full=full)
    if full:
        keep = {k: v for k, v in d.items()}
    else:
        keep = {k: d[k] for k in REDUCED_KEEP if k in d}
        meta["digests"] = {k: array_digest(d[k]) for k in HASHED if k in d}
    keep["meta_json"] = np.asarray(json.dumps(meta))
    out = os.path.join(HERE, name + ".npz")
    np.savez_compressed(out, **keep)
    return out



def c2_summary(raw_npz: str, out_name: str = "tet20_c2_summary") -> str:
    """Compact record of the reference's full 3D benchmark solve (48,000 P3
    tets, 960,000 DOFs, V(2,2), GMRES(30), rtol 1e-10): every 97th entry of
    the solution and of the residual of the harness vectors, norms and the
    residual history.  raw_npz is the output of oracle/refrun/run_reference.py
    for that mesh (options pre_smooth_its = post_smooth_its = 2)."""
    d = dict(np.load(raw_npz))
    keep = {
        "x_sub": d["x_solution"][::97].copy(), "x_norm": np.linalg.norm(d["x_solution"]),
        "x_sum": d["x_solution"].sum(), "apply_r_sub": d["apply_r"][::97].copy(),
        "rar_sub": d["RARvalues"][::7].copy(), "its": d["its"], "res_hist": d["res_hist"],
        "l2err": d["l2err"], "linferr": d["linferr"], "t_apply": d["t_apply"], "t_solve": d["t_solve"],
        "t_rar": d["t_rar"], "t_precond": d["t_precond"], "threads": d["threads"],
        "rhs_norm": np.linalg.norm(d["rhs"]), "nodes_per_level": d["nodes_per_level"],
        "ncolor": d["ncolor"],
    }
    meta = dict(kind="tet", n=20, seed=0, opts=dict(pre_smooth_its=2, post_smooth_its=2, gmres_its=400),
                full=False, stride_x=97, stride_rar=7)
    keep["meta_json"] = np.asarray(json.dumps(meta))
    out = os.path.join(HERE, out_name + ".npz")
    np.savez_compressed(out, **keep)
    return out


if __name__ == "__main__":
    args = sys.argv[1:]
    if args[:1] == ["--c2-summary"]:
        # args[1]: output of oracle/refrun/run_reference.py for the 20^3 Kuhn mesh
        print("generated", c2_summary(args[1]))
    else:
        for nm in args or list(CASES) + list(VARPROP):
            print("generated", run_case(nm))
