"""Run the reference's own z06 diffusion path on CPU and dump its results.

Test infrastructure only: this script needs the reference checkout (it is
never run by the product, the GPU tests or the benchmark).  It executes the
unmodified reference modules (z02-implicit/z06-DGtoCG/*.py) with
stand-ins for the packages this image lacks (``shims/``), follows the call
order of the reference's driver (z02-implicit/z06-DGtoCG/main.py:52-206),
and saves every intermediate the parity tests pin to an ``.npz`` file.

Usage (one mesh per process -- the reference reads its mesh at import):

    python -m oracle.refrun.run_reference MESH.msh SFC.npy OUT.npz OPTIONS.json

OPTIONS keys: eta_e, pre_smooth_its, post_smooth_its, gmres_m, gmres_its,
rtol (tolerance relative to ||b||), problem ('sin' | 'sinh2d'), seed,
do_solve (bool), do_precond (bool), threads, ref_dir (the reference's
z02-implicit/z06-DGtoCG directory; default: $DG_REFERENCE_DIR/z02-implicit/z06-DGtoCG,
and the script refuses to run when neither is given).
"""
from __future__ import annotations

import json
import os
import shutil
import sys
import tempfile
import time

import numpy as np



def default_ref_dir() -> str:
    root = os.environ.get("DG_REFERENCE_DIR")
    if not root:
        raise SystemExit("set DG_REFERENCE_DIR to the reference checkout (or pass ref_dir in OPTIONS)")
    return os.path.join(root, "z02-implicit", "z06-DGtoCG")


def _setup_paths(mesh_path, ref_dir):
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(os.path.dirname(here))
    sys.path[:0] = [os.path.join(here, "shims"), ref_dir, repo]
    sys.argv = ["main.py", "-f", mesh_path]


def main(mesh_in, sfc_in, out_path, opts):
    ref_dir = opts.get("ref_dir") or default_ref_dir()
    work = tempfile.mkdtemp(prefix="dgref_")
    mesh_path = os.path.join(work, "mesh.msh")
    shutil.copy(mesh_in, mesh_path)
    # the reference's SFC cache seam (multigrid_linearelastic.py:221-223)
    shutil.copy(sfc_in, mesh_path[:-4] + "fluid_sfc.npy")
    _setup_paths(mesh_path, ref_dir)

    import scipy.sparse as _sp
    # numpy >= 2 no longer converts a (1, 1) np.matrix to a scalar on
    # assignment; sparsity.py:138-140 relies on that (it divides by
    # ``I_cf.sum(axis=1)[k]``).  Return a flat array for row sums so the
    # reference computes the same 1/#copies weights as under numpy 1.26.
    _orig_sum = _sp.csr_matrix.sum

    def _row_sum_flat(self, axis=None, dtype=None, out=None):
        res = _orig_sum(self, axis=axis, dtype=dtype, out=out)
        return np.asarray(res).ravel() if axis == 1 else res
    _sp.csr_matrix.sum = _row_sum_flat

    import torch
    torch.set_num_threads(int(opts.get("threads", os.cpu_count())))
    torch.set_grad_enabled(False)
    import io
    import contextlib
    quiet = io.StringIO()
    with contextlib.redirect_stdout(quiet):
        import config
    config.disabletqdm = True
    config.linear_solver = "gmres-mg"
    config.mg_opt_D = 2
    config.gmres_m = int(opts.get("gmres_m", 30))
    config.gmres_its = int(opts.get("gmres_its", 400))
    config.eta_e = float(opts.get("eta_e", 90.0))
    config.pre_smooth_its = int(opts.get("pre_smooth_its", 3))
    config.post_smooth_its = int(opts.get("post_smooth_its", 3))
    t_setup0 = time.perf_counter()
    with contextlib.redirect_stdout(quiet):
        import cmmn_data
        import function_space
        import mesh_init
        import sparsity
        import volume_mf_diff
        import multigrid_linearelastic as mg
        from function_space import FuncSpace, Element
        from config import sf_nd_nb
        from get_bdiag_diag import get_bdiag_diag

        dev = config.dev
        ndim = config.ndim
        nele = config.nele
        vel_ele = Element(ele_order=config.ele_p, gi_order=config.ele_p * 2, edim=ndim, dev=dev,
                          dtype=config.dtype)
        mesh_init.scale_mesh(mesh=config.mesh, origin=np.zeros(3), scale=np.asarray([1, 1, 1]))
        fs = FuncSpace(vel_ele, name="Velocity", mesh=config.mesh, dev=dev)
        fs_ts = function_space.create_funcspacets_from_funcspace(funcspace=fs)
        sf_nd_nb.set_data(vel_func_space=fs_ts, p1cg_nonods=fs_ts.cg_nonods)
        fluid_spar, solid_spar = sparsity.get_subdomain_sparsity(
            fs.cg_ndglno, config.nele_f, config.nele_s, fs.cg_nonods)
        sf_nd_nb.set_data(sparse_f=fluid_spar, sparse_s=solid_spar)
        sf_nd_nb.set_data(bdfscm=cmmn_data.BDFdata(order=config.time_order))
        t_mesh = time.perf_counter() - t_setup0
        t0 = time.perf_counter()
        get_bdiag_diag()
        t_bdiag = time.perf_counter() - t0
    out = {}
    el = vel_ele
    for k in ("n", "nlx", "weight", "sn", "snlx", "sweight", "gi_align"):
        out["el_" + k] = getattr(el, k).cpu().numpy()
    out["x_ref_in"] = fs.x_ref_in.cpu().numpy()
    out["nbf"] = fs.nbf.cpu().numpy()
    out["alnmt"] = fs.alnmt.cpu().numpy()
    out["glb_bcface_type"] = np.asarray(fs.glb_bcface_type.cpu().numpy())
    out["cg_ndglno"] = np.asarray(fs.cg_ndglno).reshape(nele, -1)
    out["bc_node_list"] = np.asarray(fs.bc_node_list)
    sp_ = fluid_spar
    out["fina"] = np.asarray(sp_.fina)
    out["cola"] = np.asarray(sp_.cola)
    out["whichc"] = np.asarray(sp_.whichc)
    out["ncolor"] = np.asarray(sp_.ncolor)
    out["I_cf_crow"] = sp_.I_cf.crow_indices().cpu().numpy()
    out["I_cf_col"] = sp_.I_cf.col_indices().cpu().numpy()
    out["I_cf_val"] = sp_.I_cf.values().cpu().numpy()
    out["bdiagK"] = sf_nd_nb.bdiagK.cpu().numpy()
    out["diagK"] = sf_nd_nb.diagK.cpu().numpy()

    nloc = el.nloc
    nonods = nele * nloc
    rng = np.random.default_rng(int(opts.get("seed", 1234)))
    xin = rng.standard_normal(nonods)
    bin_ = rng.standard_normal(nonods)
    out["apply_x"] = xin
    out["apply_b"] = bin_
    with contextlib.redirect_stdout(quiet):
        r0 = torch.zeros(nonods, dtype=torch.float64)
        r0, _ = volume_mf_diff.get_residual_or_smooth(
            r0, torch.tensor(xin), torch.tensor(bin_), do_smooth=False)
        out["apply_r"] = r0.numpy().copy()
        # timing of one apply (median of 5 after 2 warm-ups)
        ts = []
        for it in range(int(opts.get("apply_reps", 7))):
            rr = torch.zeros(nonods, dtype=torch.float64)
            t0 = time.perf_counter()
            volume_mf_diff.get_residual_or_smooth(rr, torch.tensor(xin), torch.tensor(bin_), do_smooth=False)
            ts.append(time.perf_counter() - t0)
        out["t_apply"] = np.asarray(np.median(ts[2:]) if len(ts) > 2 else np.median(ts))
        r0 = torch.zeros(nonods, dtype=torch.float64)
        xs = torch.tensor(xin)
        r0, xs = volume_mf_diff.get_residual_or_smooth(r0, xs, torch.tensor(bin_), do_smooth=True)
        out["smooth_r"] = r0.numpy().copy()
        out["smooth_x"] = xs.numpy().copy()

        # RAR (Galerkin P1CG operator by colouring probes) and the SFC levels
        t0 = time.perf_counter()
        rar = volume_mf_diff._calc_RAR_mf_color(
            sp_.I_fc, sp_.I_cf, sp_.whichc, sp_.ncolor, sp_.spIdx_for_color,
            sp_.colIdx_for_color, sp_.fina, sp_.cola, sp_.ncola)
        t_rar = time.perf_counter() - t0
        out["RARvalues"] = rar.numpy().copy()
        t0 = time.perf_counter()
        volume_mf_diff._get_RAR_and_sfc_data_Um()
        t_rar_sfc = time.perf_counter() - t0
    sd = sf_nd_nb.sfc_data_Um
    out["sfc"] = np.asarray(sd.space_filling_curve_numbering)
    out["nlevel"] = np.asarray(sd.nlevel)
    out["nodes_per_level"] = np.asarray(sd.nodes_per_level)
    for lev in range(sd.nlevel - 1):
        a, diag, nn = sd.variables_sfc[lev]
        out["lev%d_crow" % lev] = a.crow_indices().numpy()
        out["lev%d_col" % lev] = a.col_indices().numpy()
        out["lev%d_val" % lev] = a.values().numpy()
        out["lev%d_diag" % lev] = diag.numpy().ravel()
    a_last = sd.variables_sfc[sd.nlevel - 1][0]
    out["lev_last_dense"] = np.asarray(a_last.todense())

    cg_nonods = sp_.cg_nonods
    r_cg = rng.standard_normal(cg_nonods)
    out["mg_r"] = r_cg
    with contextlib.redirect_stdout(quiet):
        e = mg.mg_on_P1CG(torch.tensor(r_cg), sd.variables_sfc, sd.nlevel, sd.nodes_per_level, cg_nonods)
        out["mg_e"] = e.numpy().copy()
        if opts.get("do_precond", True):
            rp = rng.standard_normal(nonods)
            out["pc_r"] = rp
            t0 = time.perf_counter()
            xp = volume_mf_diff._um_left_precond(torch.zeros(nonods, dtype=torch.float64), torch.tensor(rp))
            out["t_precond"] = np.asarray(time.perf_counter() - t0)
            out["pc_x"] = xp.reshape(-1).numpy().copy()

    # right-hand side: manufactured problem
    x_ref_in = fs.x_ref_in.cpu().numpy()
    X = [x_ref_in[:, d, :] for d in range(ndim)]
    prob = opts.get("problem", "sin")
    if prob == "sin":
        f = (ndim * np.pi ** 2) * np.prod([np.sin(np.pi * x) for x in X], axis=0)
        g = np.zeros_like(f)
        uex = np.prod([np.sin(np.pi * x) for x in X], axis=0)
    elif prob == "sinh2d":
        f = np.zeros_like(X[0])
        uex = np.sin(np.pi * X[0]) * np.sinh(np.pi * X[1]) / np.sinh(np.pi)
        g = uex * np.asarray(fs.bc_node_list[0]).reshape(nele, nloc)
    else:
        raise ValueError(prob)
    out["f"] = f
    out["g"] = g
    out["u_exact"] = uex
    with contextlib.redirect_stdout(quiet):
        x_rhs = torch.zeros(nele, nloc, dtype=torch.float64)
        u_bc = [torch.tensor(g)]
        alpha = torch.zeros(nele, nloc, dtype=torch.float64)
        t0 = time.perf_counter()
        x_rhs = volume_mf_diff._get_rhs(x_rhs, torch.tensor(f.reshape(-1)), u_bc, alpha)
        t_rhs = time.perf_counter() - t0
    out["rhs"] = x_rhs.reshape(-1).numpy().copy()

    if opts.get("do_solve", True):
        bnorm = float(np.linalg.norm(out["rhs"]))
        tol = float(opts.get("rtol", 1e-10)) * bnorm
        hist = []
        import builtins
        real_print = builtins.print

        def capture(*a, **k):
            if a and a[0] == "its=":
                hist.append((int(a[1]), float(a[3])))
        builtins.print = capture
        try:
            x0 = torch.zeros(nele * nloc, dtype=torch.float64)
            t0 = time.perf_counter()
            xs, its = volume_mf_diff._gmres_mg_solver(x0, x_rhs.reshape(-1).clone(), tol)
            t_solve = time.perf_counter() - t0
        finally:
            builtins.print = real_print
        out["x_solution"] = xs.reshape(-1).numpy().copy()
        out["its"] = np.asarray(its)
        out["res_hist"] = np.asarray(hist)
        out["t_solve"] = np.asarray(t_solve)
        with contextlib.redirect_stdout(quiet):
            l2, linf = volume_mf_diff.get_l2_error(xs, torch.tensor(uex))
        out["l2err"] = np.asarray(l2)
        out["linferr"] = np.asarray(linf)
    out["t_mesh_setup"] = np.asarray(t_mesh)
    out["t_bdiag"] = np.asarray(t_bdiag)
    out["t_rar"] = np.asarray(t_rar)
    out["t_rar_sfc"] = np.asarray(t_rar_sfc)
    out["t_rhs"] = np.asarray(t_rhs)
    out["threads"] = np.asarray(torch.get_num_threads())
    np.savez(out_path, **out)
    shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2], sys.argv[3], json.loads(open(sys.argv[4]).read()))
