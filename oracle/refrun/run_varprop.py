"""Run the reference's variable-property diffusion residual and dump it.

Test infrastructure only (the product, the GPU tests and the benchmark never
run it).  The per-element diffusivity convention of this build follows
z05-ns/volume_mf_um_diff_varprop.py: kappa_e in the volume term
(:422-426), (kappa_e + kappa_nb) / 2 on all three interior-face terms
(:567) and kappa_e on boundary faces (:682).  That module is part of the
reference's FSI code and reads its inputs from the z05 ``config`` module; its
residual routine ``get_residual_or_smooth`` (:347-395) and the kernels it
calls (``_k_res_one_batch``, ``_s_res_one_batch``, ``_s_res_fi``,
``_s_res_fb``) are executed here unmodified, with

  * a stand-in ``config`` module that carries only the names those routines
    read (nele, ndim, dev, eta_e, no_batch, isoparametric, sf_nd_nb);
  * ``sf_nd_nb.disp_func_space`` built from a golden case of the z06
    harness, i.e. the reference's own element tables and mesh arrays
    (x_ref_in, nbf, alnmt, glb_bcface_type);
  * an empty ``multigrid_linearelastic`` module: the residual routine never
    calls it (the module-level import pulls in the Fortran SFC wrappers).

The field is the displacement-like vector field the module solves for,
(nele, nloc, ndim); its operator is the scalar SIP operator times the
identity in the components, so each component of the output is the scalar
residual with kappa = mesh_mu.

Usage:

    python -m oracle.refrun.run_varprop GOLDEN.npz OUT.npz [SEED]

The reference checkout is found through $DG_REFERENCE_DIR (the directory
holding z05-ns/); the script refuses to run without it.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np


def reference_dir() -> str:
    ref = os.environ.get("DG_REFERENCE_DIR")
    if not ref or not os.path.isdir(os.path.join(ref, "z05-ns")):
        raise SystemExit("set DG_REFERENCE_DIR to the reference checkout (the directory holding z05-ns/)")
    return ref


def run(golden_path: str, out_path: str, seed: int = 21, eta_e: float = 90.0, sigma: float = 1.0) -> None:
    import torch
    torch.set_grad_enabled(False)
    ref = reference_dir()
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path[:0] = [os.path.join(here, "shims"), os.path.join(ref, "z05-ns")]
    g = dict(np.load(golden_path))
    x_ref_in = g["x_ref_in"]
    nele, ndim, nloc = x_ref_in.shape
    if ndim != 3:
        raise SystemExit("the varprop harness is set up for 3D golden cases")
    el = types.SimpleNamespace(
        nloc=nloc, ngi=g["el_n"].shape[1], sngi=g["el_sn"].shape[2],
        n=torch.tensor(g["el_n"]), nlx=torch.tensor(g["el_nlx"]), weight=torch.tensor(g["el_weight"]),
        sn=torch.tensor(g["el_sn"]), snlx=torch.tensor(g["el_snlx"]), sweight=torch.tensor(g["el_sweight"]),
        gi_align=torch.tensor(g["el_gi_align"]))
    fs = types.SimpleNamespace(element=el, x_ref_in=torch.tensor(x_ref_in), nbf=torch.tensor(g["nbf"]),
                               alnmt=torch.tensor(g["alnmt"]), glb_bcface_type=torch.tensor(g["glb_bcface_type"]))
    rng = np.random.default_rng(seed)
    kappa = np.exp(sigma * rng.standard_normal(nele))
    x = rng.standard_normal((nele, nloc, ndim))
    b = rng.standard_normal((nele, nloc, ndim))
    sf_nd_nb = types.SimpleNamespace(disp_func_space=fs, pre_func_space=types.SimpleNamespace(element=el),
                                     mesh_mu=torch.tensor(kappa))
    cfg = types.ModuleType("config")
    cfg.__dict__.update(mesh=None, ndim=ndim, dev=torch.device("cpu"), nele=nele, nele_f=nele, nele_s=0,
                        no_batch=1, eta_e=eta_e, jac_wei=2.0 / 3.0, isoparametric=True, sf_nd_nb=sf_nd_nb)
    sys.modules["config"] = cfg
    sys.modules["multigrid_linearelastic"] = types.ModuleType("multigrid_linearelastic")
    import volume_mf_um_diff_varprop as vp
    r0 = torch.zeros(nele * nloc * ndim, dtype=torch.float64)
    r, _ = vp.get_residual_or_smooth(r0, torch.tensor(x).reshape(-1).clone(), torch.tensor(b).reshape(-1).clone(),
                                     do_smooth=False)
    np.savez_compressed(out_path, kappa=kappa, x=x, b=b, r=r.numpy().reshape(nele, nloc, ndim),
                        eta_e=eta_e, seed=seed, sigma=sigma, source=os.path.basename(golden_path))


if __name__ == "__main__":
    run(sys.argv[1], sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else 21)
