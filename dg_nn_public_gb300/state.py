"""Module state behind the reference-compatible call surface.

The reference keeps its solver state in module globals: the ``config``
module (z02-implicit/z06-DGtoCG/config.py) and the ``sf_nd_nb`` singleton
(z02-implicit/z06-DGtoCG/cmmn_data.py:8-138).  This module holds the
equivalent for the GPU solver: a ``config`` namespace with the same knob
names and an ``sf_nd_nb`` object whose fields the drop-in functions read and
write (``diagK``, ``bdiagK``, ``sfc_data_Um``, ``its``), plus the bound
``DGSolver``.  ``bind()`` attaches a mesh; ``bind_reference_funcspace()``
builds one from the reference's own FuncSpace objects.
"""
from __future__ import annotations

import types
from typing import Optional

import numpy as np

from .element import ElementTables, drst_duv
from .mesh import DGMesh
from .solver import DGSolver, SolverConfig

# knob names and defaults of z06/config.py:103-149, 207, 245 -- with the
# benchmark solver selection (GMRES + SFC multigrid, eta = 10 p^2)
config = types.SimpleNamespace(
    linear_solver="gmres-mg", tol=1.0e-9, jac_its=500, jac_wei=2.0 / 3.0,
    pre_smooth_its=3, post_smooth_its=3, mg_opt_D=2, gmres_m=30, gmres_its=400,
    mu_f=1.0, eta_e=90.0, no_batch=1, blk_solver="jacobian", is_pmg=False,
    dtype="float64", device=0,
)


class SFCdata:
    """z06/cmmn_data.py:141-187."""

    def __init__(self):
        self.space_filling_curve_numbering = None
        self.variables_sfc = None
        self.nlevel = None
        self.nodes_per_level = None

    def set_data(self, space_filling_curve_numbering=None, variables_sfc=None, nlevel=None,
                 nodes_per_level=None):
        if space_filling_curve_numbering is not None:
            self.space_filling_curve_numbering = space_filling_curve_numbering
        if variables_sfc is not None:
            self.variables_sfc = variables_sfc
        if nlevel is not None:
            self.nlevel = nlevel
        if nodes_per_level is not None:
            self.nodes_per_level = nodes_per_level


class SfNdNb:
    """The fields of z06/cmmn_data.py:8-138 that the diffusion path uses."""

    def __init__(self):
        self.solver: Optional[DGSolver] = None
        self.mesh: Optional[DGMesh] = None
        self.diagK = None
        self.bdiagK = None
        self.sfc_data_Um = SFCdata()
        self.its = 0
        self.nits = 0
        self.isTransient = False
        self.dt = None
        self.mesh_mu = None       # per-element diffusivity (z05 convention)
        self.operator_version = -1

    def set_data(self, diagK=None, bdiagK=None, mesh_mu=None, **_):
        if diagK is not None:
            self.diagK = diagK
        if bdiagK is not None:
            self.bdiagK = bdiagK
        if mesh_mu is not None:
            self.mesh_mu = mesh_mu


sf_nd_nb = SfNdNb()


def _cfg() -> SolverConfig:
    return SolverConfig(eta_e=config.eta_e, mu_f=config.mu_f, jac_wei=config.jac_wei,
                        pre_smooth_its=config.pre_smooth_its, post_smooth_its=config.post_smooth_its,
                        gmres_m=config.gmres_m, gmres_its=config.gmres_its, device=config.device)


def bind(mesh: DGMesh, sfc_order: np.ndarray, el: Optional[ElementTables] = None,
         kappa: Optional[np.ndarray] = None) -> DGSolver:
    """Create the GPU solver for a mesh and make it the module's current one."""
    if sf_nd_nb.solver is not None:
        sf_nd_nb.solver.close()
    s = DGSolver(mesh, sfc_order, _cfg(), el)
    if kappa is not None:
        s.set_kappa(kappa)
    sf_nd_nb.solver = s
    sf_nd_nb.mesh = mesh
    sf_nd_nb.mesh_mu = kappa
    sf_nd_nb.sfc_data_Um = SFCdata()
    sf_nd_nb.sfc_data_Um.space_filling_curve_numbering = np.asarray(sfc_order).reshape(-1, 1)
    sf_nd_nb.diagK = sf_nd_nb.bdiagK = None
    return s


def bind_reference_funcspace(func_space, sfc_numbering, cg_ndglno=None) -> DGSolver:
    """Bind from the reference's objects: a FuncSpace / FuncSpaceTS
    (z06/function_space.py:83-404) and its SFC numbering ((n, 1), 1-based,
    the content of ``<mesh>fluid_sfc.npy``)."""
    def host(a):
        return a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
    el_ref = func_space.element
    D = int(el_ref.ndim)
    x = host(func_space.x_ref_in)
    nele, _, nloc = x.shape
    cg = host(cg_ndglno if cg_ndglno is not None else func_space.cg_ndglno).reshape(nele, nloc)
    uniq, inv = np.unique(cg[:, :D + 1].ravel(), return_inverse=True)
    from .element import p3_element
    el = p3_element(D)
    el.n, el.nlx, el.weight = host(el_ref.n), host(el_ref.nlx), host(el_ref.weight)
    el.sn, el.snlx, el.sweight = host(el_ref.sn), host(el_ref.snlx), host(el_ref.sweight)
    el.gi_align = host(el_ref.gi_align).astype(np.int64)
    m = DGMesh(ndim=D, nloc=nloc, nele=nele, x_ref_in=x, nbf=host(func_space.nbf).astype(np.int64),
               alnmt=host(func_space.alnmt).astype(np.int64),
               glb_bcface_type=host(func_space.glb_bcface_type).astype(np.int64), cg_ndglno=cg,
               p1cg=inv.reshape(nele, D + 1).astype(np.int64), cg_nonods=int(uniq.size),
               cg_coords=np.zeros((uniq.size, D)), bc_node_list=[])
    return bind(m, sfc_numbering, el)


def solver() -> DGSolver:
    if sf_nd_nb.solver is None:
        raise RuntimeError("no mesh bound: call dg_nn_public_gb300.state.bind(...) first")
    return sf_nd_nb.solver


def ensure_operator() -> DGSolver:
    s = solver()
    if not s.built:
        s.build_operator()
    return s


__all__ = ["config", "sf_nd_nb", "bind", "bind_reference_funcspace", "solver", "ensure_operator",
           "drst_duv"]
