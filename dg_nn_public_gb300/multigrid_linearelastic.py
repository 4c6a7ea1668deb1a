"""Drop-in for the reference's SFC multigrid module
(z02-implicit/z06-DGtoCG/multigrid_linearelastic.py).

The level hierarchy lives on the device inside the bound libdgsip context.
``mg_on_P1CG_prep`` also returns it in the reference's format (per level a
torch CSR matrix, its diagonal and size; the coarsest level as scipy CSR),
and ``mg_on_P1CG`` refuses level data other than the bound operator's.
"""
from __future__ import annotations

from .state import ensure_operator, sf_nd_nb
from . import volume_mf_diff as _vmd


def _check_levels(s, variables_sfc, nlevel, nodes_per_level, cg_nonods):
    import numpy as np
    _vmd._get_RAR_and_sfc_data_Um()
    sd = sf_nd_nb.sfc_data_Um
    if cg_nonods is not None and int(cg_nonods) != s.mesh.cg_nonods:
        raise ValueError("cg_nonods %d differs from the bound mesh's %d" % (int(cg_nonods), s.mesh.cg_nonods))
    if nlevel is not None and int(nlevel) != sd.nlevel:
        raise ValueError("nlevel %d differs from the bound operator's %d" % (int(nlevel), sd.nlevel))
    if nodes_per_level is not None and [int(v) for v in nodes_per_level] != list(sd.nodes_per_level):
        raise ValueError("nodes_per_level differs from the bound operator's")
    if variables_sfc is None or variables_sfc is sd.variables_sfc:
        return
    if len(variables_sfc) != len(sd.variables_sfc):
        raise ValueError("variables_sfc has %d levels, the bound operator %d" % (len(variables_sfc),
                                                                               len(sd.variables_sfc)))
    for lev, (given, bound) in enumerate(zip(variables_sfc, sd.variables_sfc)):
        a, b = given[0], bound[0]
        va = a.values().cpu().numpy() if hasattr(a, "values") and callable(a.values) else np.asarray(a.data)
        vb = b.values().cpu().numpy() if hasattr(b, "values") and callable(b.values) else np.asarray(b.data)
        if va.shape != vb.shape or not np.array_equal(va, vb):
            raise ValueError("variables_sfc level %d differs from the bound operator's SFC levels: the V-cycle "
                             "runs on the device levels of the bound operator" % lev)


def mg_on_P1CG(r0, variables_sfc=None, nlevel=None, nodes_per_level=None, cg_nonods=None):
    """One SFC V-cycle on the P1CG residual r0 given in curve order (:112-172).
    Level data passed in must be the bound operator's (ValueError otherwise)."""
    s = ensure_operator()
    _check_levels(s, variables_sfc, nlevel, nodes_per_level, cg_nonods)
    return s.mg_vcycle(r0.reshape(-1).contiguous())


def mg_on_P1CG_prep(fina=None, cola=None, RARvalues=None, sparse_in=None):
    """SFC ordering, coarse levels and their operators (:175-283).
    Returns (sfc, variables_sfc, nlevel, nodes_per_level)."""
    _vmd._get_RAR_and_sfc_data_Um()
    sd = sf_nd_nb.sfc_data_Um
    return sd.space_filling_curve_numbering, sd.variables_sfc, sd.nlevel, sd.nodes_per_level


def vel_pndg_to_p1dg_restrictor(x):
    """P3DG -> P1DG element restriction (:286-290)."""
    import torch
    s = ensure_operator()
    P = torch.as_tensor(s.el.p1_to_p3, device=x.device)
    return torch.einsum("ij,kj->ki", P.T, x.reshape(-1, s.mesh.nloc)).contiguous().view(-1)


def vel_p1dg_to_pndg_prolongator(x):
    """P1DG -> P3DG element prolongation (:293-297)."""
    import torch
    s = ensure_operator()
    P = torch.as_tensor(s.el.p1_to_p3, device=x.device)
    return torch.einsum("ij,kj->ki", P, x.reshape(-1, s.mesh.ndim + 1)).contiguous().view(-1)
