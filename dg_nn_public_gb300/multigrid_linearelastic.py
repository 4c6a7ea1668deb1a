"""Drop-in for the reference's SFC multigrid module
(z02-implicit/z06-DGtoCG/multigrid_linearelastic.py).

The level hierarchy lives on the device inside the bound libdgsip context;
``variables_sfc`` is kept as a list of (None, None, nodes) placeholders so
that callers that pass it back in keep working.
"""
from __future__ import annotations

from .state import ensure_operator, sf_nd_nb
from . import volume_mf_diff as _vmd


def mg_on_P1CG(r0, variables_sfc=None, nlevel=None, nodes_per_level=None, cg_nonods=None):
    """One SFC V-cycle on the P1CG residual r0 given in curve order (:112-172)."""
    s = ensure_operator()
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
