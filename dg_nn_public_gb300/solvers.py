"""Names of the reference's solver module (z02-implicit/z06-DGtoCG/solvers.py:162-280)
mapped onto the diffusion solvers; that module's own imports do not resolve
in the reference (solvers.py:13-16), the diffusion GMRES lives in
volume_mf_diff._gmres_mg_solver."""
from .volume_mf_diff import _cg_mg_solver as cg_mg_solver  # noqa: F401
from .volume_mf_diff import _gmres_mg_solver as gmres_mg_solver  # noqa: F401
from .volume_mf_diff import _mg_solver as mg_solver  # noqa: F401
