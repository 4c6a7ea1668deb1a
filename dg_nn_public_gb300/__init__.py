"""GB300-native SIP-DG diffusion solve (cubic triangles / tetrahedra).

The compute runs in libdgsip (hand-written sm_103a CUDA behind a C ABI,
include/dgsip.h); Python provides mesh generation/ingest, the reference
element tables, and the reference-compatible call surface
(volume_mf_diff, multigrid_linearelastic, get_bdiag_diag, solvers).
"""
__all__ = ["element", "mesh", "sfc", "solver", "state", "volume_mf_diff",
           "multigrid_linearelastic", "get_bdiag_diag", "solvers"]
