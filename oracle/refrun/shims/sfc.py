"""f2py module ``sfc`` for the oracle run of the reference.

Only ``calculate_nlevel_sfc`` is restated.  The space-filling-curve ordering
itself always reaches the reference through its own ``<mesh>fluid_sfc.npy``
cache (z02-implicit/z06-DGtoCG/multigrid_linearelastic.py:221-229), which
the harness writes before the run, so the Fortran generator is never called.
"""
from oracle.fortran_restated import calculate_nlevel_sfc  # noqa: F401


def ncurve_python_subdomain_space_filling_curve(*args, **kwargs):
    raise RuntimeError("the SFC ordering must be supplied through the .npy cache")
