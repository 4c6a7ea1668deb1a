"""f2py module ``map_to_sfc_matrix`` for the oracle run of the reference,
backed by the numpy restatement of z00-fortran-src/compact_fcode.f90."""
from oracle.fortran_restated import best_sfc_mapping_to_sfc_matrix_unstructured, calculate_nlevel_sfc  # noqa: F401
