"""f2py module ``get_nb`` for the oracle run of the reference, backed by the
numpy restatement of z00-fortran-src/get_neighbouring.f90."""
from oracle.fortran_restated import getfinele, getfin_p1cg  # noqa: F401
