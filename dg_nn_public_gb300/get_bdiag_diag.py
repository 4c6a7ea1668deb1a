"""Drop-in for z02-implicit/z06-DGtoCG/get_bdiag_diag.py: the element block
diagonal of the operator, copied out of the stored element blocks."""
from __future__ import annotations

from .state import ensure_operator, sf_nd_nb


def get_bdiag_diag():
    """Set sf_nd_nb.bdiagK (nele, nloc, nloc) and sf_nd_nb.diagK (nele, nloc) (:30-62)."""
    K, d = ensure_operator().bdiag()
    sf_nd_nb.set_data(diagK=d, bdiagK=K)
