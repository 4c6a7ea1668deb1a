"""Space-filling-curve ordering of the P1CG vertices.

The reference numbers the P1CG graph with a Fortran recursive-bisection
curve generator (z00-fortran-src/combined_fortran_source.f90:10575-10875 and
its RECBIS call tree) and caches the result as ``<mesh>fluid_sfc.npy``
(z02-implicit/z06-DGtoCG/multigrid_linearelastic.py:221-229).  That
generator cannot be built here (no Fortran compiler), so this module
provides a geometric space-filling curve instead: vertices are sorted by the
index of their quantised coordinates along a Hilbert curve (Skilling,
"Programming the Hilbert curve", AIP Conf. Proc. 707, 2004).  The output has
the reference's format: an (n, 1) int64 array whose entry i is the 1-based
position of vertex i along the curve, so it can be written to the
reference's cache file and both sides see the same ordering.
"""
from __future__ import annotations

import numpy as np


def _hilbert_index(q: np.ndarray, bits: int) -> np.ndarray:
    """Hilbert index of integer coordinates q (npts, ndim) in [0, 2^bits)."""
    x = q.astype(np.int64).copy()
    ndim = x.shape[1]
    m = 1 << (bits - 1)
    # inverse undo excess work (Skilling's AxestoTranspose)
    qq = m
    while qq > 1:
        p = qq - 1
        for i in range(ndim):
            hit = (x[:, i] & qq) != 0
            # invert low bits of x[0] where set
            x[hit, 0] ^= p
            # exchange low bits of x[i] and x[0] where not set
            nh = ~hit
            t = (x[nh, 0] ^ x[nh, i]) & p
            x[nh, 0] ^= t
            x[nh, i] ^= t
        qq >>= 1
    # Gray encode
    for i in range(1, ndim):
        x[:, i] ^= x[:, i - 1]
    t = np.zeros(x.shape[0], dtype=np.int64)
    qq = m
    while qq > 1:
        hit = (x[:, ndim - 1] & qq) != 0
        t[hit] ^= qq - 1
        qq >>= 1
    for i in range(ndim):
        x[:, i] ^= t
    # interleave the transposed bits into one index (most significant first)
    h = np.zeros(x.shape[0], dtype=np.int64)
    for b in range(bits - 1, -1, -1):
        for i in range(ndim):
            h = (h << 1) | ((x[:, i] >> b) & 1)
    return h


def hilbert_sfc_order(coords: np.ndarray, bits: int = 0) -> np.ndarray:
    """1-based curve position of each point, shape (n, 1), ties by index,
    computed by the library's host C++ (dg_sfc_order)."""
    from . import _capi
    return _capi.sfc_order(np.asarray(coords, dtype=np.float64), bits=bits)


def hilbert_sfc_order_numpy(coords: np.ndarray, bits: int = 0) -> np.ndarray:
    """The same numbering in numpy (cross-check of dg_sfc_order)."""
    coords = np.asarray(coords, dtype=np.float64)
    n, ndim = coords.shape
    if bits <= 0:
        bits = 20 if ndim == 2 else 16
    lo = coords.min(axis=0)
    span = np.maximum(coords.max(axis=0) - lo, 1e-300)
    scale = float((1 << bits) - 1)
    q = np.floor((coords - lo) / span.max() * scale).astype(np.int64)
    q = np.clip(q, 0, (1 << bits) - 1)
    h = _hilbert_index(q, bits)
    order = np.lexsort((np.arange(n), h))         # curve position -> vertex
    pos = np.empty(n, dtype=np.int64)
    pos[order] = np.arange(1, n + 1)
    return pos.reshape(n, 1)
