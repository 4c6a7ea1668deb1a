"""Reference-element tables for cubic (P3) Lagrange triangles and tetrahedra.

The tables have the shapes and node/quadrature orderings of the reference's
``SHATRInew`` (z02-implicit/z06-DGtoCG/shape_function.py:459-1317) and
``Element`` (z02-implicit/z06-DGtoCG/function_space.py:14-80):

=========  =======================  ==========================
name       3D (tet, P3)             2D (tri, P3)
=========  =======================  ==========================
n          (20, 24)                 (10, 12)
nlx        (3, 20, 24)              (2, 10, 12)
weight     (24,)  sum = 1/6         (12,)  sum = 1/2
sn         (4, 20, 12)              (3, 10, 4)
snlx       (4, 3, 20, 12)           (3, 2, 10, 4)
sweight    (12,)  sum = 1/2         (4,)   sum = 1
gi_align   (3, 12)                  (2, 4)
=========  =======================  ==========================

The basis functions are computed from the generic P3 Lagrange formula on
barycentric multi-indices instead of the reference's hand-expanded
polynomials; the node numbering (which multi-index sits at which local node)
and the quadrature point order are the ones the reference uses, because the
mesh arrays (``x_ref_in``, ``alnmt``) and the face-neighbour alignment
tables refer to them.  The quadrature constants are the published rules the
reference quotes, with the same number of digits (Keast rule 7 for the
tetrahedron, Strang-Fix rule 9 for triangles, 4-point Gauss-Legendre on
lines), so that face sizes ``h = sum(sdetwei)`` agree to the last bit of the
rule.  ``gi_align`` is derived here geometrically: row ``k`` maps a face
quadrature point of this side to the neighbour's point at the same physical
location when the neighbour face is related by alignment code ``k``
(z02-implicit/z06-DGtoCG/mesh_init.py:371-381).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# ---------------------------------------------------------------------------
# local node -> barycentric multi-index (entries sum to 3)
# tetrahedron: shape_function.py:509-531 (barycentric order l1, l2, l3, l4)
TET_P3_NODES = np.array([
    (3, 0, 0, 0), (0, 3, 0, 0), (0, 0, 3, 0), (0, 0, 0, 3),
    (2, 0, 1, 0), (1, 0, 2, 0),      # edge 0-2
    (2, 1, 0, 0), (1, 2, 0, 0),      # edge 0-1
    (0, 2, 1, 0), (0, 1, 2, 0),      # edge 1-2
    (2, 0, 0, 1), (1, 0, 0, 2),      # edge 0-3
    (0, 2, 0, 1), (0, 1, 0, 2),      # edge 1-3
    (0, 0, 2, 1), (0, 0, 1, 2),      # edge 2-3
    (0, 1, 1, 1), (1, 1, 1, 0),      # faces 1-2-3, 0-1-2
    (1, 0, 1, 1), (1, 1, 0, 1),      # faces 0-2-3, 0-1-3
], dtype=np.int64)
# triangle: shape_function.py:1124-1140 (gmsh triangle10 order)
TRI_P3_NODES = np.array([
    (3, 0, 0), (0, 3, 0), (0, 0, 3),
    (2, 1, 0), (1, 2, 0),            # edge 0-1
    (0, 2, 1), (0, 1, 2),            # edge 1-2
    (1, 0, 2), (2, 0, 1),            # edge 2-0
    (1, 1, 1),
], dtype=np.int64)

# Corner nodes of each local face, in the order that defines the face's own
# barycentric coordinates (mesh_init.py:298-320 for tets; :40-44 for tris).
TET_FACE_CORNERS = ((2, 1, 3), (0, 2, 3), (1, 0, 3), (0, 1, 2))
TRI_FACE_CORNERS = ((0, 1), (1, 2), (2, 0))

# Local nodes lying on each face (mesh_init.py:840-889, face_iloc_array).
TET_FACE_NODES = np.array([
    [1, 2, 3, 8, 9, 14, 15, 12, 13, 16],
    [0, 2, 3, 4, 5, 10, 11, 14, 15, 18],
    [0, 1, 3, 6, 7, 10, 11, 12, 13, 19],
    [0, 1, 2, 4, 5, 6, 7, 8, 9, 17],
], dtype=np.int64)
TRI_FACE_NODES = np.array([[0, 3, 4, 1], [1, 5, 6, 2], [2, 7, 8, 0]], dtype=np.int64)

# P1DG -> P3DG element prolongator (mesh_init.py:586-607 tet, :224-235 tri):
# row n holds the barycentric weights of local node n on the element corners.
TET_P1_TO_P3 = TET_P3_NODES / 3.0
TRI_P1_TO_P3 = TRI_P3_NODES / 3.0


# ---------------------------------------------------------------------------
# quadrature rules (published constants, same digits as the reference)

def _tet_keast7():
    """Keast rule 7: 24 points, degree 6 (shape_function.py:25-64).

    Returns (points (24, 3) in (l1, l2, l3), weights summing to 1/6).
    The points come in four orbits listed in the reference's order.
    """
    pts, wts = [], []
    # three 4-point orbits (a, a, a, b): position of b in l1, l4, l3, l2 order
    for a, b, w in ((0.2146028712591517, 0.3561913862225449, 0.0399227502581679),
                    (0.0406739585346113, 0.8779781243961660, 0.0100772110553207),
                    (0.3223378901422757, 0.0329863295731731, 0.0553571815436544)):
        for lam in ((b, a, a), (a, a, a), (a, a, b), (a, b, a)):
            pts.append(lam)
            wts.append(w)
    # one 12-point orbit (a, a, b, c)
    a, b, c = 0.0636610018750175, 0.2696723314583159, 0.6030056647916491
    for lam in ((b, a, a), (a, b, a), (a, a, b), (c, a, a), (a, c, a), (a, a, c),
                (a, b, c), (b, c, a), (c, a, b), (a, c, b), (b, a, c), (c, b, a)):
        pts.append(lam)
        wts.append(0.0482142857142857)
    return np.asarray(pts, dtype=np.float64), np.asarray(wts, dtype=np.float64) * (1.0 / 6.0)


def _tri_strang9():
    """Strang-Fix rule 9: 12 points, degree 6 (shape_function.py:271-308).

    Returns (points (12, 3) barycentric, weights summing to 1/2).  The third
    coordinate is formed as ``1 - p0 - p1`` like the reference does.
    """
    a, b = 0.873821971016996, 0.063089014491502
    c, d = 0.501426509658179, 0.249286745170910
    e, f, g = 0.636502499121399, 0.310352451033785, 0.053145049844816
    two = [(a, b), (b, a), (b, b), (c, d), (d, c), (d, d),
           (e, f), (e, g), (f, e), (f, g), (g, e), (g, f)]
    w = [0.050844906370207] * 3 + [0.116786275726379] * 3 + [0.082851075618374] * 6
    p = np.asarray(two, dtype=np.float64)
    p3 = 1 - np.sum(p, axis=1)
    return np.concatenate([p, p3[:, None]], axis=1), np.asarray(w, dtype=np.float64) * 0.5


def _line_gauss4():
    """4-point Gauss-Legendre on [0, 1] (shape_function.py:392-420).

    Returns (points (4, 2) as (p, 1-p), weights summing to 1).
    """
    a, b = 0.339981043584856, 0.861136311594053
    w1, w2 = 0.652145154862546, 0.347854845137454
    xs = [0.5 - 0.5 * b, 0.5 - 0.5 * a, 0.5 + 0.5 * a, 0.5 + 0.5 * b]
    pts = np.asarray([[x, 1 - x] for x in xs], dtype=np.float64)
    sw = np.zeros(4, dtype=np.float64)
    sw[0], sw[1], sw[2], sw[3] = w2, w1, w1, w2
    sw /= 2.0
    return pts, sw


# ---------------------------------------------------------------------------
# generic P3 Lagrange basis on barycentric coordinates

def _lagrange_factor(lam, k):
    """prod_{j<k} (3 lam - j) / (j + 1) and its derivative in lam."""
    val = np.ones_like(lam)
    der = np.zeros_like(lam)
    for j in range(k):
        f = (3.0 * lam - j) / (j + 1)
        df = 3.0 / (j + 1)
        der = der * f + val * df
        val = val * f
    return val, der


def _p3_basis(nodes, lam):
    """Values and barycentric derivatives of the P3 basis.

    nodes: (nloc, nbary) multi-indices; lam: (npts, nbary) barycentric points.
    Returns phi (nloc, npts) and dphi (nbary, nloc, npts) = d phi / d lam_k.
    """
    nloc, nb = nodes.shape
    npts = lam.shape[0]
    phi = np.ones((nloc, npts))
    fac = np.empty((nloc, nb, npts))
    dfac = np.empty((nloc, nb, npts))
    for i in range(nloc):
        for k in range(nb):
            fac[i, k], dfac[i, k] = _lagrange_factor(lam[:, k], int(nodes[i, k]))
        phi[i] = np.prod(fac[i], axis=0)
    dphi = np.empty((nb, nloc, npts))
    for k in range(nb):
        others = [kk for kk in range(nb) if kk != k]
        dphi[k] = dfac[:, k] * np.prod(fac[:, others], axis=1)
    return phi, dphi


def _local_derivatives(dphi):
    """d/d l_i with the last barycentric coordinate eliminated (l_last = 1 - sum)."""
    nb = dphi.shape[0]
    return np.stack([dphi[i] - dphi[nb - 1] for i in range(nb - 1)], axis=0)


def _face_points(face_corners, pface, nbary):
    """Barycentric coordinates (in the element) of face quadrature points."""
    nface = len(face_corners)
    out = np.zeros((nface, pface.shape[0], nbary))
    for f, corners in enumerate(face_corners):
        for k, c in enumerate(corners):
            out[f, :, c] = pface[:, k]
    return out


def _alignment_table(pface, ndim):
    """Derive gi_align: row k maps this side's face point g to the neighbour's.

    A neighbour face related by code k lists the shared corners as
    3D: k=0 (A,C,B), k=1 (B,A,C), k=2 (C,B,A) relative to this side's
    (A,B,C); 2D: k=0 (A,B) (never occurs on consistently oriented meshes),
    k=1 (B,A).  The neighbour point at the same location therefore has its
    face barycentric coordinates permuted accordingly.
    """
    if ndim == 3:
        perms = ((0, 2, 1), (1, 0, 2), (2, 1, 0))
    else:
        perms = ((0, 1), (1, 0))
    sngi = pface.shape[0]
    table = np.empty((len(perms), sngi), dtype=np.int64)
    for k, perm in enumerate(perms):
        target = pface[:, perm]
        for g in range(sngi):
            dist = np.abs(pface - target[g]).sum(axis=1)
            j = int(np.argmin(dist))
            if dist[j] > 1e-12:
                raise RuntimeError("face quadrature rule is not symmetric under alignment %d" % k)
            table[k, g] = j
    return table


@dataclass
class ElementTables:
    ndim: int
    nloc: int
    ngi: int
    sngi: int
    nface: int
    snloc: int
    n: np.ndarray
    nlx: np.ndarray
    weight: np.ndarray
    sn: np.ndarray
    snlx: np.ndarray
    sweight: np.ndarray
    gi_align: np.ndarray
    face_nodes: np.ndarray
    p1_to_p3: np.ndarray

    @property
    def ncorner(self) -> int:
        return self.ndim + 1


def p3_element(ndim: int) -> ElementTables:
    """Tables for the cubic element with quadrature degree 6 (Element(3, 6, ndim))."""
    if ndim == 3:
        nodes = TET_P3_NODES
        vpts3, weight = _tet_keast7()
        lam = np.concatenate([vpts3, (1.0 - vpts3[:, 0] - vpts3[:, 1] - vpts3[:, 2])[:, None]], axis=1)
        pface, sweight = _tri_strang9()
        corners = TET_FACE_CORNERS
        face_nodes = TET_FACE_NODES
        p1_to_p3 = TET_P1_TO_P3
    elif ndim == 2:
        nodes = TRI_P3_NODES
        lam, weight = _tri_strang9()
        pface, sweight = _line_gauss4()
        corners = TRI_FACE_CORNERS
        face_nodes = TRI_FACE_NODES
        p1_to_p3 = TRI_P1_TO_P3
    else:
        raise ValueError("only 2D triangles and 3D tetrahedra are supported")
    nbary = ndim + 1
    phi, dphi = _p3_basis(nodes, lam)
    nlx = _local_derivatives(dphi)
    spts = _face_points(corners, pface, nbary)
    nface = len(corners)
    sngi = pface.shape[0]
    nloc = nodes.shape[0]
    sn = np.empty((nface, nloc, sngi))
    snlx = np.empty((nface, ndim, nloc, sngi))
    for f in range(nface):
        sphi, sdphi = _p3_basis(nodes, spts[f])
        sn[f] = sphi
        snlx[f] = _local_derivatives(sdphi)
    return ElementTables(
        ndim=ndim, nloc=nloc, ngi=lam.shape[0], sngi=sngi, nface=nface,
        snloc=face_nodes.shape[1], n=phi, nlx=nlx, weight=weight, sn=sn,
        snlx=snlx, sweight=sweight, gi_align=_alignment_table(pface, ndim),
        face_nodes=face_nodes, p1_to_p3=np.asarray(p1_to_p3, dtype=np.float64))


# Face tangent directions d(l1..lD)/d(u, v) per local face, used for the
# face Jacobian, area element and outward normal
# (function_space.py:200-213 for tets; :214-219 for tris).
TET_DRST_DUV = np.array([
    [[0, 0], [0, 1], [1, 0]],
    [[1, 0], [0, 0], [0, 1]],
    [[0, 1], [1, 0], [0, 0]],
    [[-1, -1], [1, 0], [0, 1]],
], dtype=np.float64)
TRI_DRST_DUV = np.array([[-1.0, 1.0], [0.0, -1.0], [1.0, 0.0]], dtype=np.float64)


def drst_duv(ndim: int) -> np.ndarray:
    return TET_DRST_DUV if ndim == 3 else TRI_DRST_DUV


__all__ = ["ElementTables", "p3_element", "drst_duv"]
