"""Solution output: VTU (VTK XML unstructured grid, Lagrange cells) and
``.pt`` files.

Counterpart of the reference's ``File`` writer (z02-implicit/z06-DGtoCG/
output.py:16-186) and of its ``torch.save`` of the solution (main.py:216):
an ASCII VTU with one VTK_LAGRANGE_TETRAHEDRON (71) or VTK_LAGRANGE_TRIANGLE
(69) cell per element over the element's own (discontinuous) nodes, and
point data per DG node.

VTK orders the nodes of an order-3 Lagrange simplex as: vertices; the two
points of each edge from its first to its second vertex, edges (0,1),
(1,2), (2,0) and, for tetrahedra, (0,3), (1,3), (2,3); then one point per
face, faces (0,1,3), (1,2,3), (0,2,3), (0,1,2); then the triangle's centre
point.  ``vtk_node_order`` derives the permutation from the element's
barycentric node table, with VTK's vertices taken as the element's corners
[2, 3, 0, 1] (tet) / [1, 2, 0] (triangle), which is the reference's choice
(mesh_init.py:155, 406-411), so files from either code read the same.
"""
from __future__ import annotations

from typing import Dict

import numpy as np

from .element import TET_P3_NODES, TRI_P3_NODES

VTK_LAGRANGE_TRIANGLE = 69
VTK_LAGRANGE_TETRAHEDRON = 71
_VTK_VERTEX_TO_CORNER = {3: (2, 3, 0, 1), 2: (1, 2, 0)}
_VTK_EDGES = {3: ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)), 2: ((0, 1), (1, 2), (2, 0))}
_VTK_FACES = {3: ((0, 1, 3), (1, 2, 3), (0, 2, 3), (0, 1, 2)), 2: ((0, 1, 2),)}


def vtk_node_order(ndim: int) -> np.ndarray:
    """perm[k] = local node of the element at VTK point k (P3)."""
    nodes = TET_P3_NODES if ndim == 3 else TRI_P3_NODES
    corner = _VTK_VERTEX_TO_CORNER[ndim]
    lookup = {tuple(int(v) for v in mu): i for i, mu in enumerate(nodes)}

    def node(weights):
        mu = [0] * (ndim + 1)
        for vtk_vertex, w in weights:
            mu[corner[vtk_vertex]] += w
        return lookup[tuple(mu)]

    perm = [node([(v, 3)]) for v in range(ndim + 1)]
    for a, b in _VTK_EDGES[ndim]:
        perm += [node([(a, 2), (b, 1)]), node([(a, 1), (b, 2)])]
    for f in _VTK_FACES[ndim]:
        perm.append(node([(v, 1) for v in f]))
    assert sorted(perm) == list(range(len(nodes)))
    return np.asarray(perm, dtype=np.int64)


def write_vtu(path: str, x_ref_in: np.ndarray, point_data: Dict[str, np.ndarray]) -> str:
    """Write an ASCII VTU: ``x_ref_in`` (nele, ndim, nloc) node coordinates,
    ``point_data`` name -> (nele * nloc,) scalars or (nele * nloc, ndim)
    vectors in the element-major DG numbering."""
    x = np.asarray(x_ref_in, dtype=np.float64)
    nele, ndim, nloc = x.shape
    nonods = nele * nloc
    pts = x.transpose(0, 2, 1).reshape(nonods, ndim)
    if ndim == 2:
        pts = np.concatenate([pts, np.zeros((nonods, 1))], axis=1)
    perm = vtk_node_order(ndim)
    conn = np.arange(nonods, dtype=np.int64).reshape(nele, nloc)[:, perm]
    cell = VTK_LAGRANGE_TETRAHEDRON if ndim == 3 else VTK_LAGRANGE_TRIANGLE
    with open(path, "w") as f:
        f.write('<?xml version="1.0" ?>\n')
        f.write('<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian" header_type="UInt32">\n')
        f.write("<UnstructuredGrid>\n")
        f.write('<Piece NumberOfPoints="%d" NumberOfCells="%d">\n' % (nonods, nele))
        f.write('<Points>\n<DataArray type="Float64" NumberOfComponents="3" format="ascii">\n')
        np.savetxt(f, pts, fmt="%.17g")
        f.write("</DataArray>\n</Points>\n<Cells>\n")
        f.write('<DataArray type="Int64" Name="connectivity" format="ascii">\n')
        np.savetxt(f, conn, fmt="%d")
        f.write('</DataArray>\n<DataArray type="Int64" Name="offsets" format="ascii">\n')
        np.savetxt(f, np.arange(nloc, nonods + nloc, nloc, dtype=np.int64), fmt="%d")
        f.write('</DataArray>\n<DataArray type="UInt8" Name="types" format="ascii">\n')
        np.savetxt(f, np.full(nele, cell, dtype=np.int64), fmt="%d")
        f.write("</DataArray>\n</Cells>\n<PointData>\n")
        for name, val in point_data.items():
            v = np.asarray(val, dtype=np.float64).reshape(nonods, -1)
            ncmp = v.shape[1]
            if ncmp == 2:
                v = np.concatenate([v, np.zeros((nonods, 1))], axis=1)
                ncmp = 3
            f.write('<DataArray Name="%s" type="Float64" NumberOfComponents="%d" format="ascii">\n' % (name, ncmp))
            np.savetxt(f, v, fmt="%.17g")
            f.write("</DataArray>\n")
        f.write("</PointData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n")
    return path


def save_solution(path: str, x) -> str:
    """``torch.save`` of the solution vector (the reference saves x_i the
    same way, main.py:216)."""
    import torch
    torch.save(x.detach().cpu() if hasattr(x, "detach") else torch.as_tensor(np.asarray(x)), path)
    return path
