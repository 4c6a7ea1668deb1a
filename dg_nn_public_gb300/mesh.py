"""Synthetic P3 meshes and the mesh ingest that yields the solver's arrays.

Two jobs live here:

* generators for the benchmark meshes -- the unit square split into CCW
  triangles and the unit cube split into Kuhn (6-tet) simplices, interior
  vertices jittered uniformly from a seed, cubic nodes on straight edges --
  and a Gmsh v2 ASCII writer (the reference reads meshes with meshio from
  that format; z02-implicit/z06-DGtoCG/config.py:53);
* ``ingest``: the restatement of the reference's ``init_2d``/``init_3d`` +
  ``get_bc_node_fsi`` (z02-implicit/z06-DGtoCG/mesh_init.py:10-257,
  260-658, 744-836) that turns Gmsh-ordered cells into the per-element
  arrays the operator needs: ``x_ref_in (nele, ndim, nloc)``, the face
  neighbour table ``nbf``, the quadrature alignment code ``alnmt`` and the
  boundary type ``glb_bcface_type`` of every face ``ele * nface + iface``,
  and the P1CG vertex numbering.  The integer outputs are bit-identical to
  the reference's; the face matching uses a sorted-key join instead of the
  reference's element-adjacency scan, which yields the same unique pairs.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .element import TET_FACE_CORNERS, TRI_FACE_CORNERS, TET_FACE_NODES, TRI_FACE_NODES

# Gmsh element type ids (Gmsh v2 format).
GMSH_LINE4 = 26
GMSH_TRI10 = 21
GMSH_TET20 = 29

# Reference's reorder of a Gmsh tetra20 whose corners are right-handed
# (mesh_init.py:275-289): internal node i = gmsh node TET_REORDER[i].
TET_REORDER = np.array([3, 1, 2, 0, 12, 13, 14, 15, 6, 7, 10, 11, 5, 4, 8, 9, 16, 19, 18, 17],
                       dtype=np.int64)
# ... and of a clockwise triangle10 (mesh_init.py:20-21).
TRI_REORDER = np.array([0, 2, 1, 8, 7, 6, 5, 4, 3, 9], dtype=np.int64)


@dataclass
class GmshMesh:
    """A mesh in Gmsh node ordering, as a Gmsh v2 file would hold it."""
    ndim: int
    points: np.ndarray            # (npoints, 3) float64
    cells: np.ndarray             # (nele, nloc) int64, 0-based, gmsh order
    bfaces: np.ndarray            # (nbface, snodes) int64, boundary face cells
    bface_tag: np.ndarray         # (nbface,) int64 physical set id (0 = first set)
    set_names: tuple = ("Dirichlet",)
    meta: dict = field(default_factory=dict)

    @property
    def nele(self) -> int:
        return int(self.cells.shape[0])


# ---------------------------------------------------------------------------
# generators

def _edge_key(a, b):
    return (a, b) if a < b else (b, a)


class _NodeBuilder:
    """Creates shared high-order nodes on straight edges / faces."""

    def __init__(self, verts: np.ndarray):
        self.coords = [v for v in verts]
        self.nvert = len(verts)
        self.edge_nodes = {}
        self.face_nodes = {}

    def _add(self, x):
        self.coords.append(x)
        return len(self.coords) - 1

    def edge(self, a, b):
        """The two interior nodes of edge a->b, ordered from a to b."""
        key = _edge_key(a, b)
        if key not in self.edge_nodes:
            p, q = np.asarray(self.coords[key[0]]), np.asarray(self.coords[key[1]])
            n1 = self._add((2.0 * p + q) / 3.0)
            n2 = self._add((p + 2.0 * q) / 3.0)
            self.edge_nodes[key] = (n1, n2)
        n1, n2 = self.edge_nodes[key]
        return (n1, n2) if a == key[0] else (n2, n1)

    def face(self, a, b, c):
        key = tuple(sorted((a, b, c)))
        if key not in self.face_nodes:
            p, q, r = (np.asarray(self.coords[k]) for k in key)
            self.face_nodes[key] = self._add((p + q + r) / 3.0)
        return self.face_nodes[key]

    def points(self):
        return np.asarray(self.coords, dtype=np.float64)


def _jittered_grid(n: int, ndim: int, jitter: float, seed: int) -> np.ndarray:
    """Vertices of the unit square/cube, x index fastest, interior jittered."""
    h = 1.0 / n
    ax = np.arange(n + 1, dtype=np.float64) * h
    if ndim == 2:
        yy, xx = np.meshgrid(ax, ax, indexing="ij")
        verts = np.stack([xx.ravel(), yy.ravel(), np.zeros(xx.size)], axis=1)
    else:
        zz, yy, xx = np.meshgrid(ax, ax, ax, indexing="ij")
        verts = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)
    interior = np.all((verts[:, :ndim] > 0.5 * h) & (verts[:, :ndim] < 1.0 - 0.5 * h), axis=1)
    rng = np.random.default_rng(seed)
    idx = np.nonzero(interior)[0]
    shift = rng.uniform(-jitter * h, jitter * h, size=(idx.size, ndim))
    verts[idx, :ndim] += shift
    return verts


def unit_square_tri_mesh(n: int, jitter: float = 0.2, seed: int = 0) -> GmshMesh:
    """n x n squares, each split into two CCW triangles; P3 triangle10 cells."""
    verts = _jittered_grid(n, 2, jitter, seed)
    vid = lambda i, j: i + (n + 1) * j
    nb = _NodeBuilder(verts)
    cells = []
    for j in range(n):
        for i in range(n):
            v00, v10, v11, v01 = vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)
            for tri in ((v00, v10, v11), (v00, v11, v01)):
                a, b, c = tri
                e01, e12, e20 = nb.edge(a, b), nb.edge(b, c), nb.edge(c, a)
                cells.append([a, b, c, e01[0], e01[1], e12[0], e12[1], e20[0], e20[1],
                              nb.face(a, b, c)])
    cells = np.asarray(cells, dtype=np.int64)
    # boundary edges (line4: end points first, then the two interior nodes)
    bfaces = []
    for tri in cells:
        for (p, q), (e1, e2) in (((0, 1), (3, 4)), ((1, 2), (5, 6)), ((2, 0), (7, 8))):
            a, b = tri[p], tri[q]
            pa, pb = verts[a], verts[b]
            on_bnd = any((abs(pa[d] - s) < 1e-14 and abs(pb[d] - s) < 1e-14)
                         for d in range(2) for s in (0.0, 1.0))
            if on_bnd:
                bfaces.append([a, b, tri[e1], tri[e2]])
    bfaces = np.asarray(bfaces, dtype=np.int64)
    return GmshMesh(ndim=2, points=nb.points(), cells=cells, bfaces=bfaces,
                    bface_tag=np.zeros(len(bfaces), dtype=np.int64),
                    meta=dict(kind="square-tri", n=n, jitter=jitter, seed=seed))


_KUHN_PERMS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


def unit_cube_kuhn_mesh(n: int, jitter: float = 0.15, seed: int = 0) -> GmshMesh:
    """n^3 cubes, each split into the 6 Kuhn tetrahedra along the main diagonal.

    Every tetra20 cell is positively oriented in Gmsh corner order
    (det(x1-x0, x2-x0, x3-x0) > 0), as the reference's reorder rule expects.
    """
    verts = _jittered_grid(n, 3, jitter, seed)
    vid = lambda i, j, k: i + (n + 1) * (j + (n + 1) * k)
    nb = _NodeBuilder(verts)
    cells = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                for perm in _KUHN_PERMS:
                    p = [0, 0, 0]
                    path = [vid(i, j, k)]
                    for ax in perm:
                        p[ax] += 1
                        path.append(vid(i + p[0], j + p[1], k + p[2]))
                    v0, v1, v2, v3 = path
                    x = verts[[v0, v1, v2, v3]]
                    if np.linalg.det(x[1:] - x[0]) < 0:
                        v1, v2 = v2, v1
                    e = {}
                    for a, b in ((v0, v1), (v1, v2), (v2, v0), (v3, v0), (v3, v2), (v3, v1)):
                        e[(a, b)] = nb.edge(a, b)
                    cells.append([
                        v0, v1, v2, v3,
                        *e[(v0, v1)], *e[(v1, v2)], *e[(v2, v0)],
                        *e[(v3, v0)], *e[(v3, v2)], *e[(v3, v1)],
                        nb.face(v0, v2, v1), nb.face(v0, v1, v3),
                        nb.face(v0, v3, v2), nb.face(v3, v1, v2)])
    cells = np.asarray(cells, dtype=np.int64)
    pts = nb.points()
    # boundary triangles (triangle10 in gmsh order), taken from the cells
    face_local = ((0, 2, 1), (0, 1, 3), (0, 3, 2), (3, 1, 2))
    keys = {}
    for c in cells:
        for fl in face_local:
            key = tuple(sorted(c[list(fl)]))
            keys[key] = keys.get(key, 0) + 1
    bfaces = []
    for key, cnt in keys.items():
        if cnt == 1:
            a, b, cc = key
            e1, e2, e3 = nb.edge(a, b), nb.edge(b, cc), nb.edge(cc, a)
            bfaces.append([a, b, cc, e1[0], e1[1], e2[0], e2[1], e3[0], e3[1], nb.face(a, b, cc)])
    bfaces = np.asarray(sorted(bfaces), dtype=np.int64)
    return GmshMesh(ndim=3, points=pts, cells=cells, bfaces=bfaces,
                    bface_tag=np.zeros(len(bfaces), dtype=np.int64),
                    meta=dict(kind="cube-kuhn", n=n, jitter=jitter, seed=seed))


# ---------------------------------------------------------------------------
# Gmsh v2 ASCII writer / reader

def write_gmsh22(path: str, mesh: GmshMesh) -> None:
    """Write physical groups (boundary sets, then 'fluid') and all cells."""
    vol_type, face_type = (GMSH_TET20, GMSH_TRI10) if mesh.ndim == 3 else (GMSH_TRI10, GMSH_LINE4)
    nset = len(mesh.set_names)
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames", str(nset + 1)]
    for i, name in enumerate(mesh.set_names):
        lines.append('%d %d "%s"' % (mesh.ndim - 1, i + 1, name))
    lines.append('%d %d "fluid"' % (mesh.ndim, nset + 1))
    lines += ["$EndPhysicalNames", "$Nodes", str(len(mesh.points))]
    for i, p in enumerate(mesh.points):
        lines.append("%d %r %r %r" % (i + 1, float(p[0]), float(p[1]), float(p[2])))
    lines += ["$EndNodes", "$Elements", str(len(mesh.bfaces) + mesh.nele)]
    eid = 1
    for f, tag in zip(mesh.bfaces, mesh.bface_tag):
        lines.append("%d %d 2 %d %d %s" % (eid, face_type, tag + 1, tag + 1,
                                             " ".join(str(int(v) + 1) for v in f)))
        eid += 1
    for c in mesh.cells:
        lines.append("%d %d 2 %d %d %s" % (eid, vol_type, nset + 1, nset + 1,
                                             " ".join(str(int(v) + 1) for v in c)))
        eid += 1
    lines.append("$EndElements")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_gmsh22(path: str) -> dict:
    """Minimal Gmsh v2 ASCII reader: points, cells per type, physical tags."""
    with open(path) as fh:
        tok = fh.read().split("\n")
    i = 0
    names = {}
    points = None
    cells = {}
    phys = {}
    while i < len(tok):
        line = tok[i].strip()
        if line == "$PhysicalNames":
            n = int(tok[i + 1])
            for k in range(n):
                parts = tok[i + 2 + k].split(maxsplit=2)
                names[int(parts[1])] = (int(parts[0]), parts[2].strip().strip('"'))
            i += n + 2
        elif line == "$Nodes":
            n = int(tok[i + 1])
            arr = np.array([tok[i + 2 + k].split() for k in range(n)], dtype=object)
            points = arr[:, 1:4].astype(np.float64)
            i += n + 2
        elif line == "$Elements":
            n = int(tok[i + 1])
            for k in range(n):
                parts = [int(v) for v in tok[i + 2 + k].split()]
                etype, ntag = parts[1], parts[2]
                tags = parts[3:3 + ntag]
                nodes = [v - 1 for v in parts[3 + ntag:]]
                cells.setdefault(etype, []).append(nodes)
                phys.setdefault(etype, []).append(tags[0] if tags else 0)
            i += n + 2
        else:
            i += 1
    return dict(points=points, names=names,
                cells={k: np.asarray(v, dtype=np.int64) for k, v in cells.items()},
                phys={k: np.asarray(v, dtype=np.int64) for k, v in phys.items()})


def gmsh_mesh_from_file(path: str) -> GmshMesh:
    d = read_gmsh22(path)
    if GMSH_TET20 in d["cells"]:
        ndim, vol, face = 3, GMSH_TET20, GMSH_TRI10
    elif GMSH_TRI10 in d["cells"]:
        ndim, vol, face = 2, GMSH_TRI10, GMSH_LINE4
    else:
        raise ValueError("the mesh holds neither tetra20 nor triangle10 cells")
    bnames = sorted((tag, nm) for tag, (dim, nm) in d["names"].items() if dim == ndim - 1)
    tag_to_set = {tag: k for k, (tag, _) in enumerate(bnames)}
    bf = d["cells"].get(face, np.zeros((0, 10 if ndim == 3 else 4), dtype=np.int64))
    bt = np.array([tag_to_set.get(int(t), -1) for t in d["phys"].get(face, [])], dtype=np.int64)
    return GmshMesh(ndim=ndim, points=d["points"], cells=d["cells"][vol], bfaces=bf,
                    bface_tag=bt, set_names=tuple(nm for _, nm in bnames))


# ---------------------------------------------------------------------------
# ingest: Gmsh cells -> solver arrays (restates mesh_init.py)

@dataclass
class DGMesh:
    """Per-element arrays of a P3 DG mesh in the reference's internal layout."""
    ndim: int
    nloc: int
    nele: int
    x_ref_in: np.ndarray          # (nele, ndim, nloc) float64
    nbf: np.ndarray               # (nele*nface,) int64, -1 on boundary
    alnmt: np.ndarray             # (nele*nface,) int64, -1 on boundary
    glb_bcface_type: np.ndarray   # (nele*nface,) int64: -1 interior, k = boundary set k
    cg_ndglno: np.ndarray         # (nele, nloc) gmsh node ids in internal order
    p1cg: np.ndarray              # (nele, ndim+1) P1CG vertex numbers (0-based)
    cg_nonods: int
    cg_coords: np.ndarray         # (cg_nonods, ndim) vertex coordinates
    bc_node_list: list            # per boundary set: (nele*nloc,) bool
    meta: dict = field(default_factory=dict)

    @property
    def nface(self) -> int:
        return self.ndim + 1

    @property
    def nonods(self) -> int:
        return self.nele * self.nloc


def _internal_cells(g: GmshMesh) -> np.ndarray:
    cells = g.cells.copy()
    pts = g.points
    if g.ndim == 3:
        x = pts[cells[:, :4]]
        det = np.linalg.det(x[:, 1:4, :] - x[:, 0:1, :])
        flip = det > 0
        cells[flip] = cells[flip][:, TET_REORDER]
    else:
        # the reference decides on the mesh's first three points for every
        # triangle (mesh_init.py:27-36)
        xl = pts[0:3].copy()
        xl[:, -1] = 1.0
        if np.linalg.det(xl) < 0:
            cells = cells[:, TRI_REORDER]
    return cells


def ingest(g: GmshMesh) -> DGMesh:
    ndim = g.ndim
    nface = ndim + 1
    cells = _internal_cells(g)
    nele, nloc = cells.shape
    corners = TET_FACE_CORNERS if ndim == 3 else TRI_FACE_CORNERS
    fnodes = np.stack([cells[:, list(c)] for c in corners], axis=1)      # (nele, nface, ndim)
    fnodes = fnodes.reshape(nele * nface, ndim)
    key = np.sort(fnodes, axis=1)
    # face matching by sorted corner key
    order = np.lexsort(key.T[::-1])
    ks = key[order]
    same = np.all(ks[1:] == ks[:-1], axis=1)
    if np.any(same[1:] & same[:-1]):
        raise ValueError("a face is shared by more than two elements")
    nbf = np.full(nele * nface, -1, dtype=np.int64)
    alnmt = np.full(nele * nface, -1, dtype=np.int64)
    i1 = order[:-1][same]
    i2 = order[1:][same]
    nbf[i1] = i2
    nbf[i2] = i1
    lo, hi = np.minimum(i1, i2), np.maximum(i1, i2)
    fa, fb = fnodes[lo], fnodes[hi]
    if ndim == 3:
        code = np.where(fa[:, 0] == fb[:, 0], 0, np.where(fa[:, 1] == fb[:, 0], 1, 2))
    else:
        code = np.where(fa[:, 0] == fb[:, 0], 0, 1)
    alnmt[lo] = code
    alnmt[hi] = code
    # boundary faces -> physical set of the matching boundary cell
    glb_bcface_type = np.full(nele * nface, -1, dtype=np.int64)
    face_loc = TET_FACE_NODES if ndim == 3 else TRI_FACE_NODES
    nsets = max(len(g.set_names), 1)
    bc_node_list = [np.zeros(nele * nloc, dtype=bool) for _ in range(nsets)]
    bnd = np.nonzero(alnmt < 0)[0]
    if bnd.size and g.bfaces.size:
        bkey = np.sort(g.bfaces[:, :ndim], axis=1)
        lookup = {tuple(k): t for k, t in zip(bkey.tolist(), g.bface_tag.tolist())}
        for f in bnd.tolist():
            t = lookup.get(tuple(key[f].tolist()))
            if t is None or t < 0:
                continue
            glb_bcface_type[f] = t
            ele, iface = divmod(f, nface)
            bc_node_list[t][ele * nloc + face_loc[iface]] = True
    pts = g.points if ndim == 3 else g.points[:, :2]
    x_ref_in = np.ascontiguousarray(pts[cells].transpose(0, 2, 1))
    corner_ids = cells[:, :ndim + 1]
    uniq, inv = np.unique(corner_ids.ravel(), return_inverse=True)
    p1cg = inv.reshape(nele, ndim + 1).astype(np.int64)
    return DGMesh(ndim=ndim, nloc=nloc, nele=nele, x_ref_in=x_ref_in, nbf=nbf, alnmt=alnmt,
                  glb_bcface_type=glb_bcface_type, cg_ndglno=cells, p1cg=p1cg,
                  cg_nonods=int(uniq.size), cg_coords=pts[uniq].copy(),
                  bc_node_list=bc_node_list, meta=dict(g.meta))


def build_mesh(kind: str, n: int, jitter: Optional[float] = None, seed: int = 0) -> DGMesh:
    """Generate and ingest one of the benchmark meshes ('tri' or 'tet')."""
    if kind == "tri":
        g = unit_square_tri_mesh(n, 0.2 if jitter is None else jitter, seed)
    elif kind == "tet":
        g = unit_cube_kuhn_mesh(n, 0.15 if jitter is None else jitter, seed)
    else:
        raise ValueError(kind)
    m = ingest(g)
    m.meta.update(g.meta)
    return m


def mesh_cache_path(kind: str, n: int, seed: int, root: Optional[str] = None) -> str:
    root = root or os.path.join(os.path.expanduser("~"), ".cache", "dg_nn_public_gb300")
    return os.path.join(root, "%s_n%d_s%d.npz" % (kind, n, seed))
