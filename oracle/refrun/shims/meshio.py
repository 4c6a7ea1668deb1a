"""Stand-in for meshio (not installed here) used when the reference runs as
the oracle: reads the Gmsh v2 ASCII meshes this project writes.

It exposes the attributes the reference reads (config.py:53-90,
mesh_init.py:744-836): ``points``, ``cells_dict``, ``cell_sets_dict`` and
``cell_data_dict['gmsh:geometrical']``.  The boundary physical sets come
first, then 'fluid', then a 'gmsh:bounding_entities' set holding the face
cells, so that the reference's label count ("sets holding face cells minus
one", mesh_init.py:782-787) equals the number of boundary sets.
"""
import numpy as np

_TYPES = {26: "line4", 21: "triangle10", 29: "tetra20"}


class Mesh:
    pass


def read(filename):
    with open(filename) as fh:
        tok = fh.read().split("\n")
    names, cells, phys, points = {}, {}, {}, None
    i = 0
    while i < len(tok):
        line = tok[i].strip()
        if line == "$PhysicalNames":
            n = int(tok[i + 1])
            for k in range(n):
                dim, tag, nm = tok[i + 2 + k].split(maxsplit=2)
                names[int(tag)] = (int(dim), nm.strip().strip('"'))
            i += n + 2
        elif line == "$Nodes":
            n = int(tok[i + 1])
            points = np.array([[float(v) for v in tok[i + 2 + k].split()[1:4]] for k in range(n)])
            i += n + 2
        elif line == "$Elements":
            n = int(tok[i + 1])
            for k in range(n):
                p = [int(v) for v in tok[i + 2 + k].split()]
                key = _TYPES[p[1]]
                ntag = p[2]
                cells.setdefault(key, []).append([v - 1 for v in p[3 + ntag:]])
                phys.setdefault(key, []).append(p[3])
            i += n + 2
        else:
            i += 1
    m = Mesh()
    m.points = points
    m.cells_dict = {k: np.asarray(v, dtype=np.int64) for k, v in cells.items()}
    phys = {k: np.asarray(v) for k, v in phys.items()}
    m.cell_data_dict = {"gmsh:physical": phys, "gmsh:geometrical": phys}
    sets = {}
    for tag in sorted(names):
        dim, nm = names[tag]
        sets[nm] = {k: np.nonzero(v == tag)[0] for k, v in phys.items() if np.any(v == tag)}
    face_key = "line4" if "triangle10" in m.cells_dict and "tetra20" not in m.cells_dict else "triangle10"
    sets["gmsh:bounding_entities"] = {face_key: np.arange(len(m.cells_dict.get(face_key, [])))}
    m.cell_sets_dict = sets
    return m
