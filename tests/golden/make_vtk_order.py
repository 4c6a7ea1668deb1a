"""Extract the reference's VTK node-order tables (P3 tetrahedron and
triangle) from z02-implicit/z06-DGtoCG/mesh_init.py as text (the module is
not executed) into vtk_node_order.npz.

    python tests/golden/make_vtk_order.py /path/to/reference   (or $DG_REFERENCE_DIR)
"""
import ast
import os
import sys

import numpy as np

ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DG_REFERENCE_DIR")
if not ref:
    raise SystemExit("pass the reference checkout as the argument or set DG_REFERENCE_DIR")
src = open(os.path.join(ref, "z02-implicit", "z06-DGtoCG", "mesh_init.py")).read()
tables = []
for node in ast.walk(ast.parse(src)):
    if isinstance(node, ast.Assign) and any(getattr(t, "id", None) == "ref_node_order" for t in node.targets):
        if isinstance(node.value, ast.List):
            tables.append([ast.literal_eval(e) for e in node.value.elts])
tet = [t for t in tables if len(t) == 20][0]
tri = [t for t in tables if len(t) == 10][0]
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "vtk_node_order.npz")
np.savez(out, tet=np.array(tet), tri=np.array(tri))
print(out, tet, tri)
