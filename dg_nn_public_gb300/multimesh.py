"""Meshes of uneven size solved together: one block-diagonal operator.

The SIP-DG operator is block-sparse over elements, and elements of
different meshes share no face, so the disjoint union of several meshes is
one operator whose diagonal blocks are the meshes' own operators.  Every
stage of the solve -- the block streams of the smoothing, residual and
apply kernels, the DG->CG transfers, the Gram-Schmidt passes -- then runs as
one launch over the elements of all meshes, however uneven their sizes,
and the inner Arnoldi chunks are replayed as CUDA graphs as for a single
mesh.  The reference solves one mesh at a time
(z02-implicit/z06-DGtoCG/volume_mf_diff.py:33-150); this module has no
counterpart there.

What is shared and what is not:
  * the element blocks, the smoother, the right-hand side and the FP64
    residual are exactly each mesh's own (the union only renumbers);
  * each mesh keeps its own space-filling curve: mesh i's curve occupies
    positions offset_i + 1 .. offset_i + n_i of the union's curve, so the
    SFC levels aggregate along each mesh's curve (the one pair that can
    straddle two meshes on a coarse level couples them in the
    preconditioner only);
  * the Krylov space is shared (one GMRES for the block-diagonal system),
    so the meshes converge together; the solve runs to the smallest
    per-mesh tolerance, which bounds every mesh's residual by its own
    tolerance (||b_i - A_i x_i|| <= ||b - A x||), and each mesh's residual
    is checked on its own afterwards.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from .element import ElementTables, p3_element
from .mesh import DGMesh
from .solver import DGSolver, SolverConfig


@dataclass
class Segment:
    """Where one mesh lives in the union: elements [e0, e1), DOFs [d0, d1)."""
    e0: int
    e1: int
    d0: int
    d1: int


def union_mesh(meshes: Sequence[DGMesh], orders: Sequence[np.ndarray]):
    """Disjoint union of meshes of one element type.  Returns (mesh, sfc
    order, segments): face, vertex and curve numbers are offset per mesh."""
    if not meshes:
        raise ValueError("union_mesh needs at least one mesh")
    ndim, nloc = meshes[0].ndim, meshes[0].nloc
    if any(m.ndim != ndim or m.nloc != nloc for m in meshes):
        raise ValueError("all meshes of a union must have the same element type")
    nface = ndim + 1
    segs, xs, nbf, aln, bct, cgn, p1, coords, order = [], [], [], [], [], [], [], [], []
    e_off = v_off = g_off = 0
    nsets = max(len(m.bc_node_list) for m in meshes)
    bc = [[] for _ in range(nsets)]
    for m, o in zip(meshes, orders):
        o = np.asarray(o).reshape(-1)
        if o.size != m.cg_nonods:
            raise ValueError("SFC order size does not match its mesh")
        segs.append(Segment(e_off, e_off + m.nele, e_off * nloc, (e_off + m.nele) * nloc))
        xs.append(m.x_ref_in)
        f = np.asarray(m.nbf, dtype=np.int64)
        nbf.append(np.where(f >= 0, f + e_off * nface, f))
        aln.append(np.asarray(m.alnmt, dtype=np.int64))
        bct.append(np.asarray(m.glb_bcface_type, dtype=np.int64))
        cgn.append(np.asarray(m.cg_ndglno, dtype=np.int64) + g_off)
        p1.append(np.asarray(m.p1cg, dtype=np.int64) + v_off)
        coords.append(m.cg_coords)
        order.append(o.astype(np.int64) + v_off)
        for k in range(nsets):
            bc[k].append(np.asarray(m.bc_node_list[k]) if k < len(m.bc_node_list)
                         else np.zeros(m.nele * nloc, dtype=bool))
        e_off += m.nele
        v_off += m.cg_nonods
        g_off += int(np.asarray(m.cg_ndglno).max()) + 1
    u = DGMesh(ndim=ndim, nloc=nloc, nele=e_off, x_ref_in=np.concatenate(xs), nbf=np.concatenate(nbf),
               alnmt=np.concatenate(aln), glb_bcface_type=np.concatenate(bct), cg_ndglno=np.concatenate(cgn),
               p1cg=np.concatenate(p1), cg_nonods=v_off, cg_coords=np.concatenate(coords),
               bc_node_list=[np.concatenate(b) for b in bc], meta={"union_of": len(meshes)})
    return u, np.concatenate(order).reshape(-1, 1), segs


class MultiMeshSolver:
    """Several meshes (and per-mesh diffusivities) in one GPU operator."""

    def __init__(self, meshes: Sequence[DGMesh], orders: Sequence[np.ndarray], cfg: Optional[SolverConfig] = None,
                 el: Optional[ElementTables] = None, kappas: Optional[Sequence[Optional[np.ndarray]]] = None,
                 face_kappa: str = "mean", build: str = "affine"):
        self.meshes = list(meshes)
        self.mesh, self.order, self.segments = union_mesh(self.meshes, orders)
        self.solver = DGSolver(self.mesh, self.order, cfg, el or p3_element(self.mesh.ndim))
        self.solver.set_build_mode(build)
        if kappas is not None:
            self.solver.set_kappa(np.concatenate([np.ones(m.nele) if k is None else np.asarray(k, dtype=np.float64)
                                                  for m, k in zip(self.meshes, kappas)]))
            self.solver.set_face_kappa(face_kappa)
        self.solver.build_operator()

    def close(self):
        self.solver.close()

    def split(self, v) -> List:
        """Per-mesh views of a union vector."""
        return [v[sg.d0:sg.d1] for sg in self.segments]

    def rhs(self, fs):
        """Union right-hand side from per-mesh nodal sources (homogeneous
        Dirichlet data)."""
        import torch
        dev = "cuda:%d" % self.solver.cfg.device
        f = torch.cat([torch.as_tensor(np.asarray(fi, dtype=np.float64).reshape(-1)) for fi in fs]).to(dev)
        return self.solver.rhs(f.contiguous())

    def solve(self, fs, rtol: float = 1e-10, mode: str = "mixed"):
        """Solve every mesh's system to ||b_i - A_i x_i|| <= rtol ||b_i||.
        Returns (per-mesh solutions, inner iterations, per-mesh residual
        norms, per-mesh tolerances)."""
        import torch
        s = self.solver
        b = self.rhs(fs)
        tols = np.array([rtol * float(torch.linalg.norm(bi)) for bi in self.split(b)])
        tol = float(tols.min())
        x = torch.zeros_like(b)
        if mode == "mixed":
            its, _, _ = s.solve_mixed(x, b, tol, raise_noconv=True)
        elif mode == "fp64":
            its, _ = s.gmres(x, b, tol, raise_noconv=True)
        else:
            raise ValueError("mode must be 'mixed' or 'fp64'")
        r = s.residual(x, b)
        res = np.array([float(torch.linalg.norm(ri)) for ri in self.split(r)])
        return self.split(x), its, res, tols
