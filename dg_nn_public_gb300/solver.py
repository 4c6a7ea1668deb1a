"""Host-side object around one libdgsip context (one mesh on one GPU).

``DGSolver`` owns a C-ABI context and exposes the solve stages on torch CUDA
tensors (FP64, element-major ``(nele, nloc)`` or flat).  It is the layer the
reference-compatible modules (``volume_mf_diff``, ``multigrid_linearelastic``,
``get_bdiag_diag``) are written on.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _capi
from .element import ElementTables, drst_duv, p3_element
from .mesh import DGMesh


@dataclass
class SolverConfig:
    """Solver knobs, named after the reference's config module (z06/config.py)."""
    eta_e: float = 90.0            # penalty (reference default 36; 10 p^2 here)
    mu_f: float = 1.0
    jac_wei: float = 2.0 / 3.0
    pre_smooth_its: int = 3
    post_smooth_its: int = 3
    gmres_m: int = 30
    gmres_its: int = 400
    device: int = 0


def _torch():
    import torch
    return torch


class DGSolver:
    """One mesh + operator resident on one GPU."""

    def __init__(self, mesh: DGMesh, sfc_order: np.ndarray, cfg: Optional[SolverConfig] = None,
                 el: Optional[ElementTables] = None):
        self.mesh = mesh
        self.cfg = cfg or SolverConfig()
        self.el = el or p3_element(mesh.ndim)
        L = _capi.lib()
        D = mesh.ndim
        keep = dict(
            x=np.ascontiguousarray(mesh.x_ref_in, dtype=np.float64),
            nbf=np.ascontiguousarray(mesh.nbf, dtype=np.int64),
            aln=np.ascontiguousarray(mesh.alnmt, dtype=np.int64),
            bct=np.ascontiguousarray(mesh.glb_bcface_type, dtype=np.int64),
            p1=np.ascontiguousarray(mesh.p1cg, dtype=np.int64),
            sfc=np.ascontiguousarray(np.asarray(sfc_order).reshape(-1), dtype=np.int64),
            n=np.ascontiguousarray(self.el.n), nlx=np.ascontiguousarray(self.el.nlx),
            w=np.ascontiguousarray(self.el.weight), sn=np.ascontiguousarray(self.el.sn),
            snlx=np.ascontiguousarray(self.el.snlx), sw=np.ascontiguousarray(self.el.sweight),
            al=np.ascontiguousarray(self.el.gi_align, dtype=np.int64),
            dr=np.ascontiguousarray(drst_duv(D).reshape(D + 1, D, D - 1)),
            P=np.ascontiguousarray(self.el.p1_to_p3),
        )
        self._keep = keep
        md = _capi.dg_mesh_desc(
            ndim=D, nloc=mesh.nloc, nele=mesh.nele, x_ref_in=keep["x"].ctypes.data,
            nbf=keep["nbf"].ctypes.data, alnmt=keep["aln"].ctypes.data,
            glb_bcface_type=keep["bct"].ctypes.data, cg_nonods=mesh.cg_nonods,
            p1cg=keep["p1"].ctypes.data, sfc_order=keep["sfc"].ctypes.data,
            ngi=self.el.ngi, sngi=self.el.sngi, n=keep["n"].ctypes.data, nlx=keep["nlx"].ctypes.data,
            weight=keep["w"].ctypes.data, sn=keep["sn"].ctypes.data, snlx=keep["snlx"].ctypes.data,
            sweight=keep["sw"].ctypes.data, gi_align=keep["al"].ctypes.data,
            drst_duv=keep["dr"].ctypes.data, p1_to_p3=keep["P"].ctypes.data)
        c = self.cfg
        cf = _capi.dg_config(eta_e=c.eta_e, mu_f=c.mu_f, jac_wei=c.jac_wei,
                             pre_smooth_its=c.pre_smooth_its, post_smooth_its=c.post_smooth_its,
                             device=c.device)
        h = C.c_void_p()
        _capi.check(L.dg_create(C.byref(md), C.byref(cf), C.byref(h)))
        self._ctx = h
        self._lib = L
        self.built = False
        self.nonods = mesh.nele * mesh.nloc
        info = self.info()
        self.ncola = int(info["ncola"])
        self.ncolor = int(info["ncolor"])
        self.nlevel = int(info["nlevel"])

    # -- plumbing --------------------------------------------------------
    @property
    def ctx(self):
        return self._ctx

    def _chk(self, rc):
        _capi.check(rc, self._ctx)

    @staticmethod
    def _stream():
        torch = _torch()
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _dev(self):
        return "cuda:%d" % self.cfg.device

    def _vec(self, n=None):
        torch = _torch()
        return torch.empty(self.nonods if n is None else n, dtype=torch.float64, device=self._dev())

    @staticmethod
    def _check_t(t, n):
        if t is None:
            return None
        if not (t.is_cuda and t.dtype == _torch().float64 and t.is_contiguous() and t.numel() == n):
            raise ValueError("expected a contiguous FP64 CUDA tensor with %d entries" % n)
        return t.data_ptr()

    def info(self):
        out = np.zeros(19, dtype=np.int64)
        self._chk(self._lib.dg_info(self._ctx, out.ctypes.data, 19))
        keys = ["ndim", "nloc", "nele", "nonods", "cg_nonods", "ncola", "ncolor", "nlevel", "nbface",
                "built", "ngi", "sngi", "tma_variant", "batched_tma", "shared_faces", "batched_kernel",
                "scaled_faces", "sc_variant", "device_bytes"]
        return dict(zip(keys, out.tolist()))

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.dg_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- operator --------------------------------------------------------
    def set_kappa(self, kappa: Optional[np.ndarray]):
        k = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
        self._keep["kappa"] = k
        self._chk(self._lib.dg_set_kappa(self._ctx, None if k is None else k.ctypes.data))
        self.built = False

    def set_face_kappa(self, mode: str):
        """Interior-face diffusivity: 'mean' = (k_e + k_nb)/2 (the reference's
        variable-property convention) or 'harmonic' = 2 k_e k_nb/(k_e + k_nb)
        (weighted-average SIP, coercive under large jumps).  Rebuild after."""
        self._chk(self._lib.dg_set_face_kappa(self._ctx, {"mean": 0, "harmonic": 1}[mode]))
        self.built = False

    def build_operator(self):
        self._chk(self._lib.dg_build_operator(self._ctx, self._stream()))
        self.built = True
        self.build_count = getattr(self, "build_count", 0) + 1

    def bdiag(self):
        torch = _torch()
        N = self.mesh.nloc
        K = torch.empty(self.mesh.nele, N, N, dtype=torch.float64, device=self._dev())
        d = torch.empty(self.mesh.nele, N, dtype=torch.float64, device=self._dev())
        self._chk(self._lib.dg_get_bdiag(self._ctx, K.data_ptr(), d.data_ptr(), self._stream()))
        return K, d

    def rar_values(self):
        v = self._vec(self.ncola)
        self._chk(self._lib.dg_get_rar(self._ctx, v.data_ptr(), self._stream()))
        return v

    # -- stages ----------------------------------------------------------
    def residual(self, x, b=None, r=None, x_out=None, smooth=False):
        """r = b - A x; with smooth also x_out <- smoothed x (may alias x)."""
        n = self.nonods
        r = self._vec() if r is None else r
        if smooth and x_out is None:
            x_out = x
        self._chk(self._lib.dg_residual(self._ctx, self._check_t(x, n), self._check_t(b, n),
                                        self._check_t(r, n), self._check_t(x_out, n) if smooth else None,
                                        1 if smooth else 0, self._stream()))
        return r

    def residual_norm_noalloc(self, x, b=None, r=None, norm_out=None):
        """r = b - A x and ||r||_2 through dg_residual_norm_noalloc, which
        allocates nothing (static device scratch; at most 524288 tetrahedra or
        1048576 triangles).  Pass r (or None to skip it) and a one-entry FP64
        device tensor norm_out to keep the call free of allocations; returns
        norm_out."""
        torch = _torch()
        n = self.nonods
        norm_out = torch.empty(1, dtype=torch.float64, device=self._dev()) if norm_out is None else norm_out
        self._chk(self._lib.dg_residual_norm_noalloc(self._ctx, self._check_t(x, n), self._check_t(b, n),
                                                     self._check_t(r, n), self._check_t(norm_out, 1),
                                                     self._stream()))
        return norm_out

    def apply(self, x, y=None):
        y = self._vec() if y is None else y
        self._chk(self._lib.dg_apply(self._ctx, self._check_t(x, self.nonods), self._check_t(y, self.nonods),
                                     self._stream()))
        return y

    def apply_f32(self, x, y=None):
        """y = A x with the FP32 operator copy (FP32 CUDA tensors)."""
        torch = _torch()
        if not (x.is_cuda and x.dtype == torch.float32 and x.is_contiguous() and x.numel() == self.nonods):
            raise ValueError("expected a contiguous FP32 CUDA tensor with %d entries" % self.nonods)
        y = torch.empty_like(x) if y is None else y
        self._chk(self._lib.dg_apply_f32(self._ctx, x.data_ptr(), y.data_ptr(), self._stream()))
        return y

    def precond_f32(self, r, z=None):
        """z = the mixed preconditioner applied once to r (FP32 CUDA tensors)."""
        torch = _torch()
        if not (r.is_cuda and r.dtype == torch.float32 and r.is_contiguous() and r.numel() == self.nonods):
            raise ValueError("expected a contiguous FP32 CUDA tensor with %d entries" % self.nonods)
        z = torch.empty_like(r) if z is None else z
        self._chk(self._lib.dg_precond_f32(self._ctx, r.data_ptr(), z.data_ptr(), self._stream()))
        return z

    def smooth_pc(self, x, b, x_out=None):
        """One smoothing step of the mixed preconditioner, x_out = x + W (b - A x),
        with its FP32/BF16 block copies (FP32 CUDA tensors; x_out distinct from x)."""
        torch = _torch()
        for t in (x, b):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.numel() == self.nonods):
                raise ValueError("expected a contiguous FP32 CUDA tensor with %d entries" % self.nonods)
        x_out = torch.empty_like(x) if x_out is None else x_out
        self._chk(self._lib.dg_smooth_pc(self._ctx, x.data_ptr(), b.data_ptr(), x_out.data_ptr(),
                                         self._stream()))
        return x_out

    def rhs(self, f, g=None, gn=None, b=None):
        n = self.nonods
        b = self._vec() if b is None else b
        self._chk(self._lib.dg_rhs(self._ctx, self._check_t(f, n), self._check_t(g, n), self._check_t(gn, n),
                                   self._check_t(b, n), self._stream()))
        return b

    def precond(self, r, z=None):
        z = self._vec() if z is None else z
        self._chk(self._lib.dg_precond(self._ctx, self._check_t(r, self.nonods), self._check_t(z, self.nonods),
                                       self._stream()))
        return z

    def mg_vcycle(self, r_sfc, e_sfc=None):
        n = self.mesh.cg_nonods
        e_sfc = self._vec(n) if e_sfc is None else e_sfc
        self._chk(self._lib.dg_mg_vcycle(self._ctx, self._check_t(r_sfc, n), self._check_t(e_sfc, n),
                                         self._stream()))
        return e_sfc

    def solve(self, f, g=None, rtol=1e-10, x0=None, out=None, mode="fp64"):
        """Solve A x = M f + lift(g) to ||b - A x|| <= rtol * ||b - A x0||.

        f, g: nodal source / Dirichlet data, (nele*nloc) FP64, on the host
        (numpy or torch CPU, preferably pinned) or on this GPU.  Host inputs
        are copied in and the solution copied back into ``out`` (a host
        tensor, allocated pinned when None); device inputs give a device
        solution.  Returns (x, its, final residual norm).
        """
        torch = _torch()
        dev = self._dev()
        on_host = not (isinstance(f, torch.Tensor) and f.is_cuda)

        def to_dev(a):
            if a is None:
                return None
            if isinstance(a, np.ndarray):
                a = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1))
            return a.reshape(-1).to(dev, non_blocking=True)
        fd, gd = to_dev(f), to_dev(g)
        b = self.rhs(fd, gd)
        x = torch.zeros_like(b) if x0 is None else to_dev(x0).clone()
        r0 = b if x0 is None else self.residual(x, b)
        tol = rtol * float(torch.linalg.norm(r0))
        if mode == "mixed":
            its, res, _ = self.solve_mixed(x, b, tol)
        elif mode == "fp64":
            its, res = self.gmres(x, b, tol)
        else:
            raise ValueError("mode must be 'fp64' or 'mixed'")
        if on_host:
            if out is None:
                out = torch.empty(self.nonods, dtype=torch.float64, pin_memory=True)
            out.copy_(x, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            return out, its, res
        return x, its, res

    def solve_mixed_batched(self, X, Bm, tol, m=None, max_its=None, inner_rtol=1e-3, raise_noconv=False):
        """Solve A X[q] = Bm[q] for up to 64 right-hand sides together (FP64
        CUDA tensors of shape (nrhs, nonods), in place on X), each to
        ||Bm[q] - A X[q]|| <= tol[q].  Returns (inner its, residual norms)
        per RHS as numpy arrays."""
        torch = _torch()
        if X.dim() != 2 or X.shape != Bm.shape or X.shape[1] != self.nonods:
            raise ValueError("X and Bm must be (nrhs, %d)" % self.nonods)
        nrhs = X.shape[0]
        for t in (X, Bm):
            if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("expected contiguous FP64 CUDA tensors")
        # restart 20 by default: the per-RHS Gram-Schmidt traffic grows with
        # the restart length (c4: m = 20 is 7% faster than 30, same iterations)
        m = min(20 if m is None else m, 31)
        max_its = 100 * m if max_its is None else max_its
        tolv = np.ascontiguousarray(np.broadcast_to(np.asarray(tol, dtype=np.float64), (nrhs,)))
        its = np.zeros(nrhs, dtype=np.int32)
        res = np.zeros(nrhs, dtype=np.float64)
        rc = self._lib.dg_solve_mixed_batched(self._ctx, X.data_ptr(), Bm.data_ptr(), nrhs, tolv.ctypes.data, m,
                                              max_its, float(inner_rtol), its.ctypes.data, res.ctypes.data,
                                              self._stream())
        if rc == _capi.DG_ERR_NOCONV and not raise_noconv:
            return its, res
        self._chk(rc)
        return its, res

    # -- multi-RHS stages (64 right-hand sides, RHS-interleaved FP32) ----
    BATCHED_KERNELS = ("cuda_cores", "mma_sync4", "mma_sync8", "mma_sync_bulk", "tcgen05_bulk", "tcgen05_split",
                       "tcgen05_ws")

    def _check_batched(self, t):
        torch = _torch()
        if t is None:
            return None
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.numel() == self.nonods * 64):
            raise ValueError("expected a contiguous FP32 CUDA tensor of nonods x 64 (RHS-interleaved)")
        return t.data_ptr()

    def apply_batched(self, x, y=None):
        """Y = A X for 64 RHS-interleaved FP32 right-hand sides."""
        y = _torch().empty_like(x) if y is None else y
        self._chk(self._lib.dg_apply_batched(self._ctx, self._check_batched(x), self._check_batched(y),
                                             self._stream()))
        return y

    def smooth_scaled(self, x, cv, x_out=None):
        """x_out = x + (cv - w x - sum_f S_f x_f) on the scaled face blocks
        S_f = W A_f, with cv = W b (the preconditioner's steps after its
        zero-start one; FP32 CUDA tensors, x_out distinct from x)."""
        torch = _torch()
        for t in (x, cv):
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.numel() == self.nonods):
                raise ValueError("expected a contiguous FP32 CUDA tensor with %d entries" % self.nonods)
        x_out = torch.empty_like(x) if x_out is None else x_out
        self._chk(self._lib.dg_smooth_scaled(self._ctx, x.data_ptr(), cv.data_ptr(), x_out.data_ptr(),
                                             self._stream()))
        return x_out

    def smooth_scaled_batched(self, x, cv, x_out=None):
        """smooth_scaled for 64 right-hand sides (RHS-interleaved FP32
        vectors, the layout of apply_batched)."""
        x_out = _torch().empty_like(cv) if x_out is None else x_out
        self._chk(self._lib.dg_smooth_scaled_batched(self._ctx, self._check_batched(x), self._check_batched(cv),
                                                     self._check_batched(x_out), self._stream()))
        return x_out

    def smooth_pc_batched(self, x, b, x_out=None):
        """X_out = X + W (B - A X) with the batched preconditioner's BF16
        copies (x None = zero guess), through the batched kernel in use."""
        x_out = _torch().empty_like(b) if x_out is None else x_out
        self._chk(self._lib.dg_smooth_pc_batched(self._ctx, self._check_batched(x), self._check_batched(b),
                                                 self._check_batched(x_out), self._stream()))
        return x_out

    def set_batched_kernel(self, kernel):
        """Batched smoothing kernel: None / "auto" (timed choice at the next
        batched solve) or one of BATCHED_KERNELS."""
        v = -1 if kernel in (None, "auto") else self.BATCHED_KERNELS.index(kernel)
        self._chk(self._lib.dg_set_batched_kernel(self._ctx, v))

    def batched_tuning(self):
        """(kernel in use, {kernel: us per launch} of the last timing)."""
        us = np.full(len(self.BATCHED_KERNELS), -1.0, dtype=np.float32)
        ch = C.c_int32(0)
        self._chk(self._lib.dg_batched_tuning(self._ctx, us.ctypes.data, us.size, C.byref(ch)))
        return self.BATCHED_KERNELS[ch.value], {k: float(u) for k, u in zip(self.BATCHED_KERNELS, us) if u >= 0}

    def set_mixed_options(self, smoother="blockinv", smooth_w=0.8, precond_bf16=True, dense_max=2400):
        """Mixed preconditioner: smoother 'jacobi3' (three point-Jacobi sweeps,
        as the reference) or 'blockinv' (smooth_w * A_ee^-1); BF16 block copies
        for the preconditioner; exact dense solve on the first SFC level with
        at most dense_max rows."""
        code = {"jacobi3": 0, "blockinv": 1}[smoother]
        self._chk(self._lib.dg_set_mixed_options(self._ctx, code, float(smooth_w), 1 if precond_bf16 else 0,
                                                 int(dense_max)))
        self.mixed_options = dict(smoother=smoother, smooth_w=float(smooth_w), precond_bf16=bool(precond_bf16),
                                  dense_max=int(dense_max))

    def set_launch_options(self, use_graph=True, use_pdl=True):
        """CUDA-graph replay of Arnoldi cycles and programmatic dependent
        launches inside a mixed inner step (both on by default)."""
        self._chk(self._lib.dg_set_launch_options(self._ctx, 1 if use_graph else 0, 1 if use_pdl else 0))

    def set_vcycle_cluster(self, cluster=-1):
        """SFC V-cycle legs of the mixed preconditioner as thread-block-cluster
        launches: -1 = auto (16 CTAs, else 8), 0 = the launch chain (the
        default), 8 / 16.  Returns the cluster size in use (0 = chain), or -1
        before the first mixed solve."""
        import ctypes as C
        out = C.c_int32(-1)
        self._chk(self._lib.dg_set_vcycle_cluster(self._ctx, int(cluster), C.byref(out)))
        return out.value

    # library defaults of the mixed preconditioner (dg_create)
    mixed_options = dict(smoother="blockinv", smooth_w=0.8, precond_bf16=True, dense_max=2400)

    def solve_mixed(self, x, b, tol, m=None, max_its=None, inner_rtol=1e-3, raise_noconv=False):
        """FP64 iterative refinement around an FP32 right-preconditioned
        flexible GMRES(m) with the FP32 copy of the multigrid preconditioner;
        in place on x until ||b - A x|| <= tol.  Returns (inner its, final
        residual norm, refinement steps)."""
        m = self.cfg.gmres_m if m is None else m
        max_its = self.cfg.gmres_its if max_its is None else max_its
        its = C.c_int32(0)
        outer = C.c_int32(0)
        res = C.c_double(0.0)
        rc = self._lib.dg_solve_mixed(self._ctx, self._check_t(x, self.nonods), self._check_t(b, self.nonods),
                                      float(tol), int(m), int(max_its), float(inner_rtol), C.byref(its),
                                      C.byref(res), C.byref(outer), self._stream())
        if rc == _capi.DG_ERR_NOCONV and not raise_noconv:
            return its.value, res.value, outer.value
        self._chk(rc)
        return its.value, res.value, outer.value

    def set_build_mode(self, mode):
        """Element-block assembly: "quadrature" (default; the reference's
        isoparametric formula at every quadrature point) or "affine"
        (reference matrices times per-element factors for straight-sided
        elements: equal to rounding, ~3.4x faster).  Next build_operator."""
        modes = {"quadrature": 0, "affine": 1}
        if mode not in modes:
            raise ValueError("build mode must be one of %s" % sorted(modes))
        self._chk(self._lib.dg_set_build_mode(self._ctx, modes[mode]))
        self.built = False

    def set_gmres_ortho(self, mode):
        """Arnoldi orthogonalisation of ``gmres``: "cgs2" (default) or "mgs",
        the reference's modified Gram-Schmidt order (z06/volume_mf_diff.py:1814-1819)."""
        modes = {"cgs2": 0, "mgs": 1}
        if mode not in modes:
            raise ValueError("gmres ortho must be one of %s" % sorted(modes))
        self._chk(self._lib.dg_set_gmres_ortho(self._ctx, modes[mode]))

    def gmres(self, x, b, tol, m=None, max_its=None, raise_noconv=False):
        """Restarted GMRES(m) in place on x; returns (its, final ||b - A x||)."""
        m = self.cfg.gmres_m if m is None else m
        max_its = self.cfg.gmres_its if max_its is None else max_its
        its = C.c_int32(0)
        res = C.c_double(0.0)
        rc = self._lib.dg_gmres(self._ctx, self._check_t(x, self.nonods), self._check_t(b, self.nonods),
                                float(tol), int(m), int(max_its), C.byref(its), C.byref(res), self._stream())
        if rc == _capi.DG_ERR_NOCONV and not raise_noconv:
            return its.value, res.value
        self._chk(rc)
        return its.value, res.value
