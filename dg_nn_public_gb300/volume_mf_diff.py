"""Drop-in for the reference's ``volume_mf_diff`` module (z02-implicit/z06-DGtoCG/volume_mf_diff.py).

Same function names, argument meaning and in-place behaviour as the
reference, on FP64 CUDA tensors, executed by libdgsip through the C ABI.
State (mesh, operator, knobs) lives in ``dg_nn_public_gb300.state`` in place
of the reference's ``config`` module and ``sf_nd_nb`` singleton; bind a mesh
first with ``state.bind(...)`` or ``state.bind_reference_funcspace(...)``.

Differences a caller can observe:
  * the operator (element blocks, colour-probe P1CG operator, SFC levels) is
    assembled once per bound mesh / diffusivity and reused, where the
    reference rebuilds the P1CG operator and SFC levels inside every
    ``solve_for_diff`` call;
  * GMRES orthogonalises with CGS2 instead of MGS (results agree to
    roundoff; the iteration counts match on every pinned case);
  * ``_k_res_one_batch`` / ``_s_res_one_batch`` are not split: the stored
    element blocks hold volume and face terms together, so the combined
    ``get_residual_or_smooth`` is the entry point.
"""
from __future__ import annotations

import numpy as np

from .state import config, ensure_operator, sf_nd_nb, solver


def _torch():
    import torch
    return torch


def _flat(t):
    return t.reshape(-1)


def get_residual_or_smooth(r0, x_i, x_rhs, do_smooth=False):
    """r0 += x_rhs - A x_i; with do_smooth also x_i += w * (3 block-Jacobi
    sweeps on r0) in place.  Returns (r0, x_i) flattened (:403-483)."""
    s = ensure_operator()
    r = _flat(r0)
    x = _flat(x_i)
    if isinstance(x_rhs, (int, float)):
        b = r + float(x_rhs) if x_rhs != 0 else r.clone()
    else:
        b = r + _flat(x_rhs)
    s.residual(x, b, r=r, x_out=x if do_smooth else None, smooth=bool(do_smooth))
    return r, x


def _um_left_precond(x_i, x_rhs):
    """One DG->CG + SFC multigrid V-cycle on x_rhs from the guess x_i
    (:1934-2029).  For a nonzero guess the result is x + M(x_rhs - A x)."""
    torch = _torch()
    s = ensure_operator()
    x = _flat(x_i)
    r = _flat(x_rhs)
    if int(torch.count_nonzero(x)) == 0:
        x.copy_(s.precond(r.contiguous()))
    else:
        res = s.residual(x, r.contiguous())
        x.add_(s.precond(res))
    return x_i


def _get_rhs(x_rhs, f, u_bc, alpha_x_i):
    """x_rhs += M f + Dirichlet lifting of u_bc[0] (+ Neumann u_bc[1])
    (:153-359); with sf_nd_nb.isTransient also + M alpha_x_i / dt."""
    s = ensure_operator()
    g = u_bc[0] if len(u_bc) > 0 else None
    gn = u_bc[1] if len(u_bc) > 1 else None
    b = s.rhs(_flat(f).contiguous(), None if g is None else _flat(g).contiguous(),
              None if gn is None else _flat(gn).contiguous())
    if sf_nd_nb.isTransient and alpha_x_i is not None:
        b.add_(s.rhs((_flat(alpha_x_i) / sf_nd_nb.dt).contiguous()))
    out = _flat(x_rhs)
    out.add_(b)
    return x_rhs


def _host(a):
    if a is None:
        return None
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def bound_p1cg_structures(s=None):
    """P1CG sparsity (fina, cola, 0-based) and distance-2 colouring (whichc,
    ncolor) of the bound mesh, as the reference forms them
    (z06/sparsity.py:102-122, 235-269); host arrays, cached per solver."""
    from . import _capi
    s = s or ensure_operator()
    st = getattr(s, "_p1cg_host", None)
    if st is None:
        fina, cola = _capi.p1cg_sparsity(s.mesh.p1cg, s.mesh.cg_nonods)
        whichc, ncolor = _capi.color2(fina, cola)
        st = dict(fina=fina, cola=cola, whichc=whichc, ncolor=ncolor)
        s._p1cg_host = st
    return st


def _require_same(name, given, bound):
    g = _host(given)
    if g is None:
        return
    b = np.asarray(bound)
    if g.shape != b.shape and g.size == b.size:
        g = g.reshape(b.shape)
    if g.shape != b.shape or not np.array_equal(g, b):
        raise ValueError("%s differs from the bound mesh's (%s given, %s bound): the GPU operator is assembled "
                         "for the mesh bound with state.bind(); rebind to use other structures"
                         % (name, g.shape, b.shape))


def _calc_RAR_mf_color(I_fc=None, I_cf=None, whichc=None, ncolor=None, spIdx_for_color=None,
                       colIdx_for_color=None, fina=None, cola=None, ncola=None):
    """Galerkin P1CG operator values of the bound mesh (:1696-1754).  The
    arguments the reference passes are checked against the bound mesh's
    P1CG structures: a different sparsity, colouring or transfer shape
    raises ValueError instead of returning the bound operator silently."""
    s = ensure_operator()
    st = bound_p1cg_structures(s)
    _require_same("fina", fina, st["fina"])
    _require_same("cola", cola, st["cola"])
    _require_same("whichc", whichc, st["whichc"])
    if ncolor is not None and int(ncolor) != st["ncolor"]:
        raise ValueError("ncolor %d differs from the bound mesh's %d" % (int(ncolor), st["ncolor"]))
    if ncola is not None and int(ncola) != st["cola"].size:
        raise ValueError("ncola %d differs from the bound mesh's %d" % (int(ncola), st["cola"].size))
    ncg, ndg = s.mesh.cg_nonods, s.mesh.nele * (s.mesh.ndim + 1)
    for name, M, shape in (("I_fc", I_fc, (ndg, ncg)), ("I_cf", I_cf, (ncg, ndg))):
        if M is not None and tuple(M.shape) != shape:
            raise ValueError("%s has shape %s, the bound mesh's is %s" % (name, tuple(M.shape), shape))
    return s.rar_values()


def _sfc_level_data(s):
    """variables_sfc in the reference's format (multigrid_linearelastic.py:
    42-109, 250-283): per level (torch CSR level matrix, diagonal (1, n), n),
    the coarsest level as (scipy CSR, 0, n); built on the host from the
    bound operator's P1CG values by the same aggregation the device levels
    use (compact_fcode.f90 summation order)."""
    import scipy.sparse as sp
    import torch
    from . import _capi
    st = bound_p1cg_structures(s)
    order = np.asarray(sf_nd_nb.sfc_data_Um.space_filling_curve_numbering).reshape(-1)
    nl, start, rowp, col, val = _capi.sfc_levels(st["fina"], st["cola"], s.rar_values().cpu().numpy(), order)
    out, sizes = [], []
    for lev in range(nl):
        r0, r1 = int(start[lev]), int(start[lev + 1])
        n = r1 - r0
        crow = rowp[r0:r1 + 1] - rowp[r0]
        c = col[int(rowp[r0]):int(rowp[r1])]
        v = val[int(rowp[r0]):int(rowp[r1])]
        sizes.append(n)
        if lev == nl - 1:
            out.append((sp.csr_matrix((v.copy(), c.copy(), crow.copy()), shape=(n, n)), 0, n))
            continue
        # rows sorted by column, as the reference's torch CSR level matrices
        rows = np.repeat(np.arange(n), np.diff(crow))
        perm = np.lexsort((c, rows))
        c, v = c[perm], v[perm]
        diag = np.zeros((1, n))
        on = c == rows
        diag[0, rows[on]] = v[on]
        A = torch.sparse_csr_tensor(torch.tensor(crow), torch.tensor(c), torch.tensor(v), size=(n, n),
                                    dtype=torch.float64)
        out.append((A, torch.tensor(diag), n))
    return nl, sizes, out


def _get_RAR_and_sfc_data_Um():
    """Assemble the P1CG operator and the SFC levels (:1642-1693); the level
    data are stored in sf_nd_nb.sfc_data_Um as the reference stores them."""
    s = ensure_operator()
    sd = sf_nd_nb.sfc_data_Um
    version = (id(s), s.build_count)
    if getattr(sd, "_version", None) != version:
        nl, sizes, levels = _sfc_level_data(s)
        sd.set_data(nlevel=nl, nodes_per_level=sizes, variables_sfc=levels)
        sd._version = version
    return 0


def _gmres_mg_solver(x_i, x_rhs, tol):
    """Left-preconditioned restarted GMRES (:1757-1841); tol is absolute on
    ||b - A x||, tested after each restart cycle.  Returns (x_i, its)."""
    s = ensure_operator()
    x = _flat(x_i)
    its, res = s.gmres(x, _flat(x_rhs).contiguous(), tol, m=config.gmres_m, max_its=config.gmres_its)
    sf_nd_nb.its = its
    return x_i, its


def _mg_solver(x_i, x_rhs, tol):
    """Multigrid as a stand-alone iteration (:1844-1873)."""
    torch = _torch()
    s = ensure_operator()
    x = _flat(x_i)
    b = _flat(x_rhs).contiguous()
    r = s.residual(x, b)
    r0l2 = 1.0
    its = 0
    while r0l2 > tol and its < config.gmres_its:
        x.add_(s.precond(r))
        s.residual(x, b, r=r)
        r0l2 = float(torch.linalg.norm(r))
        its += 1
    sf_nd_nb.its = its
    return x_i, its


def _cg_mg_solver(x_i, x_rhs, tol):
    """Preconditioned conjugate gradients with the multigrid preconditioner (:1875-1931)."""
    torch = _torch()
    s = ensure_operator()
    x = _flat(x_i)
    b = _flat(x_rhs).contiguous()
    r = s.residual(x, b)
    z = s.precond(r)
    p = z.clone()
    Ap = torch.empty_like(p)
    r0l2 = 1.0
    its = 0
    while r0l2 > tol and its < config.gmres_its:
        s.apply(p, Ap)
        rz = torch.dot(r, z)
        alpha = rz / torch.dot(Ap, p)
        x.add_(alpha * p)
        r.sub_(alpha * Ap)
        s.precond(r, z)
        r0l2 = float(torch.linalg.norm(r))
        beta = torch.dot(r, z) / rz
        p.mul_(beta).add_(z)
        its += 1
    sf_nd_nb.its = its
    return x_i, its


def solve_for_diff(x_i, f, u_bc, alpha_x_i, t=None):
    """Steady diffusion solve (:33-150): assemble the operator if needed,
    form the right-hand side and run config.linear_solver.  CPU tensors are
    copied to the device and the solution copied back."""
    torch = _torch()
    s = ensure_operator()
    shape_in = x_i.shape
    host = not x_i.is_cuda
    dev = "cuda:%d" % s.cfg.device

    def d(a):
        if a is None:
            return None
        return a.to(dev, dtype=torch.float64, non_blocking=True).reshape(-1).contiguous()
    x = d(x_i) if host else _flat(x_i)
    fb = d(f)
    ub = [d(u) for u in u_bc]
    al = d(alpha_x_i) if alpha_x_i is not None else None
    _get_RAR_and_sfc_data_Um()
    x_rhs = torch.zeros(s.nonods, dtype=torch.float64, device=dev)
    _get_rhs(x_rhs, fb, ub, al)
    if config.linear_solver == "gmres-mg":
        _gmres_mg_solver(x, x_rhs, config.tol)
    elif config.linear_solver == "mg":
        _mg_solver(x, x_rhs, config.tol)
    elif config.linear_solver == "cg-mg":
        _cg_mg_solver(x, x_rhs, config.tol)
    else:
        raise ValueError("unknown linear_solver %r" % config.linear_solver)
    if host:
        x_i.reshape(-1).copy_(x.cpu())
        return x_i.view(shape_in)
    return x_i.view(shape_in)


def get_l2_error(x_num, x_ana):
    """(sum_b sum_n sum_g (phi_n (x_n - a_n))^2 |J| w)^(1/2) and the nodal
    max error, as the reference reports them (:2032-2056)."""
    torch = _torch()
    s = solver()
    m, el = s.mesh, s.el
    X = m.x_ref_in
    J = np.einsum("ing,bkn->bgik", el.nlx, X)
    det = np.abs(np.linalg.det(J))
    detwei = torch.tensor(det * el.weight[None, :], device=x_num.device)
    n = torch.tensor(el.n, device=x_num.device)
    dlt = (x_num.reshape(m.nele, -1) - x_ana.reshape(m.nele, -1).to(x_num.device))
    q = torch.einsum("ng,bn->bng", n, dlt) ** 2
    u_l2 = float(torch.sqrt(torch.einsum("bng,bg->", q, detwei)))
    u_linf = float(torch.abs(dlt).max())
    return u_l2, u_linf
