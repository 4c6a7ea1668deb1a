"""ctypes binding of libdgsip (include/dgsip.h).

The library is loaded from the package's _lib directory.  There is no
fallback: if the library is missing or fails to load, every entry point
raises, so a solve can never silently run anywhere but the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libdgsip.so")

DG_OK, DG_ERR_ARG, DG_ERR_CUDA, DG_ERR_MESH, DG_ERR_STATE, DG_ERR_NUMERIC, DG_ERR_NOCONV, DG_ERR_ALLOC = range(8)
DG_F64, DG_F32, DG_BF16 = 0, 1, 2


class DGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libdgsip error %d: %s" % (code, msg))
        self.code = code


class dg_mesh_desc(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("nloc", C.c_int32), ("nele", C.c_int64),
        ("x_ref_in", C.c_void_p), ("nbf", C.c_void_p), ("alnmt", C.c_void_p),
        ("glb_bcface_type", C.c_void_p), ("cg_nonods", C.c_int64), ("p1cg", C.c_void_p),
        ("sfc_order", C.c_void_p), ("ngi", C.c_int32), ("sngi", C.c_int32),
        ("n", C.c_void_p), ("nlx", C.c_void_p), ("weight", C.c_void_p), ("sn", C.c_void_p),
        ("snlx", C.c_void_p), ("sweight", C.c_void_p), ("gi_align", C.c_void_p),
        ("drst_duv", C.c_void_p), ("p1_to_p3", C.c_void_p),
    ]


class dg_config(C.Structure):
    _fields_ = [
        ("eta_e", C.c_double), ("mu_f", C.c_double), ("jac_wei", C.c_double),
        ("pre_smooth_its", C.c_int32), ("post_smooth_its", C.c_int32), ("device", C.c_int32),
    ]


_P = C.c_void_p
_I = C.c_int
_SIGNATURES = {
    "dg_create": (_I, [C.POINTER(dg_mesh_desc), C.POINTER(dg_config), C.POINTER(_P)]),
    "dg_destroy": (None, [_P]),
    "dg_last_error": (C.c_char_p, [_P]),
    "dg_info": (_I, [_P, _P, C.c_int32]),
    "dg_launch_count": (C.c_longlong, []),
    "dg_set_kappa": (_I, [_P, _P]),
    "dg_set_face_kappa": (_I, [_P, C.c_int32]),
    "dg_build_operator": (_I, [_P, _P]),
    "dg_get_bdiag": (_I, [_P, _P, _P, _P]),
    "dg_get_rar": (_I, [_P, _P, _P]),
    "dg_residual": (_I, [_P, _P, _P, _P, _P, C.c_int32, _P]),
    "dg_apply": (_I, [_P, _P, _P, _P]),
    "dg_rhs": (_I, [_P, _P, _P, _P, _P, _P]),
    "dg_precond": (_I, [_P, _P, _P, _P]),
    "dg_mg_vcycle": (_I, [_P, _P, _P, _P]),
    "dg_gmres": (_I, [_P, _P, _P, C.c_double, C.c_int32, C.c_int32, _P, _P, _P]),
    "dg_set_gmres_ortho": (_I, [_P, C.c_int32]),
    "dg_set_build_mode": (_I, [_P, C.c_int32]),
    "dg_solve_mixed": (_I, [_P, _P, _P, C.c_double, C.c_int32, C.c_int32, C.c_double, _P, _P, _P, _P]),
    "dg_apply_f32": (_I, [_P, _P, _P, _P]),
    "dg_solve_mixed_batched": (_I, [_P, _P, _P, C.c_int32, _P, C.c_int32, C.c_int32, C.c_double, _P, _P, _P]),
    "dg_smooth_pc": (_I, [_P, _P, _P, _P, _P]),
    "dg_smooth_scaled": (_I, [_P, _P, _P, _P, _P]),
    "dg_smooth_scaled_batched": (_I, [_P, _P, _P, _P, _P]),
    "dg_apply_batched": (_I, [_P, _P, _P, _P]),
    "dg_smooth_pc_batched": (_I, [_P, _P, _P, _P, _P]),
    "dg_set_batched_kernel": (_I, [_P, C.c_int32]),
    "dg_batched_tuning": (_I, [_P, _P, C.c_int32, _P]),
    "dg_precond_f32": (_I, [_P, _P, _P, _P]),
    "dg_set_mixed_options": (_I, [_P, C.c_int32, C.c_double, C.c_int32, C.c_int32]),
    "dg_set_launch_options": (_I, [_P, C.c_int32, C.c_int32]),
    "dg_set_vcycle_cluster": (_I, [_P, C.c_int32, C.POINTER(C.c_int32)]),
    "dg_residual_norm_noalloc": (_I, [_P, _P, _P, _P, _P, _P]),
    "dg_p1cg_sparsity": (_I, [C.c_int64, C.c_int32, _P, C.c_int64, _P, _P, C.c_int64, _P]),
    "dg_color2": (_I, [C.c_int64, _P, _P, _P, _P]),
    "dg_nlevel_sfc": (C.c_int32, [C.c_int64]),
    "dg_sfc_order": (_I, [C.c_int32, C.c_int64, _P, C.c_int32, _P]),
    "dg_sfc_levels": (_I, [C.c_int64, _P, _P, _P, _P, _P, _P, _P, _P, _P, C.c_int64, _P]),
    "dg_face_connectivity": (_I, [C.c_int32, C.c_int64, _P, _P, _P]),
    "dg_rap_contributions": (_I, [C.c_int32, C.c_int64, _P, _P, _P, _P, C.c_int64, _P, _P, C.c_int64, _P]),
    # serving: native request queue
    "dg_server_create": (_I, [C.c_int32, C.c_int32, C.POINTER(_P)]),
    "dg_server_destroy": (_I, [_P]),
    "dg_enqueue": (_I, [_P, _P, _P, _P, C.c_double, C.c_int32, C.c_int32, C.c_int32, C.c_double, _P,
                        C.POINTER(C.c_int64)]),
    "dg_poll": (_I, [_P, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                     C.POINTER(C.c_double), _P]),
    "dg_wait": (_I, [_P, C.c_int64, C.c_double, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                     C.POINTER(C.c_double), _P]),
}
DG_REQ_QUEUED, DG_REQ_RUNNING, DG_REQ_DONE = 0, 1, 2
# entry points added by later translation units (bound when present)
_OPTIONAL = {}

_lib = None
_lock = threading.Lock()


def lib():
    """Load libdgsip (raises if it is missing: there is no fallback path)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError("libdgsip.so is not built (%s); run dg_nn_public_gb300.build.build()"
                                   % LIB_PATH)
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            for name, (res, args) in _OPTIONAL.items():
                if hasattr(L, name):
                    fn = getattr(L, name)
                    fn.restype = res
                    fn.argtypes = args
            _lib = L
    return _lib


def register_optional(name, restype, argtypes):
    _OPTIONAL[name] = (restype, argtypes)
    if _lib is not None and hasattr(_lib, name):
        fn = getattr(_lib, name)
        fn.restype = restype
        fn.argtypes = argtypes


def check(rc, ctx=None):
    if rc != DG_OK:
        msg = lib().dg_last_error(ctx)
        raise DGError(rc, msg.decode() if msg else "")


def launch_count() -> int:
    return int(lib().dg_launch_count())


def ptr(a):
    """Address of a numpy array or a torch tensor (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


# ---- host-only integer layer ----------------------------------------------

def p1cg_sparsity(p1cg: np.ndarray, cg_nonods: int):
    p1 = np.ascontiguousarray(p1cg, dtype=np.int64)
    nele, nc = p1.shape
    fina = np.zeros(cg_nonods + 1, dtype=np.int64)
    cap = nele * nc * nc
    cola = np.zeros(max(cap, 1), dtype=np.int64)
    ncola = np.zeros(1, dtype=np.int64)
    check(lib().dg_p1cg_sparsity(nele, nc, ptr(p1), cg_nonods, ptr(fina), ptr(cola), cap, ptr(ncola)))
    return fina, cola[:int(ncola[0])].copy()


def rap_contributions(ndim: int, p1cg: np.ndarray, nbe: np.ndarray, fina: np.ndarray, cola: np.ndarray):
    """(ptr, entries) of the direct Galerkin P1CG assembly: entries[ptr[k]:
    ptr[k+1]] are the (block, a, c) triples of nonzero k (see
    dg_rap_contributions in include/dgsip.h)."""
    p1 = np.ascontiguousarray(p1cg, dtype=np.int64)
    nb = np.ascontiguousarray(nbe, dtype=np.int64)
    fina = np.ascontiguousarray(fina, dtype=np.int64)
    cola = np.ascontiguousarray(cola, dtype=np.int64)
    nele, nc = p1.shape
    n = fina.size - 1
    cap = nele * (ndim + 2) * nc * nc
    ptr_ = np.zeros(int(fina[-1]) + 1, dtype=np.int64)
    ent = np.zeros((max(cap, 1), 3), dtype=np.int64)
    cnt = np.zeros(1, dtype=np.int64)
    check(lib().dg_rap_contributions(ndim, nele, ptr(p1), ptr(nb), ptr(fina), ptr(cola), n, ptr(ptr_), ptr(ent),
                                     cap, ptr(cnt)))
    return ptr_, ent[:int(cnt[0])].copy()


def color2(fina, cola):
    fina = np.ascontiguousarray(fina, dtype=np.int64)
    cola = np.ascontiguousarray(cola, dtype=np.int64)
    n = fina.size - 1
    whichc = np.zeros(max(n, 1), dtype=np.int64)
    nc = np.zeros(1, dtype=np.int32)
    check(lib().dg_color2(n, ptr(fina), ptr(cola), ptr(whichc), ptr(nc)))
    return whichc[:n], int(nc[0])


def sfc_order(coords=None, order=None, bits: int = 0, ndim: int = None):
    """dg_sfc_order: with coords, the Hilbert numbering of the points ((n, 1)
    int64, 1-based); with order only, check a given numbering (e.g. the
    reference's cached curve) and return it as (n, 1) int64."""
    if coords is not None:
        X = np.ascontiguousarray(coords, dtype=np.float64)
        n, nd = X.shape
        out = np.zeros(n, dtype=np.int64)
        check(lib().dg_sfc_order(nd, n, ptr(X), bits, ptr(out)))
        return out.reshape(n, 1)
    o = np.ascontiguousarray(np.asarray(order).reshape(-1), dtype=np.int64)
    check(lib().dg_sfc_order(ndim or 3, o.size, None, 0, ptr(o)))
    return o.reshape(-1, 1)


def nlevel_sfc(n: int) -> int:
    return int(lib().dg_nlevel_sfc(n))


def sfc_levels(fina, cola, a, sfc_order):
    fina = np.ascontiguousarray(fina, dtype=np.int64)
    cola = np.ascontiguousarray(cola, dtype=np.int64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    so = np.ascontiguousarray(np.asarray(sfc_order).reshape(-1), dtype=np.int64)
    n = fina.size - 1
    nl = nlevel_sfc(n)
    total = 0
    s = n
    for _ in range(nl):
        total += s
        s = (s - 1) // 2 + 1
    cap = cola.size * nl + 16
    nlev = np.zeros(1, dtype=np.int32)
    start = np.zeros(nl + 1, dtype=np.int64)
    rowp = np.zeros(total + 1, dtype=np.int64)
    col = np.zeros(cap, dtype=np.int64)
    val = np.zeros(cap, dtype=np.float64)
    nnz = np.zeros(1, dtype=np.int64)
    check(lib().dg_sfc_levels(n, ptr(fina), ptr(cola), ptr(a), ptr(so), ptr(nlev), ptr(start), ptr(rowp),
                              ptr(col), ptr(val), cap, ptr(nnz)))
    k = int(nnz[0])
    return int(nlev[0]), start, rowp, col[:k].copy(), val[:k].copy()


def face_connectivity(ndim: int, corners: np.ndarray):
    cr = np.ascontiguousarray(corners, dtype=np.int64)
    nele = cr.shape[0]
    nbf = np.zeros(nele * (ndim + 1), dtype=np.int64)
    aln = np.zeros(nele * (ndim + 1), dtype=np.int64)
    check(lib().dg_face_connectivity(ndim, nele, ptr(cr), ptr(nbf), ptr(aln)))
    return nbf, aln
