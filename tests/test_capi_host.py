"""The C ABI without a GPU: the library builds and loads, exports every entry
point declared in include/dgsip.h, and its host-only integer layer (P1CG
sparsity, distance-2 colouring, SFC levels, face connectivity) reproduces
the oracle bit for bit."""
import ctypes
import os
import re

import numpy as np
import pytest

from dg_nn_public_gb300 import _capi, build, element, mesh, sfc
from oracle import fortran_restated as fr
from oracle.dg_oracle import OracleDG
from golden_util import load, rebuild

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "dgsip.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _capi.lib()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dg_[a-z0-9_]+)\s*\(", text)))


def test_all_declared_symbols_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    raw = ctypes.CDLL(_capi.LIB_PATH)
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing


def test_error_path_without_context(lib):
    rc = lib.dg_p1cg_sparsity(-1, 4, None, 0, None, None, 0, None)
    assert rc == _capi.DG_ERR_ARG
    assert b"bad arguments" in lib.dg_last_error(None)


@pytest.mark.parametrize("kind,n", [("tet", 3), ("tri", 6), ("tet", 6)])
def test_integer_layer_matches_oracle(lib, kind, n):
    m = mesh.build_mesh(kind, n, seed=1)
    O = OracleDG(m, element.p3_element(m.ndim), element.drst_duv(m.ndim))
    pc = O.p1cg()
    fina, cola = _capi.p1cg_sparsity(m.p1cg, m.cg_nonods)
    assert np.array_equal(fina, pc["fina"]) and np.array_equal(cola, pc["cola"])
    whichc, ncolor = _capi.color2(fina, cola)
    assert np.array_equal(whichc, pc["whichc"]) and ncolor == pc["ncolor"]
    order = sfc.hilbert_sfc_order(m.cg_coords)
    vals = np.random.default_rng(0).standard_normal(cola.size)
    nl, start, rowp, col, val = _capi.sfc_levels(fina, cola, vals, order)
    ref = fr.best_sfc_mapping_to_sfc_matrix_unstructured(
        vals, np.zeros(m.cg_nonods), np.zeros(m.cg_nonods), fina + 1, cola + 1, order.reshape(-1),
        5 * m.cg_nonods, 10 * cola.size, fr.calculate_nlevel_sfc(m.cg_nonods) + 1, cola.size, m.cg_nonods)
    a_all, fina_all, cola_all, ncola_all, _, _, fin, nall, nlevel = ref
    assert nl == nlevel == _capi.nlevel_sfc(m.cg_nonods)
    assert np.array_equal(start, fin[:nl + 1] - 1)
    assert np.array_equal(rowp, fina_all[:nall + 1] - 1)
    # Fortran stores stacked global columns, the C ABI level-local ones
    glob = np.concatenate([col[rowp[start[l]]:rowp[start[l + 1]]] + start[l] for l in range(nl)])
    assert np.array_equal(glob, cola_all[:ncola_all] - 1)
    assert np.array_equal(val, a_all[:ncola_all])          # same summation order: bit-identical
    nbf, aln = _capi.face_connectivity(m.ndim, m.cg_ndglno[:, :m.ndim + 1])
    assert np.array_equal(nbf, m.nbf) and np.array_equal(aln, m.alnmt)


def test_face_connectivity_against_reference_golden(lib):
    d, meta = load("tet3_v22")
    nbf, aln = _capi.face_connectivity(3, d["cg_ndglno"][:, :4])
    assert np.array_equal(nbf, d["nbf"]) and np.array_equal(aln, d["alnmt"])


def test_sfc_levels_rejects_bad_ordering(lib):
    m = mesh.build_mesh("tri", 3)
    fina, cola = _capi.p1cg_sparsity(m.p1cg, m.cg_nonods)
    bad = np.ones(m.cg_nonods, dtype=np.int64)
    with pytest.raises(_capi.DGError):
        _capi.sfc_levels(fina, cola, np.ones(cola.size), bad)


@pytest.mark.parametrize("kind,n", [("tet", 2), ("tri", 4)])
def test_rap_contributions_give_the_probe_operator(lib, kind, n):
    """The direct Galerkin assembly from per-block 4x4 products, driven by
    the C-ABI contribution lists, reproduces the colour-probe P1CG operator
    of the CPU restatement (dense blocks of a small jittered mesh with
    log-normal kappa); every P1CG nonzero gets at least one contribution."""
    from dg_nn_public_gb300 import _capi, element, mesh
    from oracle.dg_oracle import OracleDG
    m = mesh.build_mesh(kind, n, seed=3)
    el = element.p3_element(m.ndim)
    kap = np.exp(0.6 * np.random.default_rng(2).standard_normal(m.nele))
    O = OracleDG(m, el, element.drst_duv(m.ndim), eta_e=90.0, kappa=kap)
    pc = O.p1cg()
    probe = O.rar(pc)
    F, N, B = m.ndim + 1, m.nloc, m.nele
    bct = np.asarray(m.glb_bcface_type).reshape(B, F)
    nbe = np.where(bct < 0, np.asarray(m.nbf).reshape(B, F) // F, -1)
    ptr, ent = _capi.rap_contributions(m.ndim, np.asarray(m.p1cg), nbe, pc["fina"], pc["cola"])
    assert ptr.size == pc["cola"].size + 1 and np.all(np.diff(ptr) >= 1)
    ndg = B * N
    eye = np.eye(ndg)
    A = np.stack([O.apply_Ax(eye[i]).ravel() for i in range(ndg)], axis=1)
    P3 = np.asarray(el.p1_to_p3)                                   # (N, D+1)
    w = pc["wdg"]                                                  # (B, D+1)
    direct = np.zeros(pc["cola"].size)
    for k in range(direct.size):
        for blk, a, c in ent[ptr[k]:ptr[k + 1]]:
            e, sl = divmod(int(blk), F + 1)
            nb = e if sl == 0 else int(nbe[e, sl - 1])
            G = P3.T @ A[e * N:(e + 1) * N, nb * N:(nb + 1) * N] @ P3
            direct[k] += w[e, a] * w[nb, c] * G[a, c]
    assert np.abs(direct - probe).max() <= 1e-12 * np.abs(probe).max()


def test_rap_contributions_error_paths(lib):
    from dg_nn_public_gb300 import _capi
    p1 = np.array([[0, 1, 2, 3]], dtype=np.int64)
    fina, cola = _capi.p1cg_sparsity(p1, 4)
    nbe = -np.ones((1, 4), dtype=np.int64)
    ptr, ent = _capi.rap_contributions(3, p1, nbe, fina, cola)
    # one element, own block only: every corner pair once, in (a, c) order
    assert ent.shape == (16, 3) and np.array_equal(np.diff(ptr), np.ones(16, dtype=np.int64))
    assert sorted(map(tuple, ent.tolist())) == [(0, a, c) for a in range(4) for c in range(4)]
    with pytest.raises(_capi.DGError):
        _capi.rap_contributions(3, p1, np.array([[5, -1, -1, -1]]), fina, cola)   # neighbour out of range
    with pytest.raises(_capi.DGError):
        _capi.rap_contributions(4, p1, nbe, fina, cola)                             # bad dimension


@pytest.mark.parametrize("kind,n,seed", [("tet", 3, 0), ("tet", 20, 0), ("tri", 32, 0), ("tri", 5, 9)])
def test_sfc_order_native_equals_numpy(lib, kind, n, seed):
    """dg_sfc_order (ordering out) gives exactly the numpy Hilbert numbering
    the golden cases were generated with, in the reference's cache format."""
    from dg_nn_public_gb300 import mesh, sfc
    m = mesh.build_mesh(kind, n, seed=seed)
    a = sfc.hilbert_sfc_order(m.cg_coords)
    assert a.shape == (m.cg_nonods, 1) and a.dtype == np.int64
    assert np.array_equal(a, sfc.hilbert_sfc_order_numpy(m.cg_coords))
    assert np.array_equal(np.sort(a.ravel()), np.arange(1, m.cg_nonods + 1))


def test_sfc_order_in_validates_reference_curve(lib):
    """Ordering in: a curve read from the reference's cache (golden 'sfc') is
    accepted as is; a non-permutation is rejected with DG_ERR_ARG."""
    from dg_nn_public_gb300 import _capi
    d, _ = load("tet3_v22")
    got = _capi.sfc_order(order=d["sfc"])
    assert np.array_equal(got, d["sfc"])
    bad = d["sfc"].copy()
    bad[0] = bad[1]
    with pytest.raises(_capi.DGError) as e:
        _capi.sfc_order(order=bad)
    assert e.value.code == _capi.DG_ERR_ARG


def test_server_argument_checks(lib):
    """The native request queue rejects bad arguments before it touches a
    device: worker counts out of range, a missing server or context, an
    unknown mode, and polls of unknown servers; destroying NULL is a no-op."""
    h = ctypes.c_void_p()
    assert lib.dg_server_create(0, 0, ctypes.byref(h)) == _capi.DG_ERR_ARG
    assert lib.dg_server_create(0, 65, ctypes.byref(h)) == _capi.DG_ERR_ARG
    assert b"nworkers" in lib.dg_last_error(None)
    rid = ctypes.c_int64(0)
    rc = lib.dg_enqueue(None, None, None, None, 1e-10, 0, 30, 100, 1e-3, None, ctypes.byref(rid))
    assert rc == _capi.DG_ERR_ARG
    st = ctypes.c_int32(0)
    assert lib.dg_poll(None, 1, ctypes.byref(st), None, None, None, None) == _capi.DG_ERR_ARG
    assert lib.dg_wait(None, 1, 0.0, ctypes.byref(st), None, None, None, None) == _capi.DG_ERR_ARG
    assert lib.dg_server_destroy(None) == _capi.DG_OK


def test_native_queue_needs_a_device():
    """Without a CUDA device the queue reports DG_ERR_CUDA at creation
    instead of starting workers that could not run anything."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from dg_nn_public_gb300 import serving
    with pytest.raises(_capi.DGError) as ei:
        serving.NativeQueue(nworkers=1)
    assert ei.value.code == _capi.DG_ERR_CUDA
