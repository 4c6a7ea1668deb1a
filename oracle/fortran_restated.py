"""CPU restatement of the reference's Fortran helpers (test infrastructure).

This module is part of the oracle: it is imported only by the tests, by the
golden-vector generator and by the shims that let the reference's own Python
run here.  The reference builds these routines with f2py from Fortran
(z02-implicit/z06-DGtoCG/compile_f90.sh:2-4); no Fortran compiler exists in
this image, so they are restated in numpy, following the Fortran loop by
loop where the result depends on the order of operations:

* ``getfinele``  <- z00-fortran-src/get_neighbouring.f90:1-130
* ``getfin_p1cg`` <- z00-fortran-src/get_neighbouring.f90:133-157
* ``calculate_nlevel_sfc`` <- z00-fortran-src/compact_fcode.f90:229-250
* ``best_sfc_mapping_to_sfc_matrix_unstructured``
  <- z00-fortran-src/compact_fcode.f90:7-225 (the coarse values are summed in
  the Fortran traversal order, so they are bit-identical to a compiled run)

Return values follow the f2py conventions (1-based Fortran indices,
fixed-size output arrays padded with zeros).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def getfinele(totele, nloc, snloc, nonods, ndglno, mx_nface_p1, mxnele):
    """Element adjacency: elements sharing >= snloc nodes (self included).

    get_neighbouring.f90:1-130.  Returns (ncolele, finele, colele, midele),
    1-based, rows sorted ascending (the Fortran bubble sort, :101-110).
    """
    ndg = np.asarray(ndglno, dtype=np.int64).reshape(totele, nloc) - 1
    rows = np.repeat(np.arange(totele), nloc)
    inc = sp.csr_matrix((np.ones(totele * nloc), (rows, ndg.ravel())), shape=(totele, nonods))
    inc.data[:] = 1.0
    inc.sum_duplicates()
    inc.data[:] = 1.0
    share = (inc @ inc.T).tocsr()
    share.sort_indices()
    keep = share.data >= snloc
    rr = np.repeat(np.arange(totele), np.diff(share.indptr))[keep]
    cc = share.indices[keep]
    counts = np.bincount(rr, minlength=totele)
    finele = np.zeros(totele + 1, dtype=np.int64)
    finele[1:] = np.cumsum(counts)
    finele += 1
    colele = np.zeros(mxnele, dtype=np.int64)
    colele[:cc.size] = cc + 1
    midele = np.zeros(totele, dtype=np.int64)
    for e in range(totele):
        seg = colele[finele[e] - 1:finele[e + 1] - 1]
        hit = np.nonzero(seg == e + 1)[0]
        if hit.size:
            midele[e] = finele[e] + hit[-1]
    return int(cc.size), finele, colele, midele


def getfin_p1cg(cg_noglbn, nele, nloc, p1dg_nonods):
    """All (i, j) P1CG node pairs of every element (get_neighbouring.f90:133-157)."""
    g = np.asarray(cg_noglbn, dtype=np.int64).reshape(nele, nloc)
    i = np.repeat(g, nloc, axis=1).ravel()
    j = np.tile(g, (1, nloc)).ravel()
    idx = np.stack([i, j], axis=0)
    return idx, int(idx.shape[1])


def calculate_nlevel_sfc(nonods):
    """Number of 1-D SFC grid levels (compact_fcode.f90:229-250)."""
    if nonods == 1:
        return 1
    course = nonods
    nlevel = 1
    for ilevel in range(2, 201):
        fine = course
        course = (fine - 1) // 2 + 1
        nlevel = ilevel
        if course == 1:
            break
    return nlevel


def _coarsen_vec(fine):
    """map_sfc_fine_grid_2_course_grid_vec (compact_fcode.f90:253-282)."""
    nc = (fine.size - 1) // 2 + 1
    out = np.zeros(nc)
    out[: (fine.size + 1) // 2] += fine[0::2]
    out[: fine.size // 2] += fine[1::2]
    return out


def best_sfc_mapping_to_sfc_matrix_unstructured(a, b, ml, fina, cola, sfc_node_ordering,
                                                max_nonods_sfc_all_grids, max_ncola_sfc_all_un,
                                                max_nlevel, ncola, nonods):
    """All SFC grid levels of a CSR matrix (compact_fcode.f90:7-225).

    Level l (1-based) maps SFC position s to coarse node (s-1) // 2^(l-1);
    each coarse row lists its columns in first-appearance order while the
    fine rows are walked in SFC order and each fine row in CSR order, and
    the values are summed in that same order.
    """
    a = np.asarray(a, dtype=np.float64)
    fina0 = np.asarray(fina, dtype=np.int64) - 1
    cola0 = np.asarray(cola, dtype=np.int64) - 1
    sfc = np.asarray(sfc_node_ordering, dtype=np.int64) - 1      # node -> SFC position
    nlevel = calculate_nlevel_sfc(nonods)
    b_sfc = np.zeros(max_nonods_sfc_all_grids)
    ml_sfc = np.zeros(max_nonods_sfc_all_grids)
    bl = np.zeros(nonods)
    mll = np.zeros(nonods)
    bl[sfc] = np.asarray(b, dtype=np.float64)
    mll[sfc] = np.asarray(ml, dtype=np.float64)
    fin = np.zeros(max_nlevel + 1, dtype=np.int64)
    fin[0] = 1
    fin[1] = 1 + nonods
    sizes = [nonods]
    b_sfc[0:nonods] = bl
    ml_sfc[0:nonods] = mll
    for il in range(2, nlevel + 1):
        fine = sizes[-1]
        if fine <= 1:
            raise RuntimeError("stop 13331")
        course = (fine - 1) // 2 + 1
        bl = _coarsen_vec(bl)
        mll = _coarsen_vec(mll)
        b_sfc[fin[il - 1] - 1:fin[il - 1] - 1 + course] = bl
        ml_sfc[fin[il - 1] - 1:fin[il - 1] - 1 + course] = mll
        fin[il] = fin[il - 1] + course
        sizes.append(course)
    nonods_all = int(fin[nlevel] - 1)
    if max_nonods_sfc_all_grids < nonods_all:
        raise RuntimeError("stop 2822")
    inv = np.empty(nonods, dtype=np.int64)
    inv[sfc] = np.arange(nonods)                                  # SFC position -> node
    # traversal order of the fine entries: SFC rows, CSR order within a row
    rowlen = fina0[1:] - fina0[:-1]
    rows_sfc = np.repeat(np.arange(nonods), rowlen[inv])
    ent = np.concatenate([np.arange(fina0[n], fina0[n + 1]) for n in inv]) if nonods else np.zeros(0, np.int64)
    jcol_sfc = sfc[cola0[ent]]
    vals = a[ent]
    fina_all = np.zeros(max_nonods_sfc_all_grids + 1, dtype=np.int64)
    cola_all = np.zeros(max_ncola_sfc_all_un, dtype=np.int64)
    a_all = np.zeros(max_ncola_sfc_all_un)
    count_all = 0
    for il in range(1, nlevel + 1):
        shift = il - 1
        disp = int(fin[il - 1])                                   # 1-based start of the level
        nc = sizes[il - 1]
        ic = rows_sfc >> shift
        jc = jcol_sfc >> shift
        key = ic * nc + jc
        # first appearance of each (ic, jc) in traversal order
        uniq, first, inverse = np.unique(key, return_index=True, return_inverse=True)
        order = np.lexsort((first, uniq // nc))                   # by row, then first appearance
        pos = np.empty(uniq.size, dtype=np.int64)
        pos[order] = np.arange(uniq.size)
        acc = np.zeros(uniq.size)
        np.add.at(acc, pos[inverse], vals)                        # sequential, in traversal order
        row_of = (uniq // nc)[order]
        col_of = (uniq % nc)[order]
        cnt = np.bincount(row_of, minlength=nc)
        start = count_all
        cola_all[start:start + uniq.size] = disp + col_of
        a_all[start:start + uniq.size] = acc
        ptr = start + np.concatenate([[0], np.cumsum(cnt)])
        fina_all[disp - 1:disp - 1 + nc + 1] = ptr + 1
        count_all += uniq.size
    ncola_all = int(fina_all[nonods_all] - 1)
    if max_ncola_sfc_all_un < ncola_all:
        raise RuntimeError("stop 2825")
    return a_all, fina_all, cola_all, ncola_all, b_sfc, ml_sfc, fin, nonods_all, nlevel
