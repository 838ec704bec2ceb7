"""Caller-side mesh preparation and the C-ABI library (CPU only): the arrays
the Fortran host would pass are bit-identical to the oracle's, and the shared
library exports every entry point include/mfbem.h declares."""
import ctypes
import os
import re

import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, _abi
from multifebe_gb300.bem import BemRegion

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _prep(d):
    L = _abi.load()
    X = np.ascontiguousarray(d.nodes)
    conn = np.ascontiguousarray(d.conn, dtype=np.int32)
    ct = np.ascontiguousarray(d.ctype, dtype=np.int32)
    cv = np.ascontiguousarray(d.cvalue)
    gl = np.array([2, 3, 4, 5, 6, 7, 8, 9], dtype=np.int32)
    pp = L.mfbem_prep_create(d.n_nodes, X.ctypes.data_as(_abi._dp), d.n_elements, conn.ctypes.data_as(_abi._ip),
                             ct.ctypes.data_as(_abi._ip), cv.view(np.float64).ctypes.data_as(_abi._dp), 1e-6, 16, 8,
                             gl.ctypes.data_as(_abi._ip), 1e-6)
    return L, pp, (X, conn, ct, cv, gl)


@pytest.mark.parametrize("deck", [M.cube_clamped_top_traction(4), M.cube_confined_kat(2), M.surface_patch(10.0, 8, 1.0),
                                  M.slab(4, 1)], ids=lambda d: d.name)
def test_prep_matches_oracle_bit_exact(oracle, deck):
    L, pp, keep = _prep(deck)
    try:
        desc = L.mfbem_prep_desc(pp).contents
        ne = deck.n_elements
        cl = np.ctypeslib.as_array(desc.csize, shape=(ne,))
        gf = np.ctypeslib.as_array(desc.n_phi, shape=(ne,))
        ball = np.ctypeslib.as_array(desc.bball, shape=(4 * ne,)).reshape(ne, 4)
        P = oracle.Problem(deck)
        ocl, ogf, oball = P.element_data()
        assert np.array_equal(cl, ocl) and np.array_equal(gf, ogf) and np.array_equal(ball, oball)
        dof = np.zeros(3 * deck.n_nodes, dtype=np.int32)
        order = np.zeros(deck.n_nodes, dtype=np.int32)
        L.mfbem_prep_dof(pp, dof.ctypes.data_as(_abi._ip), order.ctypes.data_as(_abi._ip))
        odof, oorder = P.dof_map()
        assert np.array_equal(dof.reshape(-1, 3), odof) and np.array_equal(order, oorder)
        # 1-based rows / columns as node%row, node%col
        row = np.ctypeslib.as_array(desc.row, shape=(3 * deck.n_nodes,)).reshape(-1, 3)
        assert np.array_equal(row - 1, odof)
        # MCA collocation points = oracle's collocation points of kind 1
        x, info = P.colloc()
        xm = np.ctypeslib.as_array(desc.x_i_sbie_mca, shape=(24 * ne,)).reshape(ne, 8, 3)
        for i in np.nonzero(info[:, 1] == 1)[0]:
            assert np.array_equal(xm[info[i, 2], info[i, 3]], x[i])
    finally:
        L.mfbem_prep_free(pp)


@pytest.mark.parametrize("form", ["hbie", "dual_bm", "dual_bm_mixed"])
def test_prep_hbie_points_match_oracle(oracle, form):
    """HBIE points and their unit normals (src/build_data_at_collocation_points.f90:
    148-160,368-376), the node members of the dual descriptor and the MCA
    points ('dual_bm_mixed' moves them by 0.22540333)."""
    deck = M.cube_confined_kat(2)
    L, pp, keep = _prep(deck)
    try:
        nn, ne = deck.n_nodes, deck.n_elements
        code = {"hbie": 1, "dual_bm": 2, "dual_bm_mixed": 3}[form]
        f = np.full(nn, code, dtype=np.int32)
        f[::5] = 0  # a few nodes keep the SBIE
        a = np.linspace(0.5, 1.5, nn)
        dl = np.full(nn, 0.3)
        assert L.mfbem_prep_set_formulation(pp, f.ctypes.data_as(_abi._ip), a.ctypes.data_as(_abi._dp),
                                            dl.ctypes.data_as(_abi._dp)) == 0
        dd = L.mfbem_prep_dual(pp).contents
        hb = np.ctypeslib.as_array(dd.hbie, shape=(nn,))
        du = np.ctypeslib.as_array(dd.dual, shape=(nn,))
        co = np.ctypeslib.as_array(dd.dual_is_common, shape=(nn,))
        assert np.array_equal(hb, f != 0) and np.array_equal(du, f >= 2) and np.array_equal(co, f == 2)
        xh = np.ctypeslib.as_array(dd.x_i_hbie, shape=(24 * ne,)).reshape(ne, 8, 3)
        nh = np.ctypeslib.as_array(dd.n_i_hbie, shape=(24 * ne,)).reshape(ne, 8, 3)
        P = oracle.Problem(deck)
        P.set_formulation(f, alpha=a, delta=dl)
        x, info = P.colloc()
        nrm = P.colloc_normals()
        sel = np.nonzero(info[:, 1] >= 2)[0]
        assert len(sel) == np.isin(deck.conn, np.nonzero(f)[0]).sum()
        for i in sel:
            assert np.abs(xh[info[i, 2], info[i, 3]] - x[i]).max() <= 1e-15
            assert np.abs(nh[info[i, 2], info[i, 3]] - nrm[i]).max() <= 1e-15
        desc = L.mfbem_prep_desc(pp).contents
        xm = np.ctypeslib.as_array(desc.x_i_sbie_mca, shape=(24 * ne,)).reshape(ne, 8, 3)
        mca = np.nonzero(info[:, 1] == 1)[0]
        assert len(mca) > 0
        for i in mca:
            assert np.array_equal(xm[info[i, 2], info[i, 3]], x[i])
    finally:
        L.mfbem_prep_free(pp)


@pytest.mark.parametrize("mk", [lambda: M.penny_crack(1.0, 2, 2, 1.0), lambda: M.penny_crack_in_box(1.0, 2, 1, 2.0, 2)],
                         ids=["penny", "penny_in_box"])
def test_prep_crack_matches_oracle(oracle, mk):
    """Crack-like boundaries: the six-row DOF layout of the crack nodes
    (src/build_auxiliary_variables_mechanics_static.f90:146-207), their
    (hbie, dual, dual_is_common) = (1, 2, 1) and points, as the oracle's."""
    deck, (ce, ct2, cv2) = mk()
    L, pp, keep = _prep(deck)
    try:
        nn, ne = deck.n_nodes, deck.n_elements
        cei = np.ascontiguousarray(ce, dtype=np.int32)
        ct2 = np.ascontiguousarray(ct2, dtype=np.int32)
        cv2 = np.ascontiguousarray(cv2, dtype=np.complex128)
        assert L.mfbem_prep_set_crack(pp, cei.ctypes.data_as(_abi._ip), ct2.ctypes.data_as(_abi._ip),
                                      cv2.view(np.float64).ctypes.data_as(_abi._dp)) == 0
        P = oracle.Problem(deck)
        P.set_crack(ce, ct2, cv2)
        desc = L.mfbem_prep_desc(pp).contents
        assert desc.n_dof == P.n == 3 * nn + 3 * len(np.unique(deck.conn[ce]))
        dof = np.zeros(3 * nn, dtype=np.int32)
        order = np.zeros(nn, dtype=np.int32)
        dof2 = np.zeros(3 * nn, dtype=np.int32)
        L.mfbem_prep_dof(pp, dof.ctypes.data_as(_abi._ip), order.ctypes.data_as(_abi._ip))
        L.mfbem_prep_dof2(pp, dof2.ctypes.data_as(_abi._ip))
        odof, oorder = P.dof_map()
        assert np.array_equal(dof.reshape(-1, 3), odof) and np.array_equal(order, oorder)
        assert np.array_equal(dof2.reshape(-1, 3), P.dof2_map())
        row = np.ctypeslib.as_array(desc.row, shape=(3 * nn,)).reshape(-1, 3)
        assert np.array_equal(row - 1, odof)
        dd = L.mfbem_prep_dual(pp).contents
        cn = np.zeros(nn, bool)
        cn[np.unique(deck.conn[ce])] = True
        hb = np.ctypeslib.as_array(dd.hbie, shape=(nn,))
        du = np.ctypeslib.as_array(dd.dual, shape=(nn,))
        co = np.ctypeslib.as_array(dd.dual_is_common, shape=(nn,))
        assert np.array_equal(hb, cn) and np.array_equal(du, 2 * cn) and np.array_equal(co, cn)
        assert np.array_equal(np.ctypeslib.as_array(dd.crack_el, shape=(ne,)), cei)
        x, info = P.colloc()
        xh = np.ctypeslib.as_array(dd.x_i_hbie, shape=(24 * ne,)).reshape(ne, 8, 3)
        sel = np.nonzero(info[:, 1] == 4)[0]
        assert len(sel) == 8 * ce.sum()
        for i in sel:
            assert np.abs(xh[info[i, 2], info[i, 3]] - x[i]).max() <= 1e-15
        # a crack node in an ordinary element is refused
        bad = cei.copy()
        bad[0] = 0
        assert L.mfbem_prep_set_crack(pp, bad.ctypes.data_as(_abi._ip), ct2.ctypes.data_as(_abi._ip),
                                      cv2.view(np.float64).ctypes.data_as(_abi._dp)) == -1
    finally:
        L.mfbem_prep_free(pp)


def test_library_exports_every_declared_symbol():
    L = _abi.load()
    hdr = open(os.path.join(ROOT, "include", "mfbem.h")).read()
    declared = set(re.findall(r"\b(mfbem_[a-z_]+)\s*\(", hdr))
    assert declared == set(_abi.ABI_SYMBOLS)
    for s in sorted(declared) + _abi.PREP_SYMBOLS:
        assert hasattr(L, s), s
    assert b"sm_103a" in L.mfbem_version()


def test_no_device_is_an_error_status_not_a_crash():
    from conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present")
    with pytest.raises(_abi.MfbemError) as e:
        BemRegion(M.cube_clamped_top_traction(2))
    assert e.value.code == _abi.MFBEM_ECUDA


@pytest.mark.parametrize("entry", ["mfbem_solve_c", "mfbem_solve_r", "mfbem_solve_c_static"])
def test_reused_factors_with_foreign_pivots_are_refused_before_any_device_work(entry):
    """factorize = 0 takes the caller's ipiv: values outside getrf's range
    (ipiv(j) in [j, n], 1-based) are refused on the host, so no kernel ever
    indexes the vectors with them (checked without a GPU: the call returns
    before the first CUDA call)."""
    L = _abi.load()
    n = 8
    cplx = entry != "mfbem_solve_r"
    A = np.asfortranarray(np.eye(n, dtype=np.complex128 if cplx else np.float64))
    b = np.ones((n, 1), dtype=A.dtype, order="F")
    for bad in ([1, 2, 3, 4, 5, 6, 7, 9], [0, 2, 3, 4, 5, 6, 7, 8], [2, 1, 3, 4, 5, 6, 7, 8], [1, 2, 3, 4, 5, 6, 7, -3]):
        ip = np.array(bad, dtype=np.int32)
        if entry == "mfbem_solve_c_static":
            rc = L.mfbem_solve_c_static(n, A.ctypes.data_as(_abi._dp), ip.ctypes.data_as(_abi._ip), 1,
                                        b.ctypes.data_as(_abi._dp), 0)
        else:
            rc = getattr(L, entry)(n, A.ctypes.data_as(_abi._dp), ip.ctypes.data_as(_abi._ip), 1, None, None, None,
                                   None, 1, b.ctypes.data_as(_abi._dp), 0, 0, 0, 0)
        assert rc == _abi.MFBEM_EARG, bad
        assert b"is not a pivot of getrf" in L.mfbem_last_error()
