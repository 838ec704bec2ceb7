"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
arm load this module. The oracle restates MultiFEBE's collocation BEM path
(see orc.h) and solves the assembled systems with LAPACK getrf/getrs through
scipy (OpenBLAS), as src/solve_lse_r.f90:137,189 and src/solve_lse_c.f90:124,176 do.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def build(force=False):
    if force or not os.path.exists(LIB) or any(
            os.path.getmtime(os.path.join(HERE, f)) > os.path.getmtime(LIB)
            for f in os.listdir(HERE) if f.endswith((".cpp", ".h"))):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_problem_new.restype = ctypes.c_void_p
        L.orc_problem_new.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _ip, _dp, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_int, _ip, ctypes.c_double]
        L.orc_problem_free.argtypes = [ctypes.c_void_p]
        L.orc_n_dof.argtypes = [ctypes.c_void_p]
        L.orc_n_colloc.argtypes = [ctypes.c_void_p]
        L.orc_dof_map.argtypes = [ctypes.c_void_p, _ip, _ip]
        L.orc_element_data.argtypes = [ctypes.c_void_p, _dp, _ip, _dp]
        L.orc_colloc.argtypes = [ctypes.c_void_p, _dp, _ip]
        L.orc_node_geometry.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_char_p]
        L.orc_assemble_staela.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _dp, _dp, ctypes.c_int,
                                          _lp]
        L.orc_assemble_harela_nu.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 8 + [_dp, _dp, ctypes.c_int, _lp]
        L.orc_internal_points_staela.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                 _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int]
        L.orc_internal_points_harela.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 6 + [ctypes.c_int, _dp, _dp,
                                                                                          _dp, _dp, _dp, _dp,
                                                                                          ctypes.c_int]
        L.orc_pair_staela.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                      _dp, _dp]
        L.orc_pair_harela.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6 + [_dp, _dp]
        L.orc_harela_parameters.argtypes = [ctypes.c_double] * 6 + [_dp]
        L.orc_gauss_tables.argtypes = [_dp] * 4
        L.orc_qs_parameters.argtypes = [ctypes.c_double, _dp]
        L.orc_qs_estimate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_zexp.argtypes = [ctypes.c_double, ctypes.c_double, _dp]
        L.orc_nearest_quad8.argtypes = [_dp, ctypes.c_double, _dp, _dp, _dp, _dp, _ip]
        L.orc_freeterm.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_double, _dp]
        L.orc_problem_set_halfspace.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.orc_hsc_point.argtypes = [ctypes.c_double] * 3 + [_dp] * 5
        L.orc_hsc_hbie_point.argtypes = [ctypes.c_double] * 3 + [_dp] * 6
        L.orc_hsc_sigma_ad.argtypes = [ctypes.c_double] * 3 + [_dp] * 3
        L.orc_pair_hsc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   _dp, _dp]
        L.orc_problem_set_formulation.argtypes = [ctypes.c_void_p, _ip, _dp, _dp]
        L.orc_problem_set_crack.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _ip, _dp]
        L.orc_dof2_map.argtypes = [ctypes.c_void_p, _ip]
        L.orc_colloc_normals.argtypes = [ctypes.c_void_p, _dp]
        L.orc_pair_hbie_staela.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, _dp, _dp]
        L.orc_pair_hbie_harela.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6 + \
            [_dp, _dp]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


# settings defaults, src/read_settings.f90:86,101,143-145,164
DEFAULTS = dict(qsi_re=1e-6, ns_max=16, ps_gln=(2, 3, 4, 5, 6, 7, 8, 9), geo_tol=1e-6)


class Problem:
    """One BE region of a deck prepared as the reference's build_data* and
    build_auxiliary_variables_* leave it."""

    def __init__(self, deck, **settings):
        s = dict(DEFAULTS)
        s.update(settings)
        self.deck = deck
        L = lib()
        X = np.ascontiguousarray(deck.nodes, dtype=np.float64)
        conn = np.ascontiguousarray(deck.conn, dtype=np.int32)
        ct = np.ascontiguousarray(deck.ctype, dtype=np.int32)
        cv = np.ascontiguousarray(deck.cvalue, dtype=np.complex128).view(np.float64)
        gl = np.array(s["ps_gln"], dtype=np.int32)
        self._h = L.orc_problem_new(deck.n_nodes, _p(X), deck.n_elements, _p(conn, _ip), _p(ct, _ip), _p(cv),
                                    s["qsi_re"], s["ns_max"], len(gl), _p(gl, _ip), s["geo_tol"])
        self.n = L.orc_n_dof(self._h)
        self.settings = s

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_problem_free(self._h)
            self._h = None

    def dof_map(self):
        nn = self.deck.n_nodes
        dof = np.zeros(3 * nn, dtype=np.int32)
        order = np.zeros(nn, dtype=np.int32)
        lib().orc_dof_map(self._h, _p(dof, _ip), _p(order, _ip))
        return dof.reshape(nn, 3), order

    def element_data(self):
        ne = self.deck.n_elements
        cl = np.zeros(ne)
        gf = np.zeros(ne, dtype=np.int32)
        ball = np.zeros((ne, 4))
        lib().orc_element_data(self._h, _p(cl), _p(gf, _ip), _p(ball))
        return cl, gf, ball

    def colloc(self):
        m = lib().orc_n_colloc(self._h)
        x = np.zeros((m, 3))
        info = np.zeros((m, 4), dtype=np.int32)
        lib().orc_colloc(self._h, _p(x), _p(info, _ip))
        return x, info

    def set_halfspace(self, n=-3, x=0.0, bc=1):
        """Half-space region (read_regions.f90:130-200): hyperplane normal n,
        coordinate x, traction-free surface (bc 1). The static builder adds the
        complementary kernel (n = -3 only) and both builders double the free
        term of collocation points on the surface."""
        if lib().orc_problem_set_halfspace(self._h, int(n), float(x), int(bc)) != 0:
            raise ValueError("half-space: n in -3..3 and bc = 1 only")

    _ERR = {-1: "invalid normals/tangents configuration at a free-term node",
            -2: "a point lies outside the half-space",
            -3: "an element containing a collocation point on the free surface does not lie on it",
            -4: "the static half-space kernel needs the hyperplane normal n = -3",
            -5: "HBIE formulations in a half-space region are not available",
            -6: "the HBIE cannot be collocated at an element edge"}

    FORMULATIONS = {"sbie": 0, "hbie": 1, "dual_bm": 2, "dual_bm_mixed": 3}

    def set_formulation(self, form, alpha=None, delta=None):
        """BEM formulation of every node (src/read_bem_formulation_selected_nodes.f90):
        form is one name of FORMULATIONS for all nodes or an array of codes per
        node (0 default SBIE, 1 'hbie', 2 'dual_bm_same', 3 'dual_bm_mixed');
        alpha (Burton &
        Miller weight) and delta (HBIE point offset, default 0.22540333) per
        node or scalar. Rebuilds the collocation points."""
        nn = self.deck.n_nodes
        f = np.full(nn, self.FORMULATIONS[form], dtype=np.int32) if isinstance(form, str) else \
            np.ascontiguousarray(form, dtype=np.int32)
        a = np.ascontiguousarray(np.broadcast_to(1.0 if alpha is None else alpha, (nn,)), dtype=np.float64)
        dl = np.ascontiguousarray(np.broadcast_to(0.22540333 if delta is None else delta, (nn,)), dtype=np.float64)
        if lib().orc_problem_set_formulation(self._h, _p(f, _ip), _p(a), _p(dl)) != 0:
            raise ValueError("formulation codes must be 0, 1, 2 or 3")

    def set_crack(self, crack_el, ctype2, cvalue2):
        """Crack-like boundary (dual BEM): crack_el [ne] bool marks its
        elements; ctype2, cvalue2 [nn, 3] the boundary conditions of face 2
        (face 1: the deck's ctype / cvalue). Renumbers the DOF."""
        ce = np.ascontiguousarray(np.asarray(crack_el, dtype=bool).astype(np.int8))
        ct = np.ascontiguousarray(ctype2, dtype=np.int32)
        cv = np.ascontiguousarray(cvalue2, dtype=np.complex128).view(np.float64)
        if lib().orc_problem_set_crack(self._h, ce.ctypes.data_as(ctypes.c_char_p), _p(ct, _ip), _p(cv)) != 0:
            raise ValueError("a crack node also belongs to an ordinary element")
        self.n = lib().orc_n_dof(self._h)
        self._crack = (np.asarray(crack_el, dtype=bool), ct.copy(), np.asarray(cvalue2, dtype=np.complex128).copy())

    def dof2_map(self):
        nn = self.deck.n_nodes
        d = np.zeros(3 * nn, dtype=np.int32)
        lib().orc_dof2_map(self._h, _p(d, _ip))
        return d.reshape(nn, 3)

    def solution_faces(self, x):
        """(u1, t1, u2, t2) [nn, 3]: face 1 of every node, face 2 of the crack
        nodes (zero elsewhere)."""
        u1, t1 = self.solution(x)
        ce, ct2, cv2 = self._crack
        d2 = self.dof2_map()
        u2 = np.zeros_like(u1)
        t2 = np.zeros_like(t1)
        nodes = np.unique(self.deck.conn[ce])
        for s in nodes:
            for c in range(3):
                v = x[d2[s, c]]
                kv = cv2[s, c] if np.iscomplexobj(x) else cv2[s, c].real
                if ct2[s, c] == 0:
                    u2[s, c], t2[s, c] = kv, v
                else:
                    u2[s, c], t2[s, c] = v, kv
        return u1, t1, u2, t2

    def colloc_normals(self):
        m = lib().orc_n_colloc(self._h)
        nrm = np.zeros((m, 3))
        lib().orc_colloc_normals(self._h, _p(nrm))
        return nrm

    def pair_hbie(self, ci, e, mu=None, nu=None, mat=None, omega=None):
        """HBIE kernels (m, l [8, 3, 3]) of collocation point ci against element
        e: static with mu, nu, harmonic with mat, omega."""
        cplx = omega is not None
        dt = np.complex128 if cplx else np.float64
        m = np.zeros((8, 3, 3), dtype=dt)
        l = np.zeros((8, 3, 3), dtype=dt)
        if cplx:
            lam, mu_ = complex(mat["lambda"]), complex(mat["mu"])
            cls = lib().orc_pair_hbie_harela(self._h, ci, e, lam.real, lam.imag, mu_.real, mu_.imag,
                                             float(mat["rho"]), float(omega), _p(m), _p(l))
        else:
            cls = lib().orc_pair_hbie_staela(self._h, ci, e, float(mu), float(nu), _p(m), _p(l))
        if cls < 0:
            raise RuntimeError("oracle: " + self._ERR.get(cls, str(cls)))
        return cls, m, l

    def assemble_staela(self, mu, nu, nthreads=0):
        n = self.n
        A = np.zeros((n, n), dtype=np.float64, order="F")
        b = np.zeros(n, dtype=np.float64)
        st = np.zeros(12, dtype=np.int64)
        rc = lib().orc_assemble_staela(self._h, mu, nu, _p(A), _p(b), nthreads, _p(st, _lp))
        if rc != 0:
            raise RuntimeError("oracle: " + self._ERR.get(rc, str(rc)))
        self.stats = st
        return A, b

    def pair_hsc(self, ci, e, mu, nu):
        h = np.zeros((8, 3, 3))
        g = np.zeros((8, 3, 3))
        cls = lib().orc_pair_hsc(self._h, ci, e, mu, nu, _p(h), _p(g))
        if cls < 0:
            raise RuntimeError("oracle: " + self._ERR.get(cls, str(cls)))
        return cls, h, g

    def assemble_harela(self, mat, omega, nthreads=0):
        n = self.n
        A = np.zeros((n, n), dtype=np.complex128, order="F")
        b = np.zeros(n, dtype=np.complex128)
        st = np.zeros(12, dtype=np.int64)
        lam, mu, nu = complex(mat["lambda"]), complex(mat["mu"]), complex(mat["nu"])
        rc = lib().orc_assemble_harela_nu(self._h, lam.real, lam.imag, mu.real, mu.imag, float(mat["rho"]),
                                          float(omega), nu.real, nu.imag, _p(A), _p(b), nthreads, _p(st, _lp))
        if rc != 0:
            raise RuntimeError("oracle: " + self._ERR.get(rc, str(rc)))
        self.stats = st
        return A, b

    def pair_staela(self, ci, e, mu, nu):
        h = np.zeros((8, 3, 3))
        g = np.zeros((8, 3, 3))
        cls = lib().orc_pair_staela(self._h, ci, e, mu, nu, _p(h), _p(g))
        return cls, h, g

    def pair_harela(self, ci, e, mat, omega):
        h = np.zeros((8, 3, 3), dtype=np.complex128)
        g = np.zeros((8, 3, 3), dtype=np.complex128)
        lam, mu = complex(mat["lambda"]), complex(mat["mu"])
        cls = lib().orc_pair_harela(self._h, ci, e, lam.real, lam.imag, mu.real, mu.imag, float(mat["rho"]),
                                    float(omega), _p(h), _p(g))
        return cls, h, g

    def internal_points(self, xip, u, t, mat=None, omega=None, mu=None, nu=None, nthreads=0, u2=None, t2=None):
        """Displacement [nip,3] and stresses [nip,3,3] (sigma[:, il, kc]) at
        internal points from nodal u, t [nn,3] (and face 2's u2, t2 with
        crack-like boundaries); static with mu, nu, harmonic with mat, omega."""
        xip = np.ascontiguousarray(xip, dtype=np.float64)
        nip = len(xip)
        cplx = omega is not None
        dt = np.complex128 if cplx else np.float64
        u = np.ascontiguousarray(u, dtype=dt)
        t = np.ascontiguousarray(t, dtype=dt)
        if u2 is not None:
            u2 = np.ascontiguousarray(u2, dtype=dt)
            t2 = np.ascontiguousarray(t2, dtype=dt)
        out = np.zeros((nip, 4, 3), dtype=dt)
        if cplx:
            lam, m = complex(mat["lambda"]), complex(mat["mu"])
            rc = lib().orc_internal_points_harela(self._h, lam.real, lam.imag, m.real, m.imag, float(mat["rho"]),
                                                  float(omega), nip, _p(xip), _p(u), _p(t), _p(u2), _p(t2), _p(out),
                                                  nthreads)
        else:
            rc = lib().orc_internal_points_staela(self._h, float(mu), float(nu), nip, _p(xip), _p(u), _p(t), _p(u2),
                                                  _p(t2), _p(out), nthreads)
        if rc == -7:
            raise RuntimeError("half-space internal points: normal -3 and a traction-free surface only")
        if rc == -8:
            raise RuntimeError("half-space internal points: a point lies outside the half-space")
        if rc:
            raise ValueError(f"internal point {rc - 1} lies on the boundary (on an element away from its nodes, "
                             "or at a node of a crack-like boundary)")
        return out[:, 0, :], np.transpose(out[:, 1:, :], (0, 2, 1))

    def solution(self, x):
        """Nodal (u, t) from the solved unknown vector: the variable of each
        (node, direction) DOF is u if the traction is known, t otherwise
        (src/assign_solution_mechanics_static.f90:130-150)."""
        d = self.deck
        dof, _ = self.dof_map()
        u = np.zeros((d.n_nodes, 3), dtype=x.dtype)
        t = np.zeros((d.n_nodes, 3), dtype=x.dtype)
        known_u = d.ctype == 0
        u[known_u] = d.cvalue[known_u].astype(x.dtype) if np.iscomplexobj(x) else d.cvalue[known_u].real
        t[~known_u] = d.cvalue[~known_u].astype(x.dtype) if np.iscomplexobj(x) else d.cvalue[~known_u].real
        vals = x[dof]
        u[~known_u] = vals[~known_u]
        t[known_u] = vals[known_u]
        return u, t


def lu_solve(A, b, threads=None, overwrite=False, rcond=False):
    """getrf + getrs (partial pivoting) through scipy's OpenBLAS. overwrite:
    factorise A in place (no copy of a large system); rcond: also return
    LAPACK's ?gecon estimate of the reciprocal one-norm condition number."""
    import scipy.linalg as sl
    anorm = float(np.abs(A).sum(axis=0).max()) if rcond else 0.0
    lu, piv = sl.lu_factor(A, overwrite_a=overwrite, check_finite=False)
    x = sl.lu_solve((lu, piv), b, check_finite=False)
    if not rcond:
        return x
    con = sl.lapack.zgecon if np.iscomplexobj(lu) else sl.lapack.dgecon
    rc, info = con(lu, anorm, norm="1")
    return x, float(rc)


def hsc_point(mu, nu, xp, x_i, x, n):
    """Complementary half-space kernel at one point: u, t [3, 3] (load, component)."""
    u = np.zeros((3, 3))
    t = np.zeros((3, 3))
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (x_i, x, n)]
    rc = lib().orc_hsc_point(mu, nu, xp, *[_p(v) for v in a], _p(u), _p(t))
    if rc:
        raise ValueError("point outside the half-space")
    return u, t


def hsc_hbie_point(mu, nu, xp, x_i, n_i, x, n):
    """Complementary half-space HBIE kernels at one point: d, s [3, 3]."""
    d = np.zeros((3, 3))
    s = np.zeros((3, 3))
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (x_i, n_i, x, n)]
    if lib().orc_hsc_hbie_point(mu, nu, xp, *[_p(v) for v in a], _p(d), _p(s)):
        raise ValueError("point outside the half-space")
    return d, s


def hsc_sigma_ad(mu, nu, xp, x_i, x):
    """Complementary stress sigma[l, k, j] (load l) from the differentiated u*."""
    sig = np.zeros((3, 3, 3))
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (x_i, x)]
    lib().orc_hsc_sigma_ad(mu, nu, xp, *[_p(v) for v in a], _p(sig))
    return sig


def gauss_tables():
    a = [np.zeros(32 * 32) for _ in range(4)]
    lib().orc_gauss_tables(*[_p(x) for x in a])
    return [x.reshape(32, 32) for x in a]  # [rule-1, point-1]
