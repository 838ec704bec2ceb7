"""Host-side mirror of the reference's region-builder / solver interface for the
collocation-BEM path (the calls MultiFEBE's Fortran makes, from Python).

    region = BemRegion(deck)                         # build_data* + mesh upload
    A, b = region.build_lse_staela(mu, nu)           # build_lse_mechanics_bem_staela
    A, b = region.build_lse_harela(material, omega)  # build_lse_mechanics_bem_harela
    x = solve_lse(A, b)                              # solve_lse_r / solve_lse_c (FP64 LU on the GPU)
    X = region.sweep_harela(material, omegas, precision="mixed")   # batched device sweep
    u, t = region.solution(x)                        # assign_solution_*

Every compute call goes through the native library (CUDA kernels for sm_103a);
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import check

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)

# src/read_settings.f90 defaults
DEFAULT_SETTINGS = dict(qsi_relative_error=1e-6, qsi_ns_max=16, precalset_gln=(2, 3, 4, 5, 6, 7, 8, 9),
                        geometric_tolerance=1e-6)


# precision argument of mfbem_sweep_harela / mfbem_solve_staela
PRECISION = {"plain": 0, "mixed": 1, "mixed-gmres": 2}


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


class BemRegion:
    """One BE region (ordinary boundaries, continuous quad8) on the GPU.

    formulation: None / 'sbie' (the default SBIE with MCA at mesh-boundary
    nodes), 'hbie', 'dual_bm' ('dual_bm_same': Burton & Miller with weight
    alpha at common points) or 'dual_bm_mixed' (the SBIE at its own nodal or
    MCA point), for every node or as an array of codes per node (0..3); delta
    moves the HBIE points into the elements (default 0.22540333). crack:
    (crack_el [ne] bool, ctype2 [nn, 3], cvalue2 [nn, 3]) marks the elements
    of crack-like boundaries (dual BEM) and gives face 2's conditions; the
    deck's ctype / cvalue are face 1's. See mfbem_mesh_upload_dual."""

    FORMULATIONS = {"sbie": 0, "hbie": 1, "dual_bm": 2, "dual_bm_mixed": 3}

    def __init__(self, deck, formulation=None, alpha=None, delta=None, crack=None, **settings):
        s = dict(DEFAULT_SETTINGS)
        s.update(settings)
        self.deck = deck
        self.settings = s
        L = _abi.load()
        self._X = np.ascontiguousarray(deck.nodes, dtype=np.float64)
        self._conn = np.ascontiguousarray(deck.conn, dtype=np.int32)
        self._ct = np.ascontiguousarray(deck.ctype, dtype=np.int32)
        self._cv = np.ascontiguousarray(deck.cvalue, dtype=np.complex128)
        self._gl = np.ascontiguousarray(s["precalset_gln"], dtype=np.int32)
        self._prep = L.mfbem_prep_create(deck.n_nodes, _p(self._X), deck.n_elements, _p(self._conn, _ip),
                                         _p(self._ct, _ip), _p(self._cv.view(np.float64)), s["qsi_relative_error"],
                                         s["qsi_ns_max"], len(self._gl), _p(self._gl, _ip),
                                         s["geometric_tolerance"])
        self.desc = L.mfbem_prep_desc(self._prep)
        self._h = ctypes.c_void_p()
        self.crack = None
        if formulation is None and crack is None:
            self.n = int(self.desc.contents.n_dof)
            check(L.mfbem_mesh_upload(self.desc, ctypes.byref(self._h)))
            return
        nn = deck.n_nodes
        if formulation is None:
            formulation = "sbie"
        f = np.full(nn, self.FORMULATIONS[formulation], dtype=np.int32) if isinstance(formulation, str) else \
            np.ascontiguousarray(formulation, dtype=np.int32)
        a = np.ascontiguousarray(np.broadcast_to(1.0 if alpha is None else alpha, (nn,)), dtype=np.float64)
        dl = np.ascontiguousarray(np.broadcast_to(0.22540333 if delta is None else delta, (nn,)), dtype=np.float64)
        if L.mfbem_prep_set_formulation(self._prep, _p(f, _ip), _p(a), _p(dl)) != 0:
            raise ValueError("formulation codes must be 0, 1, 2 or 3")
        if crack is not None:
            ce = np.ascontiguousarray(np.asarray(crack[0], dtype=bool), dtype=np.int32)
            ct2 = np.ascontiguousarray(crack[1], dtype=np.int32)
            cv2 = np.ascontiguousarray(crack[2], dtype=np.complex128)
            rc = L.mfbem_prep_set_crack(self._prep, _p(ce, _ip), _p(ct2, _ip), _p(cv2.view(np.float64)))
            if rc == -1:
                raise ValueError("a node of a crack-like element also belongs to an ordinary element")
            if rc != 0:
                raise ValueError("ctype2 must be 0 or 1")
            self.crack = (ce.astype(bool), ct2, cv2)
            self._crack_keep = (ce, ct2, cv2)
        self.n = int(self.desc.contents.n_dof)
        check(L.mfbem_mesh_upload_dual(self.desc, L.mfbem_prep_dual(self._prep), ctypes.byref(self._h)))

    def close(self):
        L = _abi.load()
        if getattr(self, "_h", None) is not None and self._h.value:
            L.mfbem_mesh_release(self._h)
            self._h = ctypes.c_void_p()
        if getattr(self, "_prep", None):
            L.mfbem_prep_free(self._prep)
            self._prep = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- data
    def dof_map(self):
        nn = self.deck.n_nodes
        dof = np.zeros(3 * nn, dtype=np.int32)
        order = np.zeros(nn, dtype=np.int32)
        _abi.load().mfbem_prep_dof(self._prep, _p(dof, _ip), _p(order, _ip))
        return dof.reshape(nn, 3), order

    def element_data(self):
        d = self.desc.contents
        ne = self.deck.n_elements
        cl = np.ctypeslib.as_array(d.csize, shape=(ne,)).copy()
        gf = np.ctypeslib.as_array(d.n_phi, shape=(ne,)).copy()
        ball = np.ctypeslib.as_array(d.bball, shape=(ne * 4,)).reshape(ne, 4).copy()
        return cl, gf, ball

    def stats(self):
        s = _abi.Stats()
        check(_abi.load().mfbem_last_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def set_halfspace(self, n=-3, x=0.0, bc=1):
        """Region space (src/read_regions.f90:130-200): n = 0 full space, else
        the half-space with hyperplane normal n (+-1..3), coordinate x and a
        traction-free surface (bc 1). See mfbem_set_halfspace."""
        L = _abi.load()
        L.mfbem_set_halfspace.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_int32]
        check(L.mfbem_set_halfspace(self._h, int(n), float(x), int(bc)))

    # ---------------------------------------------------------------- builders
    def build_lse_staela(self, mu, nu, A=None, b=None):
        n = self.n
        if A is None:
            A = np.zeros((n, n), dtype=np.float64, order="F")
        if b is None:
            b = np.zeros(n, dtype=np.float64)
        assert A.flags.f_contiguous and A.dtype == np.float64 and b.dtype == np.float64
        check(_abi.load().mfbem_assemble_staela(self._h, float(mu), float(nu), _p(A), A.shape[0], _p(b), 0))
        return A, b

    def build_lse_harela(self, mat, omega, A=None, b=None):
        n = self.n
        if A is None:
            A = np.zeros((n, n), dtype=np.complex128, order="F")
        if b is None:
            b = np.zeros(n, dtype=np.complex128)
        assert A.flags.f_contiguous and A.dtype == np.complex128 and b.dtype == np.complex128
        lam = np.array([complex(mat["lambda"]).real, complex(mat["lambda"]).imag])
        mu = np.array([complex(mat["mu"]).real, complex(mat["mu"]).imag])
        nu = np.array([complex(mat["nu"]).real, complex(mat["nu"]).imag])
        check(_abi.load().mfbem_assemble_harela(self._h, _p(lam), _p(mu), float(mat["rho"]), _p(nu), float(omega),
                                                _p(A), A.shape[0], _p(b), 0))
        return A, b

    # ---------------------------------------------------------------- device pipelines
    def sweep_harela(self, mat, omegas, precision="plain", rel_tol=1e-12):
        """Assemble + factorise + solve every frequency on the device.
        precision 'plain': FP64 LU; 'mixed': complex64 LU + FP64 refinement
        (classical, then GMRES-based when it stalls); 'mixed-gmres': complex64
        LU + GMRES-based refinement from the start."""
        om = np.ascontiguousarray(omegas, dtype=np.float64)
        nf = om.size
        X = np.zeros((nf, self.n), dtype=np.complex128)
        lam = np.array([complex(mat["lambda"]).real, complex(mat["lambda"]).imag])
        mu = np.array([complex(mat["mu"]).real, complex(mat["mu"]).imag])
        nu = np.array([complex(mat["nu"]).real, complex(mat["nu"]).imag])
        st = _abi.Stats()
        prec = PRECISION[precision]
        check(_abi.load().mfbem_sweep_harela(self._h, _p(lam), _p(mu), float(mat["rho"]), _p(nu), nf, _p(om), prec,
                                             rel_tol, _p(X), 0, ctypes.byref(st)))
        self.last_stats = st.as_dict()
        return X

    def set_learned_quadrature(self, weights=None, log10_tol=-6.0, kernel=0, kcl=0.0):
        """Rebuild the quasi-singular (adaptive) pairs' rules: with `weights`
        (a trained qlearn network) each pair takes the cheapest rule whose
        predicted log10 relative error is <= log10_tol, or keeps the reference
        adaptive rule when none qualifies; weights=None restores the reference
        rule everywhere. Returns the number of pairs on a learned rule."""
        from . import qlearn
        L = qlearn._lib()
        nl = ctypes.c_int32(0)
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        check(L.mfbem_set_learned_quadrature(self._h, None if w is None else w.ctypes.data, float(log10_tol),
                                             int(kernel), float(kcl), ctypes.byref(nl)))
        return int(nl.value)

    def solve_staela(self, mu, nu, precision="plain", rel_tol=1e-12):
        x = np.zeros(self.n, dtype=np.float64)
        st = _abi.Stats()
        prec = PRECISION[precision]
        check(_abi.load().mfbem_solve_staela(self._h, float(mu), float(nu), prec, rel_tol, _p(x), 0,
                                             ctypes.byref(st)))
        self.last_stats = st.as_dict()
        return x

    def internal_points(self, xip, u, t, mat=None, omega=None, mu=None, nu=None, u2=None, t2=None):
        """calculate_internal_points_mechanics_bem_{staela,harela}: displacement
        [nip, 3] and stress tensor [nip, 3, 3] (sigma[:, il, kc]) at points
        inside the region from the nodal solution u, t [n_nodes, 3] (as
        solution() returns it; with crack-like boundaries also face 2's u2,
        t2, as solution_faces() returns them). Static with mu, nu; harmonic
        with mat, omega."""
        L = _abi.load()
        xip = np.ascontiguousarray(xip, dtype=np.float64).reshape(-1, 3)
        nip = len(xip)
        cplx = omega is not None
        dt = np.complex128 if cplx else np.float64
        u = np.ascontiguousarray(u, dtype=dt)
        t = np.ascontiguousarray(t, dtype=dt)
        assert u.shape == (self.deck.n_nodes, 3) and t.shape == u.shape
        faces = u2 is not None
        if faces:
            u2 = np.ascontiguousarray(u2, dtype=dt)
            t2 = np.ascontiguousarray(t2, dtype=dt)
            assert u2.shape == u.shape and t2.shape == u.shape
        ui = np.zeros((nip, 3), dtype=dt)
        si = np.zeros((nip, 3, 3), dtype=dt)  # [ip][kc][il], as value_c(il, kc)
        if cplx:
            lam = np.array([complex(mat["lambda"]).real, complex(mat["lambda"]).imag])
            m = np.array([complex(mat["mu"]).real, complex(mat["mu"]).imag])
            if faces:
                check(L.mfbem_internal_points_faces_harela(self._h, _p(lam), _p(m), float(mat["rho"]), float(omega),
                                                           nip, _p(xip), _p(u), _p(t), _p(u2), _p(t2), _p(ui),
                                                           _p(si)))
            else:
                check(L.mfbem_internal_points_harela(self._h, _p(lam), _p(m), float(mat["rho"]), float(omega), nip,
                                                     _p(xip), _p(u), _p(t), _p(ui), _p(si)))
        elif faces:
            check(L.mfbem_internal_points_faces_staela(self._h, float(mu), float(nu), nip, _p(xip), _p(u), _p(t),
                                                       _p(u2), _p(t2), _p(ui), _p(si)))
        else:
            check(L.mfbem_internal_points_staela(self._h, float(mu), float(nu), nip, _p(xip), _p(u), _p(t), _p(ui),
                                                 _p(si)))
        return ui, np.transpose(si, (0, 2, 1))

    def solution(self, x):
        """Nodal (u, t): the unknown of each (node, direction) is u when the
        traction is prescribed and t otherwise (src/assign_solution_mechanics_static.f90:130-150)."""
        d = self.deck
        dof, _ = self.dof_map()
        cplx = np.iscomplexobj(x)
        dt = np.complex128 if cplx else np.float64
        cv = d.cvalue if cplx else d.cvalue.real
        known_u = d.ctype == 0
        u = np.where(known_u, cv, 0).astype(dt)
        t = np.where(~known_u, cv, 0).astype(dt)
        vals = x[dof]
        u[~known_u] = vals[~known_u]
        t[known_u] = vals[known_u]
        return u, t

    def solution_faces(self, x):
        """(u1, t1, u2, t2) [n_nodes, 3] of a region with crack-like
        boundaries: face 1 of every node (solution()) and face 2 of the crack
        nodes (zero elsewhere)."""
        u1, t1 = self.solution(x)
        ce, ct2, cv2 = self.crack
        nn = self.deck.n_nodes
        d2 = np.zeros(3 * nn, dtype=np.int32)
        _abi.load().mfbem_prep_dof2(self._prep, _p(d2, _ip))
        d2 = d2.reshape(nn, 3)
        cplx = np.iscomplexobj(x)
        cv = cv2 if cplx else cv2.real
        on = d2 >= 0
        known_u = on & (ct2 == 0)
        known_t = on & (ct2 == 1)
        vals = np.where(on, x[np.maximum(d2, 0)], 0)
        u2 = np.where(known_u, cv, np.where(known_t, vals, 0)).astype(u1.dtype)
        t2 = np.where(known_t, cv, np.where(known_u, vals, 0)).astype(u1.dtype)
        return u1, t1, u2, t2


class LseState:
    """The caller-owned arrays solve_lse_{r,c} keep between calls (Ao, equed,
    r, c: src/problem_variables.f90 Ao_r/Ao_c, scal_equed, scal_r, scal_c)
    and the diagnostics the reference prints (rcond, ferr, berr)."""

    def __init__(self):
        self.Ao = None
        self.equed = "N"
        self.r = None
        self.c = None
        self.rcond = float("nan")
        self.ferr = None
        self.berr = None


def solve_lse(A, b, ipiv=None, factorize=True, scaling=False, condition=False, refine=False, state=None):
    """solve_lse_r / solve_lse_c with LAPACK semantics: A (Fortran order) is
    overwritten by its (equilibrated) LU factors, ipiv by the 1-based pivots,
    b by x. scaling / condition / refine are the reference's lse_scaling,
    lse_condition and lse_refine; their arrays live in `state` (an LseState),
    which a later call with factorize=False must be given again."""
    L = _abi.load()
    n = A.shape[0]
    assert A.flags.f_contiguous
    if ipiv is None:
        ipiv = np.zeros(n, dtype=np.int32)
    bb = b if b.ndim == 2 else b.reshape(n, 1)
    nrhs = bb.shape[1]
    assert bb.flags.f_contiguous
    if (scaling or condition or refine) and state is None:
        raise ValueError("scaling / condition / refine need an LseState")
    st = state
    Ao = eq = r = c = None
    aodim = 1
    if condition or refine:
        if st.Ao is None or st.Ao.shape != A.shape or st.Ao.dtype != A.dtype:
            if not factorize:
                raise ValueError("refine without factorize needs the state of the factorising call")
            st.Ao = np.zeros_like(A, order="F")
        Ao, aodim = st.Ao, n
    if scaling:
        if st.r is None or st.r.shape != (n,):
            st.r, st.c = np.zeros(n), np.zeros(n)
        eq = ctypes.create_string_buffer(st.equed.encode(), 2)
        r, c = st.r, st.c
    fn = L.mfbem_solve_c if np.iscomplexobj(A) else L.mfbem_solve_r
    rc = fn(n, _p(A), _p(ipiv, _ip), aodim, _p(Ao), eq, _p(r), _p(c), nrhs, _p(bb), 1 if factorize else 0,
            int(bool(scaling)), int(bool(condition)), int(bool(refine)))
    check(rc)
    if st is not None:
        if scaling:
            st.equed = eq.value.decode()
        rcond = ctypes.c_double()
        fe, be = np.zeros(nrhs), np.zeros(nrhs)
        check(L.mfbem_solve_report(ctypes.byref(rcond), nrhs, _p(fe), _p(be)))
        st.rcond = rcond.value
        st.ferr, st.berr = (fe, be) if refine else (None, None)
    return b, ipiv


def sweep_harela_batch(regions, materials, omegas, precision="mixed", rel_tol=1e-12):
    """Sweeps of several meshes (uneven sizes allowed) in one call: every
    mesh's sweep runs concurrently on the GPU (its own stream). Returns the
    list of solution arrays [n_freq_i, n_i] and the per-mesh stats."""
    k = len(regions)
    vp = ctypes.c_void_p
    L = _abi.load()
    if not getattr(L, "_batch_set", False):
        L.mfbem_sweep_harela_batch.argtypes = [ctypes.c_int32, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int32,
                                               ctypes.c_double, vp, ctypes.c_int32, vp]
        L._batch_set = True
    mats = materials if isinstance(materials, (list, tuple)) else [materials] * k
    oms = [np.ascontiguousarray(o, dtype=np.float64) for o in omegas]
    lam = np.array([[complex(m["lambda"]).real, complex(m["lambda"]).imag] for m in mats])
    mu = np.array([[complex(m["mu"]).real, complex(m["mu"]).imag] for m in mats])
    nu = np.array([[complex(m["nu"]).real, complex(m["nu"]).imag] for m in mats])
    rho = np.array([float(m["rho"]) for m in mats])
    nf = np.array([len(o) for o in oms], dtype=np.int32)
    X = [np.zeros((len(o), r.n), dtype=np.complex128) for o, r in zip(oms, regions)]
    hs = (vp * k)(*[r._h.value for r in regions])
    op = (vp * k)(*[o.ctypes.data for o in oms])
    xp = (vp * k)(*[x.ctypes.data for x in X])
    st = (_abi.Stats * k)()
    check(L.mfbem_sweep_harela_batch(k, hs, lam.ctypes.data, mu.ctypes.data, rho.ctypes.data, nu.ctypes.data,
                                     nf.ctypes.data, op, PRECISION[precision], rel_tol, xp, 0, st))
    return X, [s.as_dict() for s in st]
