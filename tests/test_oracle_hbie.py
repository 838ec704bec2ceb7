"""The oracle's HBIE (traction boundary integral equation) on the boundary and
the Burton & Miller / HBIE formulations of the region builders.

Pins the restatement of the interior (hypersingular) integration
fbem_bem_staela3d_hbie_int (lib/fbem/src/bem_staela3d.f90:4918-5353), its line
integrals (:5356-5578), fbem_bem_harela3d_hbie_int (bem_harela3d.f90:3169-3630)
and shbie_auto (:4888-4957) against identities and closed forms:
  - rigid-body translation: the integrated s* kernel of a closed surface sums
    to zero for every collocation point (to the quadrature tolerance, which
    the singular element dominates);
  - uniform stress state: 1/2 t(x_i) + sum m u = sum l t with u linear and t
    = sigma n exact on a flat-faced cube;
  - the harmonic kernels tend to the static ones as omega -> 0;
  - a plane P wave satisfies the harmonic identity to the discretisation
    error, which shrinks with the mesh;
  - the builders with 'dual_bm_same', 'hbie' and 'dual_bm_mixed'
    formulations reproduce the closed forms of docs/examples/ME-ST-EL-002
    (confined cube, exact linear field) and ME-TH-EL-001 (P-wave column).
"""
import numpy as np
import pytest

from multifebe_gb300 import meshgen as M

MU, NU = 0.4, 0.25


def hbie_problem(oracle, n, qsi=1e-6, form="hbie"):
    d = M.box((1.0, 1.0, 1.0), (n, n, n), split_faces=False)
    P = oracle.Problem(d, qsi_re=qsi)
    P.set_formulation(form)
    return d, P


@pytest.mark.parametrize("qsi,tol", [(1e-6, 2e-6), (1e-9, 2e-9), (1e-12, 2e-10)])
def test_rigid_body_translation(oracle, qsi, tol):
    d, P = hbie_problem(oracle, 2, qsi)
    x, info = P.colloc()
    assert set(info[:, 1]) == {2} and len(x) == 8 * d.n_elements
    worst = 0.0
    for ci in range(0, len(x), 7):
        S = np.zeros((3, 3))
        tot = 0.0
        classes = set()
        for e in range(d.n_elements):
            cls, m, _ = P.pair_hbie(ci, e, MU, NU)
            classes.add(cls)
            S += m.sum(axis=0)
            tot += np.abs(m).sum()
        assert 101 in classes  # the element holding the point: interior integration
        worst = max(worst, np.abs(S).max() / tot)
    assert worst < tol, worst


@pytest.mark.parametrize("qsi,tol", [(1e-6, 1e-4), (1e-10, 2e-8)])
def test_uniform_stress_state(oracle, qsi, tol):
    lam = 2 * MU * NU / (1 - 2 * NU)
    sig = np.array([[1.0, 0.3, -0.2], [0.3, -0.5, 0.4], [-0.2, 0.4, 0.8]])
    eps = (sig - lam / (3 * lam + 2 * MU) * np.trace(sig) * np.eye(3)) / (2 * MU)
    d, P = hbie_problem(oracle, 2, qsi)
    x, info = P.colloc()
    nrm = P.colloc_normals()
    enorm = {int(info[ci, 2]): nrm[ci] for ci in range(len(x))}  # flat faces
    uN = d.nodes @ eps.T
    worst = 0.0
    for ci in range(0, len(x), 5):
        res = np.zeros(3)
        for e in range(d.n_elements):
            _, m, l = P.pair_hbie(ci, e, MU, NU)
            te = sig @ enorm[e]
            for k, s in enumerate(d.conn[e]):
                res += m[k] @ uN[s] - l[k] @ te
        ti = sig @ nrm[ci]
        worst = max(worst, np.abs(res + 0.5 * ti).max() / np.abs(ti).max())
    assert worst < tol, worst


def test_harmonic_static_limit(oracle):
    mat = M.viscoelastic(1.0, NU, 1.0, 0.0)
    d, P = hbie_problem(oracle, 2)
    x, _ = P.colloc()
    worst = 0.0
    for ci in range(0, len(x), 9):
        for e in range(d.n_elements):
            _, ms, ls = P.pair_hbie(ci, e, float(np.real(mat["mu"])), NU)
            _, mh, lh = P.pair_hbie(ci, e, mat=mat, omega=1e-4)
            sc = max(np.abs(ms).max(), np.abs(ls).max())
            worst = max(worst, np.abs(mh - ms).max() / sc, np.abs(lh - ls).max() / sc)
    assert worst < 1e-7, worst


def _plane_p_wave(mat, om, X, n, dvec=np.array([0.6, 0.48, 0.64])):
    lam, mu = complex(mat["lambda"]), complex(mat["mu"])
    k = om / np.sqrt((lam + 2 * mu) / mat["rho"])
    ph = np.exp(1j * k * (X @ dvec))
    u = ph[:, None] * dvec[None, :]
    sig = (lam * np.eye(3)[None] + 2 * mu * np.outer(dvec, dvec)[None]) * (1j * k * ph)[:, None, None]
    return u, np.einsum("pij,pj->pi", sig, n)


def test_plane_wave_identity_converges(oracle):
    mat = M.viscoelastic(1.0, NU, 1.0, 0.05)
    om = 1.5
    errs = []
    for n in (2, 4):
        d, P = hbie_problem(oracle, n, 1e-9)
        x, info = P.colloc()
        nrm = P.colloc_normals()
        enorm = {int(info[ci, 2]): nrm[ci] for ci in range(len(x))}
        uN, _ = _plane_p_wave(mat, om, d.nodes, np.zeros_like(d.nodes))
        worst = 0.0
        for ci in range(0, len(x), 11):
            res = np.zeros(3, complex)
            for e in range(d.n_elements):
                _, m, l = P.pair_hbie(ci, e, mat=mat, omega=om)
                _, tN = _plane_p_wave(mat, om, d.nodes[d.conn[e]], np.tile(enorm[e], (8, 1)))
                for k, s in enumerate(d.conn[e]):
                    res += m[k] @ uN[s] - l[k] @ tN[k]
            _, ti = _plane_p_wave(mat, om, x[ci:ci + 1], nrm[ci:ci + 1])
            worst = max(worst, np.abs(res + 0.5 * ti[0]).max() / np.abs(ti).max())
        errs.append(worst)
    assert errs[0] < 5e-3 and errs[1] < 1e-3 and errs[1] < errs[0] / 3, errs


@pytest.mark.parametrize("form", ["dual_bm", "hbie", "dual_bm_mixed"])
def test_confined_cube_static(oracle, form):
    """ME-ST-EL-002 through the static builder: Burton & Miller (alpha = 1,
    build_lse_mechanics_bem_staela.f90:835-841) and HBIE alone."""
    mat = M.elastic(1.0, 0.25)
    d = M.cube_confined_kat(2)
    P = oracle.Problem(d)
    P.set_formulation(form)
    A, b = P.assemble_staela(mat["mu"], mat["nu"])
    u, _ = P.solution(oracle.lu_solve(A, b))
    assert np.abs(u[:, 0] - (1.25 * 0.5 / 0.75) * d.nodes[:, 0]).max() < 2e-5
    assert np.abs(u[:, 1:]).max() < 2e-5
    # every pair of the HBIE points is integrated: 8 points per element
    assert P.stats[8] + P.stats[9] + P.stats[10] == (8 * d.n_elements) * d.n_elements
    assert P.stats[10] == 8 * d.n_elements


@pytest.mark.parametrize("form", ["dual_bm", "hbie", "dual_bm_mixed"])
def test_p_wave_column_harmonic(oracle, form):
    """ME-TH-EL-001 through the harmonic builder (Burton & Miller weight
    alpha i / c2, build_lse_mechanics_bem_harela.f90:1174-1181)."""
    mat = M.viscoelastic(2.4, 0.2, 1.0, 0.02)
    om = 2.0
    lam2mu = mat["lambda"] + 2.0 * mat["mu"]
    k = om / np.sqrt(lam2mu / mat["rho"])
    errs = []
    for n in (2, 4):
        d = M.cube_confined_kat(n)
        P = oracle.Problem(d)
        P.set_formulation(form)
        A, b = P.assemble_harela(mat, om)
        u, _ = P.solution(oracle.lu_solve(A, b))
        ue = np.sin(k * d.nodes[:, 0]) / (lam2mu * k * np.cos(k))
        errs.append(np.abs(u[:, 0] - ue).max() / np.abs(ue).max())
    assert errs[1] < 1e-3 and errs[1] < errs[0] / 4, errs


def test_burton_miller_is_the_weighted_sum(oracle):
    """With SBIE and HBIE at the same points, the Burton & Miller system is
    the SBIE-MCA system plus alpha times the HBIE system (static: the two
    kernels keep their own classification, bem_staela3d sbie_auto and
    hbie_auto)."""
    mat = M.elastic(1.0, 0.25)
    d = M.box((1.0, 1.0, 1.0), (2, 2, 2), split_faces=False)
    d.ctype[d.nodes[:, 2] < 1e-12] = 0
    alpha = 0.7
    sys = {}
    for form in ("dual_bm", "hbie"):
        P = oracle.Problem(d)
        P.set_formulation(form, alpha=alpha)
        sys[form] = P.assemble_staela(mat["mu"], mat["nu"])
    # SBIE-MCA at the same points: Burton & Miller with alpha = 0
    P = oracle.Problem(d)
    P.set_formulation("dual_bm", alpha=0.0)
    A0, b0 = P.assemble_staela(mat["mu"], mat["nu"])
    A1, b1 = sys["dual_bm"]
    Ah, bh = sys["hbie"]
    scale = np.abs(A1).max()
    assert np.abs(A1 - (A0 + alpha * Ah)).max() < 1e-13 * scale
    assert np.abs(b1 - (b0 + alpha * bh)).max() < 1e-13 * max(np.abs(b1).max(), 1.0)


@pytest.mark.parametrize("harmonic", [False, True])
def test_dual_bm_mixed_is_the_weighted_sum(oracle, harmonic):
    """'dual_bm_mixed' (src/read_bem_formulation_selected_nodes.f90:243-295):
    the node's SBIE at its own point (nodal, or MCA on the mesh boundary) plus
    beta alpha times the HBIE at the HBIE points of its elements, each
    integrated on its own (sbie_auto, hbie_auto), so the system is the SBIE
    system plus beta alpha times the 'hbie' system. The reference's
    non-common branch keeps the SBIE's h of a nodal point for the node's
    later elements; the oracle and the library assemble the weighted sum.
    (One closed boundary: every SBIE point nodal, as in the 'sbie' system.)"""
    d = M.box((1.0, 1.0, 1.0), (2, 2, 2), split_faces=False)
    d.ctype[d.nodes[:, 2] < 1e-12] = 0
    d.cvalue[d.nodes[:, 2] < 1e-12] = (0.1, -0.2, 0.3)
    d.cvalue[d.nodes[:, 2] > 1 - 1e-12] = (0.0, 0.0, -1.0)
    alpha = 0.7
    sysd = {}
    for form in ("dual_bm_mixed", "hbie", "sbie"):
        P = oracle.Problem(d)
        P.set_formulation(form, alpha=alpha)
        if harmonic:
            mat = M.viscoelastic(2.4, 0.2, 1.0, 0.02)
            sysd[form] = P.assemble_harela(mat, 2.0)
        else:
            sysd[form] = P.assemble_staela(MU, NU)
    beta = alpha * 1j / np.sqrt(mat["mu"] / mat["rho"]) if harmonic else alpha
    (A1, b1), (Ah, bh), (A0, b0) = sysd["dual_bm_mixed"], sysd["hbie"], sysd["sbie"]
    assert np.abs(A1 - (A0 + beta * Ah)).max() < 1e-14 * np.abs(A1).max()
    assert np.abs(b1 - (b0 + beta * bh)).max() < 1e-14 * max(np.abs(b1).max(), 1.0)


def test_dual_bm_mixed_points(oracle):
    """'dual_bm_mixed' collocation points: one HBIE point per element of the
    node (delta_hbie) and the SBIE at the node (nodal) or, on a mesh boundary,
    at MCA points moved by the quadratic default 0.22540333
    (read_bem_formulation_selected_nodes.f90:243-295)."""
    d = M.cube_confined_kat(1)  # six boundaries: every node on a mesh boundary
    P = oracle.Problem(d)
    P.set_formulation("dual_bm_mixed", delta=0.3)
    x, info = P.colloc()
    kinds = info[:, 1]
    assert (kinds == 5).sum() == 8 * d.n_elements and (kinds == 1).sum() == 8 * d.n_elements
    assert (kinds == 0).sum() == 0
    on_x1 = np.all(np.abs(d.nodes[d.conn[info[:, 2]]][:, :, 0] - 1.0) < 1e-12, axis=1)
    yz = {k: set(map(tuple, np.round(x[on_x1 & (kinds == k)][:, 1:], 10))) for k in (1, 5)}
    c1, c5 = 0.5 * 0.22540333, 0.5 * 0.3
    assert (c1, c1) in yz[1] and (1 - c1, 1 - c1) in yz[1]
    assert (c5, c5) in yz[5] and (1 - c5, 1 - c5) in yz[5]


def test_formulation_errors(oracle):
    d = M.halfspace_footing(1.0, 2, 1.0)
    P = oracle.Problem(d)
    with pytest.raises(ValueError):
        P.set_formulation(np.full(d.n_nodes, 4))
    P.set_formulation("dual_bm")
    P.set_halfspace(-3, 0.0, 1)
    with pytest.raises(RuntimeError, match="half-space"):
        P.assemble_staela(MU, NU)


def test_hbie_points(oracle):
    """HBIE points: xi of every element node moved by delta_hbie
    (src/build_data_at_collocation_points.f90:148-160) with the element's
    unit normal there (:368-376); the x = 1 face has normal +e1."""
    d = M.box((1.0, 1.0, 1.0), (1, 1, 1), split_faces=False)
    P = oracle.Problem(d)
    P.set_formulation("hbie", delta=0.3)
    x, info = P.colloc()
    nrm = P.colloc_normals()
    on_x1 = np.all(np.abs(d.nodes[d.conn[info[:, 2]]][:, :, 0] - 1.0) < 1e-12, axis=1)
    assert on_x1.sum() == 8
    assert np.allclose(nrm[on_x1], [1.0, 0.0, 0.0])
    assert np.allclose(x[on_x1][:, 0], 1.0)
    # xi -> xi (1 - delta): corners at 0.15 / 0.85 of the unit face, mid-edge
    # nodes at 0.5 and 0.15 / 0.85
    yz = set(map(tuple, np.round(x[on_x1][:, 1:], 12)))
    assert yz == {(0.15, 0.15), (0.85, 0.15), (0.85, 0.85), (0.15, 0.85), (0.5, 0.15), (0.85, 0.5), (0.5, 0.85),
                  (0.15, 0.5)}
