"""Oracle against the reference's closed-form known answers and the method's
identities (CPU only, small meshes)."""
import numpy as np
import pytest

from multifebe_gb300 import meshgen as M


@pytest.mark.parametrize("n,qsi,tol", [(1, 1e-6, 2e-5), (2, 1e-6, 2e-5), (2, 1e-10, 2e-9)])
def test_kat_confined_cube(oracle, n, qsi, tol):
    """docs/examples/ME-ST-EL-002: u1 = (1+nu)(1-2nu)/(E(1-nu)) P x1 = 0.8333 x1,
    u2 = u3 = 0, sigma11 = P, sigma22 = sigma33 = nu/(1-nu) P; linear, so any
    mesh reproduces it to quadrature accuracy."""
    d = M.cube_confined_kat(n)
    P = oracle.Problem(d, qsi_re=qsi)
    mat = M.elastic(1.0, 0.25)
    A, b = P.assemble_staela(mat["mu"], mat["nu"])
    x = oracle.lu_solve(A, b)
    u, t = P.solution(x)
    assert np.abs(u[:, 0] - (1.25 * 0.5 / 0.75) * d.nodes[:, 0]).max() < tol
    assert np.abs(u[:, 1:]).max() < tol
    # normal traction on the rollers: -1 on x=0, -1/3 and +1/3 on the lateral faces
    x0 = np.abs(d.nodes[:, 0]) < 1e-12
    inner = x0 & (d.nodes[:, 1] > 1e-6) & (d.nodes[:, 1] < 1 - 1e-6) & (d.nodes[:, 2] > 1e-6) & (d.nodes[:, 2] < 1 - 1e-6)
    if inner.any():
        assert np.abs(t[inner, 0] + 1.0).max() < 50 * tol


def _p_wave_column(mat, om, x, L=1.0, P=1.0):
    """docs/examples/ME-TH-EL-001: laterally constrained column loaded by a
    harmonic traction P on x = L, fixed normal displacement at x = 0:
    u1 = P sin(k x) / ((lambda + 2 mu) k cos(k L)), k = omega / c_p with the
    complex c_p = sqrt((lambda + 2 mu) / rho)."""
    lam2mu = mat["lambda"] + 2.0 * mat["mu"]
    k = om / np.sqrt(lam2mu / mat["rho"])
    return P * np.sin(k * x) / (lam2mu * k * np.cos(k * L))


@pytest.mark.parametrize("om,tol4", [(2.0, 2e-4), (5.0, 3e-3)])
def test_kat_harmonic_p_wave_column(oracle, om, tol4):
    """docs/examples/ME-TH-EL-001 (mu = 1, nu = 0.2, rho = 1, xi = 0.02, below
    and above the first resonance omega_1 = 2.57): the quad8 solution converges
    to the closed form (error 6.5e-4 -> 7.9e-5 at omega = 2, 8.4e-3 -> 1.3e-3
    at omega = 5 from 2x2 to 4x4 elements per face); lateral displacements
    vanish to the same order."""
    mat = M.viscoelastic(2.4, 0.2, 1.0, 0.02)
    errs = []
    for n in (2, 4):
        d = M.cube_confined_kat(n)
        P = oracle.Problem(d)
        A, b = P.assemble_harela(mat, om)
        u, _ = P.solution(oracle.lu_solve(A, b))
        ue = _p_wave_column(mat, om, d.nodes[:, 0])
        errs.append(np.abs(u[:, 0] - ue).max() / np.abs(ue).max())
        assert np.abs(u[:, 1:]).max() < errs[-1] * np.abs(ue).max()
    assert errs[1] < tol4 and errs[1] < errs[0] / 4, errs


INTERIOR = np.array([[0.5, 0.5, 0.5], [0.25, 0.3, 0.7], [0.9, 0.1, 0.5], [0.98, 0.5, 0.5],
                     [0.13, 0.77, 0.41], [0.62, 0.05, 0.88]])


def test_kat_internal_points_static(oracle):
    """Internal points of docs/examples/ME-ST-EL-002: u1 = 0.8333 x1 and the
    uniform stress sigma11 = P, sigma22 = sigma33 = nu/(1-nu) P from the HBIE
    kernels (d*, s*), down to points 0.02 from the boundary."""
    d = M.cube_confined_kat(2)
    P = oracle.Problem(d, qsi_re=1e-10)
    mat = M.elastic(1.0, 0.25)
    A, b = P.assemble_staela(mat["mu"], mat["nu"])
    u, t = P.solution(oracle.lu_solve(A, b))
    ui, si = P.internal_points(INTERIOR, u, t, mu=mat["mu"], nu=mat["nu"])
    assert np.abs(ui[:, 0] - (1.25 * 0.5 / 0.75) * INTERIOR[:, 0]).max() < 1e-9
    assert np.abs(ui[:, 1:]).max() < 1e-9
    assert np.abs(si - np.diag([1.0, 1.0 / 3.0, 1.0 / 3.0])).max() < 5e-8


def test_kat_internal_points_harmonic(oracle):
    """Internal points of docs/examples/ME-TH-EL-001: u1, sigma11 = P cos(kx) /
    cos(kL) and sigma22 = lambda / (lambda + 2 mu) sigma11 converge to the
    closed form from 2x2 to 4x4 elements per face."""
    mat = M.viscoelastic(2.4, 0.2, 1.0, 0.02)
    om = 2.0
    lam2mu = mat["lambda"] + 2.0 * mat["mu"]
    k = om / np.sqrt(lam2mu / mat["rho"])
    s11 = np.cos(k * INTERIOR[:, 0]) / np.cos(k)
    errs = []
    for n in (2, 4):
        d = M.cube_confined_kat(n)
        P = oracle.Problem(d)
        A, b = P.assemble_harela(mat, om)
        u, t = P.solution(oracle.lu_solve(A, b))
        ui, si = P.internal_points(INTERIOR, u, t, mat=mat, omega=om)
        ue = _p_wave_column(mat, om, INTERIOR[:, 0])
        errs.append([np.abs(ui[:, 0] - ue).max() / np.abs(ue).max(),
                     np.abs(si[:, 0, 0] - s11).max(),
                     np.abs(si[:, 1, 1] - mat["lambda"] / lam2mu * s11).max()])
    errs = np.array(errs)
    # points down to 0.02 from the boundary: stresses there carry most of the
    # discretisation error (1.6e-3 -> 7e-4 for sigma11)
    assert np.all(errs[1] < [1e-4, 1.5e-3, 1e-3]) and np.all(errs[1] < errs[0] / 2), errs


def test_internal_point_at_a_node_and_on_an_element(oracle):
    """At a boundary node: the node's displacement and zero stress; on an
    element away from its nodes: rejected."""
    d = M.cube_confined_kat(2)
    P = oracle.Problem(d)
    mat = M.elastic(1.0, 0.25)
    A, b = P.assemble_staela(mat["mu"], mat["nu"])
    u, t = P.solution(oracle.lu_solve(A, b))
    for s in (7, 20):
        ui, si = P.internal_points(d.nodes[s:s + 1], u, t, mu=mat["mu"], nu=mat["nu"])
        # the deck duplicates edge nodes (one per boundary); the last node at
        # the point, in node order, gives the value
        last = np.flatnonzero(np.linalg.norm(d.nodes - d.nodes[s], axis=1) < 1e-12).max()
        assert np.array_equal(ui[0], u[last]) and np.all(si == 0)
    e = d.conn[0]
    xm = 0.5 * (d.nodes[e[0]] + d.nodes[e[4]]) * 0.5 + 0.5 * (d.nodes[e[4]] + d.nodes[e[6]]) * 0.5
    with pytest.raises(ValueError):
        P.internal_points(xm[None, :], u, t, mu=mat["mu"], nu=mat["nu"])


def test_rigid_body_translation(oracle):
    """Closed surface, all tractions prescribed: A = H + C and a rigid
    translation is in its null space, sum over the u_k columns of each row = 0."""
    d = M.box((1, 1, 1), (2, 2, 2))
    d.ctype[:] = 1
    P = oracle.Problem(d)
    mat = M.elastic(1.0, 0.25)
    A, _ = P.assemble_staela(mat["mu"], mat["nu"])
    dof, _ = P.dof_map()
    for k in range(3):
        s = A[:, dof[:, k]].sum(axis=1)
        assert np.abs(s).max() < 1e-5 * np.abs(A).max()


def test_harmonic_tends_to_static(oracle):
    """omega -> 0: the time-harmonic kernels converge linearly to the static ones."""
    d = M.cube_clamped_top_traction(2)
    P = oracle.Problem(d)
    m = M.viscoelastic(1.0, 0.25, 1.0, 0.0)
    A0, b0 = P.assemble_staela(m["mu_real"], 0.25)
    diffs = []
    for om in (1e-4, 1e-5):
        A1, b1 = P.assemble_harela(m, om)
        diffs.append(np.abs(A1 - A0).max() / np.abs(A0).max())
    assert diffs[1] < 2e-6
    assert 8 < diffs[0] / diffs[1] < 12


def test_pair_classes_cover_all_pairs(oracle):
    d = M.cube_confined_kat(2)
    P = oracle.Problem(d)
    mat = M.elastic(1.0, 0.25)
    P.assemble_staela(mat["mu"], mat["nu"])
    x, info = P.colloc()
    npairs = x.shape[0] * d.n_elements
    st = P.stats
    assert st[0] + st[1] + st[2] == npairs
    # every (node, element) incidence is singular once: nodal SBIE points with
    # each element around them, MCA points with the element they sit in
    assert st[2] == 8 * d.n_elements
