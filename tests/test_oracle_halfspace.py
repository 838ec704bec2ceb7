"""The oracle's half-space complementary kernel and builder rules.

Pins the restatement of fbem_bem_staela3d_hsc_sbie
(lib/fbem/src/bem_staela3d.f90:7438-7563) against closed forms of elastostatics
for the half-space x3 >= 0 with a traction-free surface, whose complete
fundamental solution is Kelvin's plus the complementary part (Mindlin):
  - the complete traction kernel vanishes on the free surface;
  - Boussinesq (normal surface load) and Cerruti (tangential surface load)
    surface displacements;
  - Betti reciprocity of the complete displacement kernel;
  - Love's settlement of the centre of a uniformly loaded square, through the
    builder (complementary kernel on every pair, free term doubled on the
    surface, build_lse_mechanics_bem_staela.f90:502-513, 861-875).
"""
import numpy as np
import pytest

from multifebe_gb300 import meshgen as M

MU, NU = 0.4, 0.25


def kelvin(xi, x, n):
    rv = np.asarray(x, float) - np.asarray(xi, float)
    r = np.linalg.norm(rv)
    dr = rv / r
    d = np.eye(3)
    u = ((3 - 4 * NU) * d + np.outer(dr, dr)) / (16 * np.pi * MU * (1 - NU) * r)
    t = -(dr @ n * ((1 - 2 * NU) * d + 3 * np.outer(dr, dr)) + (1 - 2 * NU) * (np.outer(n, dr) - np.outer(dr, n))) \
        / (8 * np.pi * (1 - NU) * r ** 2)
    return u, t


def complete(oracle, xi, x, n=(0.0, 0.0, -1.0)):
    uk, tk = kelvin(xi, x, np.asarray(n))
    uh, th = oracle.hsc_point(MU, NU, 0.0, xi, x, n)
    return uk + uh, tk + th


def test_traction_free_surface(oracle):
    rng = np.random.default_rng(1)
    for _ in range(300):
        xi = np.array([*rng.uniform(-1, 1, 2), rng.uniform(1e-3, 3)])
        x = np.array([*rng.uniform(-3, 3, 2), 0.0])
        uk, tk = kelvin(xi, x, np.array([0.0, 0.0, -1.0]))
        _, t = complete(oracle, xi, x)
        assert np.abs(t).max() <= 1e-14 * np.abs(tk).max()


def test_boussinesq_and_cerruti_on_the_surface(oracle):
    xi = np.zeros(3)
    for x1, x2 in ((0.7, 0.3), (-0.2, 1.1), (2.0, 0.0)):
        x = np.array([x1, x2, 0.0])
        r = np.hypot(x1, x2)
        u, _ = complete(oracle, xi, x)
        # normal load: w = (1 - nu) / (2 pi mu r), u_r = -(1 - 2 nu) / (4 pi mu r)
        assert u[2, 2] == pytest.approx((1 - NU) / (2 * np.pi * MU * r), rel=1e-13)
        ur = (u[2, 0] * x1 + u[2, 1] * x2) / r
        assert ur == pytest.approx(-(1 - 2 * NU) / (4 * np.pi * MU * r), rel=1e-13)
        # tangential load along x1: u1 = (1 / (4 pi mu r)) (1 + x1^2 / r^2 + (1 - 2 nu)(1 - x1^2 / r^2)),
        # u2 = (1 / (4 pi mu r)) (x1 x2 / r^2)(1 - (1 - 2 nu)), u3 = (1 - 2 nu) x1 / (4 pi mu r^2)
        c = 1.0 / (4 * np.pi * MU * r)
        assert u[0, 0] == pytest.approx(c * (1 + x1 ** 2 / r ** 2 + (1 - 2 * NU) * (1 - x1 ** 2 / r ** 2)), rel=1e-13)
        assert u[0, 1] == pytest.approx(c * x1 * x2 / r ** 2 * (1 - (1 - 2 * NU)), rel=1e-12, abs=1e-15)
        assert u[0, 2] == pytest.approx((1 - 2 * NU) * x1 / (4 * np.pi * MU * r ** 2), rel=1e-13, abs=1e-15)


def test_reciprocity(oracle):
    """u_lk(x; x_i) = u_kl(x_i; x) for the complete kernel (Betti)."""
    rng = np.random.default_rng(2)
    for _ in range(100):
        a = np.array([*rng.uniform(-1, 1, 2), rng.uniform(0.01, 2)])
        b = np.array([*rng.uniform(-1, 1, 2), rng.uniform(0.01, 2)])
        uab, _ = complete(oracle, a, b)
        uba, _ = complete(oracle, b, a)
        assert np.abs(uab - uba.T).max() <= 1e-13 * np.abs(uab).max()


def test_points_outside_the_half_space_are_rejected(oracle):
    with pytest.raises(ValueError):
        oracle.hsc_point(MU, NU, 0.0, [0.0, 0.0, -0.1], [1.0, 0.0, 0.0], [0.0, 0.0, -1.0])


@pytest.mark.parametrize("n", [4, 6])
def test_love_loaded_square(oracle, n):
    """Centre settlement of a uniformly loaded square through the static
    builder: Love's closed form to the quadrature accuracy (the collocation
    points lie on the free surface, where H reduces to the doubled free term)."""
    d = M.halfspace_footing(1.0, n, 1.0)
    mat = M.elastic(1.0, 0.25)
    P = oracle.Problem(d)
    P.set_halfspace(-3, 0.0, 1)
    A, b = P.assemble_staela(mat["mu"], mat["nu"])
    u, _ = P.solution(oracle.lu_solve(A, b))
    c = np.argmin(np.linalg.norm(d.nodes, axis=1))
    w = M.love_square_centre(1.0, 1.0, 1.0, 0.25)
    assert abs(u[c, 2] - w) <= 1e-8 * w
    assert np.abs(u[c, :2]).max() <= 1e-12 * w
    # every complementary pair of a surface mesh is singular or regular, and the
    # singular ones are the full-space singular pairs
    assert P.stats[7] == P.stats[2]


def test_free_term_doubling_on_the_surface_harmonic(oracle):
    """The harmonic builder applies the doubling rule alone: A changes by the
    free terms of the surface points (1/2 I at nodal points of a flat surface)."""
    d = M.halfspace_footing(1.0, 3, 1.0)
    mat = M.viscoelastic(1.0, 0.25, 1.0, 0.05)
    w = float(M.omega_from_a0([0.7], mat)[0])
    P0 = oracle.Problem(d)
    A0, b0 = P0.assemble_harela(mat, w)
    P1 = oracle.Problem(d)
    P1.set_halfspace(-3, 0.0, 1)
    A1, b1 = P1.assemble_harela(mat, w)
    D = A1 - A0
    dof, _ = P1.dof_map()
    x, info = P1.colloc()
    interior = [int(s) for s, k in zip(info[:, 0], info[:, 1]) if k == 0]
    for s in interior:
        blk = D[np.ix_(dof[s], dof[s])]
        assert np.abs(blk - 0.5 * np.eye(3)).max() <= 1e-14
    assert np.abs(b1 - b0).max() == 0.0  # all tractions prescribed: b carries g t only


def test_static_kernel_needs_the_x3_normal(oracle):
    d = M.halfspace_footing(1.0, 2, 1.0)
    P = oracle.Problem(d)
    P.set_halfspace(3, 0.0, 1)
    with pytest.raises(RuntimeError, match="n = -3"):
        P.assemble_staela(0.4, 0.25)


def test_complementary_stress_from_the_differentiated_displacement(oracle):
    """The Cartesian complementary u* differentiated in x (jets) gives the
    closed-form complementary stress of hsc_sbie (bem_staela3d.f90:7438-7563)
    used by the builder: the basis of the d*, s* kernels of hsc_hbie."""
    mu, nu = 0.4, 0.25
    rng = np.random.default_rng(1)
    worst = 0.0
    for _ in range(20):
        xi = rng.uniform([-1, -1, 0.05], [1, 1, 1.5])
        x = rng.uniform([-1, -1, 0.0], [1, 1, 1.5])
        sig = oracle.hsc_sigma_ad(mu, nu, 0.0, xi, x)
        for j in range(3):
            n = np.zeros(3)
            n[j] = 1.0
            _, t = oracle.hsc_point(mu, nu, 0.0, xi, x, n)
            worst = max(worst, np.abs(t - sig[:, :, j]).max() / np.abs(sig).max())
    assert worst < 1e-13, worst


def test_internal_stresses_under_a_loaded_square(oracle):
    """Static internal points of a half-space region (the complementary
    kernels hsc_sbie_auto / hsc_hbie_auto, calculate_internal_points_
    mechanics_static.f90:288-310,401-418): the vertical stress below the
    centre of a uniformly loaded square 2a x 2a is Holl's closed form
    -(2p/pi) [atan(a^2 / (z R)) + 2 a^2 z / (R (a^2 + z^2))], R^2 = 2a^2 + z^2,
    to the quadrature tolerance; the shear stresses vanish on the axis."""
    a, p = 1.0, 1.0
    mat = M.elastic(1.0, 0.25)
    d = M.halfspace_footing(a, 4, p)
    P = oracle.Problem(d)
    P.set_halfspace(-3, 0.0, 1)
    u, t = P.solution(oracle.lu_solve(*P.assemble_staela(mat["mu"], mat["nu"])))
    zs = np.array([0.25, 0.5, 1.0, 2.0])
    xip = np.stack([np.zeros(4), np.zeros(4), zs], 1)
    ui, si = P.internal_points(xip, u, t, mu=mat["mu"], nu=mat["nu"])
    R = np.sqrt(2 * a * a + zs ** 2)
    holl = -(2 * p / np.pi) * (np.arctan(a * a / (zs * R)) + (a * a * zs / R) * (2.0 / (a * a + zs ** 2)))
    assert np.abs(si[:, 2, 2] - holl).max() < 1e-6 * np.abs(holl).max()
    assert np.abs(si[:, 0, 2]).max() < 1e-12 and np.abs(si[:, 1, 2]).max() < 1e-12
    assert np.all(np.diff(ui[:, 2]) < 0)
    with pytest.raises(RuntimeError, match="outside"):
        P.internal_points(np.array([[0.0, 0.0, -0.1]]), u, t, mu=mat["mu"], nu=mat["nu"])
