"""Crack-like boundaries (dual BEM) in the oracle's builders.

A crack-like boundary (src/read_boundaries.f90:105) has two faces on one
mesh: face 1 with the elements' normal, face 2 with the reversed one. Every
node of it carries both faces' unknowns and two equations at the same
collocation point (moved into the element by delta_sbie_mca): the SBIE with
the free term 1/2 on both faces' displacements and the HBIE with 1/2 on both
faces' tractions (build_lse_mechanics_bem_staela.f90:199-213, the two
assemble_bem_staela_equation calls of :519-529 and :1010-1020;
build_lse_mechanics_bem_harela.f90:344-360). Face 2 takes the integrals of
the reversed element: h- = -h+, g- = g+, m- = -m+, l- = l+.

Known answers: Sneddon's opening of a pressurised penny crack in a full
space and the sliding of a sheared one (Kassir and Sih), to the error of
quadratic elements without crack-tip elements (a few parts in 1e3).
"""
import numpy as np
import pytest

from multifebe_gb300 import meshgen as M

E, NU = 1.0, 0.25


def crack_problem(oracle, m, k, load):
    d, (ce, ct2, cv2) = M.penny_crack(1.0, m, k, 1.0)
    d.cvalue[:] = 0.0
    cv2[:] = 0.0
    d.cvalue[:, load] = -1.0
    cv2[:, load] = 1.0
    P = oracle.Problem(d)
    P.set_crack(ce, ct2, cv2)
    return d, P


def faces(oracle, d, P):
    mat = M.elastic(E, NU)
    x = oracle.lu_solve(*P.assemble_staela(mat["mu"], mat["nu"]))
    return P.solution_faces(x)


@pytest.mark.parametrize("m,k", [(2, 2), (2, 3)])
def test_sneddon_pressurised_penny_crack(oracle, m, k):
    d, P = crack_problem(oracle, m, k, 2)
    u1, t1, u2, t2 = faces(oracle, d, P)
    r = np.linalg.norm(d.nodes[:, :2], axis=1)
    ex = M.sneddon_opening(r, 1.0, 1.0, E, NU)
    cod = u2[:, 2] - u1[:, 2]
    c = np.argmin(r)
    assert abs(cod[c] - ex[c]) < 2e-3 * ex[c], (cod[c], ex[c])
    inner = r < 0.6
    assert np.abs(cod[inner] - ex[inner]).max() < 4e-3 * ex[c]
    # mirror symmetry about the crack plane: opening antisymmetric, in-plane
    # displacements equal on both faces
    assert np.abs(u1[:, 2] + u2[:, 2]).max() < 1e-12 * ex[c]
    assert np.abs(u1[:, :2] - u2[:, :2]).max() < 1e-12 * ex[c]
    # both faces' tractions are the prescribed ones
    assert np.allclose(t1[:, 2], -1.0) and np.allclose(t2[:, 2], 1.0)


def test_sheared_penny_crack(oracle):
    d, P = crack_problem(oracle, 2, 3, 0)
    u1, _, u2, _ = faces(oracle, d, P)
    r = np.linalg.norm(d.nodes[:, :2], axis=1)
    ex = 16.0 * (1.0 - NU ** 2) / (np.pi * (2.0 - NU) * E) * np.sqrt(np.maximum(1.0 - r * r, 0.0))
    slip = u2[:, 0] - u1[:, 0]
    c = np.argmin(r)
    inner = r < 0.6
    assert abs(slip[c] - ex[c]) < 1e-3 * ex[c]
    assert np.abs(slip[inner] - ex[inner]).max() < 4e-3 * ex[c]
    # no opening under shear; the transverse slip is discretisation error only
    assert np.abs(u2[:, 2] - u1[:, 2]).max() < 1e-12 * ex[c]
    assert np.abs(u2[:, 1] - u1[:, 1]).max() < 4e-3 * ex[c]


def test_crack_dof_layout(oracle):
    """Both faces' unknowns of a crack node interleave: component c of face 1
    at r + 2c, of face 2 at r + 2c + 1 (six rows per node)."""
    d, P = crack_problem(oracle, 2, 1, 2)
    assert P.n == 6 * d.n_nodes
    d2 = P.dof2_map()
    assert sorted(d2.ravel()) == list(range(1, 6 * d.n_nodes, 2))
    assert np.all(d2[:, 1] - d2[:, 0] == 2) and np.all(d2[:, 2] - d2[:, 1] == 2)


def test_crack_harmonic_static_limit(oracle):
    d, P = crack_problem(oracle, 2, 2, 2)
    ms = M.elastic(E, NU)
    As, bs = P.assemble_staela(ms["mu"], ms["nu"])
    mat = M.viscoelastic(E, NU, 1.0, 0.0)
    errs = []
    for om in (1e-2, 1e-3):
        Ah, bh = P.assemble_harela(mat, om)
        errs.append(np.abs(Ah - As).max() / np.abs(As).max())
        assert np.abs(bh - bs).max() < 1e-14
    # the dynamic part of the kernels is O(omega^2)
    assert errs[0] < 1e-5 and 80 < errs[0] / errs[1] < 120, errs


def test_crack_errors(oracle):
    d, (ce, ct2, cv2) = M.penny_crack(1.0, 2, 1, 1.0)
    P = oracle.Problem(d)
    half = ce.copy()
    half[::2] = False  # crack nodes shared with ordinary elements
    with pytest.raises(ValueError, match="crack node"):
        P.set_crack(half, ct2, cv2)
    P.set_crack(ce, ct2, cv2)
    P.set_halfspace(-3, -1.0, 1)
    with pytest.raises(RuntimeError, match="half-space"):
        P.assemble_staela(0.4, 0.25)


def test_internal_points_of_a_cracked_region(oracle):
    """Internal points with both faces' solution (calculate_internal_points_
    mechanics_static.f90:320-354,431-465): approaching the crack from either
    side the displacement tends to that face's, sigma_zz to the pressure, and
    the field is mirror-symmetric; face 1 alone gives nothing of the sort."""
    d, P = crack_problem(oracle, 2, 3, 2)
    mat = M.elastic(E, NU)
    x = oracle.lu_solve(*P.assemble_staela(mat["mu"], mat["nu"]))
    u1, t1, u2, t2 = P.solution_faces(x)
    c = np.argmin(np.linalg.norm(d.nodes, axis=1))
    z = np.array([0.02, 0.3, 1.0])
    xp = np.stack([np.zeros(3), np.zeros(3), z], 1)
    up, sp = P.internal_points(xp, u1, t1, mu=mat["mu"], nu=mat["nu"], u2=u2, t2=t2)
    um, sm = P.internal_points(-xp, u1, t1, mu=mat["mu"], nu=mat["nu"], u2=u2, t2=t2)
    assert abs(up[0, 2] - u2[c, 2]) < 0.02 * u2[c, 2] and abs(um[0, 2] - u1[c, 2]) < 0.02 * u2[c, 2]
    assert abs(sp[0, 2, 2] + 1.0) < 0.03
    assert np.allclose(up[:, 2], -um[:, 2], rtol=1e-12, atol=0) and np.allclose(sp[:, 2, 2], sm[:, 2, 2], rtol=1e-12)
    assert np.abs(sp[:, :2, 2]).max() < 1e-12 and np.abs(up[:, :2]).max() < 1e-12
    assert np.all(np.diff(up[:, 2]) < 0)  # the opening decays away from the crack
    u0, _ = P.internal_points(xp[:1], u1, t1, mu=mat["mu"], nu=mat["nu"])
    assert abs(u0[0, 2] - u2[c, 2]) > 0.5 * u2[c, 2]
    # a point at a crack node has no single value
    with pytest.raises(ValueError):
        P.internal_points(d.nodes[c:c + 1], u1, t1, mu=mat["mu"], nu=mat["nu"], u2=u2, t2=t2)
