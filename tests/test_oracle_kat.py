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
