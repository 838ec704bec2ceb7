"""Internal points on the device (mfbem_internal_points_{staela,harela}) against
the oracle's restatement of calculate_internal_points_mechanics_bem_* and the
closed forms of docs/examples/ME-ST-EL-002 and ME-TH-EL-001. Both sides get
the same nodal solution, so the comparison isolates the internal-point step.

Tolerances (max-norm relative to the largest value): displacement and stress
<= 1e-11 against the oracle (FP64 on both sides; FMA contraction and the
device's transcendental functions); <= 1e-9 where quasi-singular subdivision
dominates (thin slab)."""
import numpy as np
import pytest

from multifebe_gb300 import MfbemError, BemRegion, meshgen as M, _abi
from test_oracle_kat import INTERIOR, _p_wave_column

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_static_internal_points(oracle):
    d = M.cube_confined_kat(2)
    mat = M.elastic(1.0, 0.25)
    P = oracle.Problem(d, qsi_re=1e-10)
    A, b = P.assemble_staela(mat["mu"], mat["nu"])
    u, t = P.solution(oracle.lu_solve(A, b))
    R = BemRegion(d, qsi_relative_error=1e-10)
    ui, si = R.internal_points(INTERIOR, u, t, mu=mat["mu"], nu=mat["nu"])
    uo, so = P.internal_points(INTERIOR, u, t, mu=mat["mu"], nu=mat["nu"])
    R.close()
    assert rel(ui, uo) < 1e-11 and rel(si, so) < 1e-11, (rel(ui, uo), rel(si, so))
    assert np.abs(ui[:, 0] - (1.25 * 0.5 / 0.75) * INTERIOR[:, 0]).max() < 1e-9
    assert np.abs(si - np.diag([1.0, 1.0 / 3.0, 1.0 / 3.0])).max() < 5e-8


@pytest.mark.parametrize("om", [2.0, 5.0])
def test_harmonic_internal_points(oracle, om):
    d = M.cube_confined_kat(4)
    mat = M.viscoelastic(2.4, 0.2, 1.0, 0.02)
    P = oracle.Problem(d)
    A, b = P.assemble_harela(mat, om)
    u, t = P.solution(oracle.lu_solve(A, b))
    R = BemRegion(d)
    ui, si = R.internal_points(INTERIOR, u, t, mat=mat, omega=om)
    uo, so = P.internal_points(INTERIOR, u, t, mat=mat, omega=om)
    R.close()
    assert rel(ui, uo) < 1e-11 and rel(si, so) < 1e-11, (rel(ui, uo), rel(si, so))
    ue = _p_wave_column(mat, om, INTERIOR[:, 0])
    assert np.abs(ui[:, 0] - ue).max() / np.abs(ue).max() < (3e-3 if om > 3 else 1e-4)


def test_thin_slab_quasi_singular_internal_points(oracle):
    """Points inside a slab 0.02 thick: every pair with the nearby faces is
    quasi-singular (subdivision trees for both the SBIE and the HBIE)."""
    d = M.slab(4, 1)
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.02)
    om = float(M.omega_from_a0([0.5], mat)[0])
    P = oracle.Problem(d)
    A, b = P.assemble_harela(mat, om)
    u, t = P.solution(oracle.lu_solve(A, b))
    rng = np.random.default_rng(4)
    xy = rng.uniform(0.1, 0.9, (12, 2))
    z = np.array([0.01, 0.004, 0.016] * 4)
    xip = np.column_stack([xy, z])
    R = BemRegion(d)
    ui, si = R.internal_points(xip, u, t, mat=mat, omega=om)
    uo, so = P.internal_points(xip, u, t, mat=mat, omega=om)
    R.close()
    assert rel(ui, uo) < 1e-9 and rel(si, so) < 1e-9, (rel(ui, uo), rel(si, so))


def test_internal_points_at_nodes_and_on_elements():
    d = M.cube_confined_kat(2)
    mat = M.elastic(1.0, 0.25)
    R = BemRegion(d)
    rng = np.random.default_rng(1)
    u = rng.normal(size=(d.n_nodes, 3))
    t = rng.normal(size=(d.n_nodes, 3))
    for s in (7, 20):
        ui, si = R.internal_points(d.nodes[s:s + 1], u, t, mu=mat["mu"], nu=mat["nu"])
        last = np.flatnonzero(np.linalg.norm(d.nodes - d.nodes[s], axis=1) < 1e-12).max()
        assert np.array_equal(ui[0], u[last]) and np.all(si == 0)
    e = d.conn[0]
    xm = 0.25 * (d.nodes[e[0]] + d.nodes[e[4]]) + 0.25 * (d.nodes[e[4]] + d.nodes[e[6]])
    with pytest.raises(MfbemError) as ex:
        R.internal_points(np.vstack([INTERIOR[:1], xm[None, :]]), u, t, mu=mat["mu"], nu=mat["nu"])
    assert ex.value.code == _abi.MFBEM_EUNSUPPORTED
    R.close()
