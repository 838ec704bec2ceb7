"""Half-space regions on the device against the oracle, through the C-ABI.

mfbem_set_halfspace(-3, 0, 1): the static builder adds the complementary
kernel of Mindlin's solution (classified on the images of the collocation
points, fbem_bem_staela3d_hsc_sbie_auto, lib/fbem/src/bem_staela3d.f90:9047-9118)
to every pair and doubles the free term of points on the free surface
(src/build_lse_mechanics_bem_staela.f90:502-513); the harmonic builder doubles
the free term only. Meshes:
  footing    loaded square on the surface (singular complementary pairs)
  excavation open box cut into the surface, rim nodes SBIE-MCA just below it
             (adaptive complementary pairs)
  cavity     closed cube buried 0.02 below the surface (adaptive
             complementary pairs through the thin ligament)
Tolerances as the full-space parity: A, b <= 1e-11 (max-norm relative), pair
and point counts identical; Love's closed form for the footing's centre.
"""
import ctypes

import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, BemRegion, MfbemError
from multifebe_gb300 import _abi

pytestmark = pytest.mark.gpu

CASES = [("footing", lambda: M.halfspace_footing(1.0, 6, 1.0)),
         ("excavation", lambda: M.halfspace_excavation(0.5, 0.5, 3)),
         ("cavity", lambda: M.halfspace_cavity(0.25, 0.02, 3))]


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def hs_counts(R):
    L = _abi.load()
    L.mfbem_internal_hs_counts.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    out = np.zeros(7, dtype=np.int64)
    _abi.check(L.mfbem_internal_hs_counts(R._h, out.ctypes.data))
    return out


@pytest.mark.parametrize("name,mk", CASES, ids=[c[0] for c in CASES])
def test_halfspace_staela_matches_oracle(oracle, name, mk):
    d = mk()
    mat = M.elastic(1.0, 0.25)
    P = oracle.Problem(d)
    P.set_halfspace(-3, 0.0, 1)
    Ao, bo = P.assemble_staela(mat["mu"], mat["nu"])
    R = BemRegion(d)
    R.set_halfspace(-3, 0.0, 1)
    A, b = R.build_lse_staela(mat["mu"], mat["nu"])
    c = hs_counts(R)
    print(name, "complementary pairs reg/adp/sing", c[:3], "oracle adp/sing", P.stats[6:8], "A", rel(A, Ao),
          "b", rel(b, bo))
    assert (c[1], c[2]) == (P.stats[6], P.stats[7])
    assert rel(A, Ao) < 1e-11 and rel(b, bo) < 1e-11
    # the full-space system of the same mesh differs (the kernel is really added)
    R0 = BemRegion(d)
    A0, _ = R0.build_lse_staela(mat["mu"], mat["nu"])
    assert rel(A0, A) > 1e-3
    R0.close()
    R.close()


def test_love_square_through_the_device_solver():
    d = M.halfspace_footing(1.0, 6, 1.0)
    mat = M.elastic(1.0, 0.25)
    R = BemRegion(d)
    R.set_halfspace(-3, 0.0, 1)
    for precision in ("plain", "mixed"):
        u, _ = R.solution(R.solve_staela(mat["mu"], mat["nu"], precision=precision))
        c = np.argmin(np.linalg.norm(d.nodes, axis=1))
        w = M.love_square_centre(1.0, 1.0, 1.0, 0.25)
        assert abs(u[c, 2] - w) <= 1e-8 * w, (precision, u[c, 2], w)
    R.close()


def test_halfspace_harela_free_term_rule(oracle):
    d = M.halfspace_footing(1.0, 4, 1.0)
    mat = M.viscoelastic(1.0, 0.3, 1.0, 0.05)
    P = oracle.Problem(d)
    P.set_halfspace(-3, 0.0, 1)
    R = BemRegion(d)
    R.set_halfspace(-3, 0.0, 1)
    for a0 in (0.3, 1.2):
        om = float(M.omega_from_a0(a0, mat))
        Ao, bo = P.assemble_harela(mat, om)
        A, b = R.build_lse_harela(mat, om)
        assert rel(A, Ao) < 1e-11 and rel(b, bo) < 1e-11
    R.close()


def test_halfspace_geometry_errors():
    mat = M.elastic(1.0, 0.25)
    # a cavity reaching above the surface
    d = M.halfspace_cavity(0.25, -0.1, 2)
    R = BemRegion(d)
    R.set_halfspace(-3, 0.0, 1)
    with pytest.raises(MfbemError) as e:
        R.build_lse_staela(mat["mu"], mat["nu"])
    assert e.value.code == _abi.MFBEM_EGEOMETRY
    # static kernel only for n = -3; bc = 0 is not available
    R.set_halfspace(3, 0.0, 1)
    with pytest.raises(MfbemError) as e:
        R.build_lse_staela(mat["mu"], mat["nu"])
    assert e.value.code == _abi.MFBEM_EUNSUPPORTED
    with pytest.raises(MfbemError) as e:
        R.set_halfspace(-3, 0.0, 0)
    assert e.value.code == _abi.MFBEM_EUNSUPPORTED
    # back to the full space: assembles again
    R.set_halfspace(0, 0.0, 1)
    R.build_lse_staela(mat["mu"], mat["nu"])
    R.close()


def test_static_internal_points_of_a_half_space(oracle):
    """Static internal points of a half-space region: the complementary
    kernels (hsc_sbie_auto, hsc_hbie_auto) added from the points' images
    (calculate_internal_points_mechanics_static.f90:288-310,401-418), device
    against the oracle (<= 1e-10) and Holl's vertical stress below the centre
    of the loaded square (quadrature tolerance); a point above the free surface
    is refused."""
    a, p = 1.0, 1.0
    d = M.halfspace_footing(a, 4, p)
    mat = M.elastic(1.0, 0.25)
    P = oracle.Problem(d)
    P.set_halfspace(-3, 0.0, 1)
    R = BemRegion(d)
    R.set_halfspace(-3, 0.0, 1)
    u, t = R.solution(R.solve_staela(mat["mu"], mat["nu"], precision="plain"))
    zs = np.array([0.25, 0.5, 1.0, 2.0])
    xip = np.concatenate([np.stack([np.zeros(4), np.zeros(4), zs], 1),
                          np.array([[0.7, -0.4, 0.3], [1.5, 1.2, 0.05], [-2.0, 0.5, 1.0]])])
    ud, sd = R.internal_points(xip, u, t, mu=mat["mu"], nu=mat["nu"])
    uo, so = P.internal_points(xip, u, t, mu=mat["mu"], nu=mat["nu"])
    print("u", rel(ud, uo), "sigma", rel(sd, so))
    assert rel(ud, uo) <= 1e-10 and rel(sd, so) <= 1e-10
    R2 = np.sqrt(2 * a * a + zs ** 2)
    holl = -(2 * p / np.pi) * (np.arctan(a * a / (zs * R2)) + (a * a * zs / R2) * (2.0 / (a * a + zs ** 2)))
    assert np.abs(sd[:4, 2, 2] - holl).max() < 1e-6 * np.abs(holl).max()
    with pytest.raises(MfbemError) as e:
        R.internal_points(np.array([[0.0, 0.0, -0.1]]), u, t, mu=mat["mu"], nu=mat["nu"])
    assert e.value.code == _abi.MFBEM_EGEOMETRY
    R.close()
