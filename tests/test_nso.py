"""Nodal-solution export (*.nso): the Fortran edit descriptors of the export
settings (E for sci_*, EN for eng_*, I for integers) on known values, the
record layout and export order of export_solution_mechanics_*_nso for an
ordinary boundary of a BE region, and a write -> read round trip of a
solution at sci_double (16 significant digits)."""
import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, nsoio


@pytest.mark.parametrize("kind,w,d,e,v,out", [
    ("E", 25, 16, 3, 1.0, "  0.1000000000000000E+001"),
    ("E", 25, 16, 3, -123.456, " -0.1234560000000000E+003"),
    ("E", 25, 16, 3, 0.0, "  0.0000000000000000E+000"),
    ("E", 25, 16, 3, 2.5e-7, "  0.2500000000000000E-006"),
    ("E", 16, 8, 2, 0.99999999999, "  0.10000000E+01"),
    ("E", 11, 3, 2, -0.000123456, " -0.123E-03"),
    ("N", 18, 8, 2, 1234.5, "    1.23450000E+03"),
    ("N", 18, 8, 2, 0.000123, "  123.00000000E-06"),
    ("N", 18, 8, 2, 0.0, "    0.00000000E+00"),
    ("N", 18, 8, 2, -12.5, "  -12.50000000E+00"),
    ("N", 18, 8, 2, 999.9999999999, "    1.00000000E+03"),
    ("N", 13, 3, 2, 0.1, "  100.000E-03"),
    ("N", 27, 16, 3, 3.0, "    3.0000000000000000E+000"),
    ("I", 5, 0, 1, 42, "   42"),
    ("I", 3, 0, 1, 12345, "***"),
])
def test_edit_descriptors(kind, w, d, e, v, out):
    assert nsoio.fortran_format(kind, w, d, e, v) == out


def test_records_order_and_round_trip(tmp_path):
    d = M.cube_confined_kat(2)  # six boundaries with their own nodes
    rng = np.random.default_rng(4)
    u = rng.standard_normal((d.n_nodes, 3)) + 1j * rng.standard_normal((d.n_nodes, 3))
    t = rng.standard_normal((d.n_nodes, 3)) + 1j * rng.standard_normal((d.n_nodes, 3))
    p = tmp_path / "kat.nso"
    order = nsoio.write_nso(p, d, u, t, omega=2.5, kf=3, real="sci_double")
    text = p.read_text().splitlines()
    assert text[0] == "# Program      : multifebe" and text[2] == "# File_format  : nso"
    assert text[-len(order) - 1].startswith("#_") and text[-len(order) - 1].endswith("C44")
    R = nsoio.read_nso(p)
    assert R.shape == (len(order), 12 + 24)
    # every node once (one boundary per node), boundaries in increasing id
    assert sorted(s for s, _ in order) == list(range(d.n_nodes))
    assert list(R[:, 5]) == sorted(R[:, 5])
    assert np.all(R[:, 0] == 3) and np.all(R[:, 1] == 2.5)
    assert np.all(R[:, 2:5] == [1, 1, 2]) and np.all(R[:, 6:8] == [1, 1])
    idx = [s for s, _ in order]
    assert np.array_equal(R[:, 8].astype(int), np.array(idx) + 1)
    assert np.allclose(R[:, 9:12], d.nodes[idx], rtol=0, atol=1e-16)
    vals = np.concatenate([u[idx], t[idx]], axis=1)
    got = R[:, 12:24:2] + 1j * R[:, 13:24:2]
    assert np.abs(got - vals).max() / np.abs(vals).max() < 1e-15
    assert np.all(R[:, 24:] == 0.0)
    # static file: one column per variable, C1 = C2 = 0, the default EN18.8E2
    q = tmp_path / "kat_static.nso"
    nsoio.write_nso(q, d, u.real, t.real)
    S = nsoio.read_nso(q)
    assert S.shape == (len(order), 18) and np.all(S[:, :2] == 0)
    assert np.abs(S[:, 12:] - np.concatenate([u.real[idx], t.real[idx]], 1)).max() < 1e-8
    # polar notation: |z| and arg z
    r = tmp_path / "kat_polar.nso"
    nsoio.write_nso(r, d, u, t, omega=1.0, real="sci_double", complex_notation=2 - 1)
    P = nsoio.read_nso(r)
    z = P[:, 12] * np.exp(1j * P[:, 13])
    assert np.abs(z - u[idx, 0]).max() < 1e-14
