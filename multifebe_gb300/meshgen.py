"""Input decks for the collocation-BEM path: quad8 surface meshes and nodal
boundary conditions, in the form MultiFEBE's input pipeline hands to its region
builders (one BE region, ordinary boundaries, continuous quad8 elements).

A deck is what a MultiFEBE ``.dat`` + ``.msh`` pair describes for this path:
node coordinates, element connectivity (quad8 node order of
lib/fbem/src/resources_shape_functions/xi_quad8.rc, element normal T1 x T2
pointing out of the region), and per node and direction the boundary condition
type (0: displacement known, 1: traction known) with its value
(``[conditions over nodes]``, docs/manual/manual.tex:2010-2036).

Element order is face by face and row by row; DOF numbering follows from it
(first appearance of a node over elements, see
src/build_auxiliary_variables_mechanics_static.f90:60-140).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Deck:
    name: str
    nodes: np.ndarray          # (nn, 3) float64
    conn: np.ndarray           # (ne, 8) int32, 0-based
    ctype: np.ndarray          # (nn, 3) int32: 0 displacement known, 1 traction known
    cvalue: np.ndarray         # (nn, 3) complex128
    boundary_of_element: np.ndarray = field(default=None)  # (ne,) face id (informational)

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def n_elements(self) -> int:
        return int(self.conn.shape[0])

    @property
    def n_dof(self) -> int:
        return 3 * self.n_nodes


# faces of an axis-aligned box: (axis, side, u, v) with u x v the outward normal
_BOX_FACES = [
    (2, 0, 1, 0),  # z = 0, normal -z: u = +y, v = +x
    (2, 1, 0, 1),  # z = L, normal +z
    (0, 0, 2, 1),  # x = 0, normal -x: u = +z, v = +y
    (0, 1, 1, 2),  # x = L, normal +x
    (1, 0, 0, 2),  # y = 0, normal -y
    (1, 1, 2, 0),  # y = L, normal +y
]


def _quad8_from_corner(p1, du, dv):
    """Integer half-step coordinates of the 8 nodes of the quad whose corner 1 is
    p1 and whose sides are du (xi1) and dv (xi2)."""
    p1 = np.asarray(p1)
    du = np.asarray(du)
    dv = np.asarray(dv)
    return [p1, p1 + du, p1 + du + dv, p1 + dv,
            p1 + du // 2, p1 + du + dv // 2, p1 + dv + du // 2, p1 + dv // 2]


def box(dims=(1.0, 1.0, 1.0), divs=(4, 4, 4), split_faces=False, name="box"):
    """Closed quad8 surface of the box [0,Lx]x[0,Ly]x[0,Lz].

    split_faces=False: one closed boundary with shared nodes (18 n^2 + 2 nodes
    for an n x n x n cube). split_faces=True: six boundaries with their own nodes
    (duplicated along the box edges), the layout of the reference tutorials.
    """
    dims = np.asarray(dims, dtype=np.float64)
    divs = np.asarray(divs, dtype=np.int64)
    key_to_node = {}
    coords = []
    conn = []
    face_of = []
    for fid, (axis, side, ua, va) in enumerate(_BOX_FACES):
        nu, nv = int(divs[ua]), int(divs[va])
        for b in range(nv):
            for a in range(nu):
                p1 = np.zeros(3, dtype=np.int64)
                p1[axis] = side * 2 * divs[axis]
                p1[ua] = 2 * a
                p1[va] = 2 * b
                du = np.zeros(3, dtype=np.int64)
                dv = np.zeros(3, dtype=np.int64)
                du[ua] = 2
                dv[va] = 2
                el = []
                for p in _quad8_from_corner(p1, du, dv):
                    key = (fid if split_faces else -1, int(p[0]), int(p[1]), int(p[2]))
                    if key not in key_to_node:
                        key_to_node[key] = len(coords)
                        coords.append(p * dims / (2 * divs))
                    el.append(key_to_node[key])
                conn.append(el)
                face_of.append(fid)
    nodes = np.array(coords, dtype=np.float64)
    conn = np.array(conn, dtype=np.int32)
    nn = nodes.shape[0]
    ctype = np.ones((nn, 3), dtype=np.int32)
    cvalue = np.zeros((nn, 3), dtype=np.complex128)
    return Deck(name, nodes, conn, ctype, cvalue, np.array(face_of, dtype=np.int32))


def cube_clamped_top_traction(n, L=1.0, traction=(0.0, 0.0, -1.0), name=None):
    """Unit cube, n x n quad8 per face, one closed boundary with shared nodes.
    Bottom-face nodes (z=0, edges included): u = 0. Top-face nodes (z=L, edges
    included): t = traction. All other nodes traction-free."""
    d = box((L, L, L), (n, n, n), split_faces=False, name=name or f"cube{n}")
    z = d.nodes[:, 2]
    tol = 1e-12 * L
    top = np.abs(z - L) <= tol
    bot = np.abs(z) <= tol
    d.ctype[:] = 1
    d.cvalue[:] = 0.0
    d.cvalue[top] = np.asarray(traction, dtype=np.complex128)
    d.ctype[bot] = 0
    d.cvalue[bot] = 0.0
    return d


def cube_confined_kat(n, L=1.0, P=1.0):
    """Confined cube of docs/examples/ME-ST-EL-002 (rollers on five faces,
    traction P on x=L), six boundaries with duplicated edge nodes as in the
    tutorial deck t2.dat. Exact field: u1 = (1+nu)(1-2nu)/(E(1-nu)) P x1."""
    d = box((L, L, L), (n, n, n), split_faces=True, name=f"kat_s{n}")
    d.ctype[:] = 1
    d.cvalue[:] = 0.0
    for e in range(d.n_elements):
        axis, side, _, _ = _BOX_FACES[int(d.boundary_of_element[e])]
        for s in d.conn[e]:
            if axis == 0 and side == 1:
                d.ctype[s] = 1
                d.cvalue[s] = (P, 0.0, 0.0)
            else:
                d.ctype[s, axis] = 0
                d.cvalue[s, axis] = 0.0
    return d


def slab(nxy=16, nz=1, dims=(1.0, 1.0, 0.02), traction_top=(0.0, 0.0, -1.0)):
    """Thin slab: nxy x nxy quad8 on each large face, nxy x nz on each edge face.
    Face x=0 clamped (u=0 on its nodes, edges included); top face (z=Lz)
    loaded with traction_top; all other nodes traction-free."""
    d = box(dims, (nxy, nxy, nz), split_faces=False, name=f"slab{nxy}x{nz}")
    tol = 1e-12
    x = d.nodes[:, 0]
    z = d.nodes[:, 2]
    d.ctype[:] = 1
    d.cvalue[:] = 0.0
    top = np.abs(z - dims[2]) <= tol
    d.cvalue[top] = np.asarray(traction_top, dtype=np.complex128)
    clamp = np.abs(x) <= tol
    d.ctype[clamp] = 0
    d.cvalue[clamp] = 0.0
    return d


def surface_patch(half=10.0, n=40, load_half=1.0, traction=(0.0, 0.0, -1.0)):
    """Open square patch [-half,half]^2 of the free surface z=0 (normal +z, out
    of the half-space z<0), n x n quad8 elements, traction on the nodes with
    |x|,|y| <= load_half, traction-free elsewhere. Rim nodes lie on the mesh
    boundary and get the SBIE-MCA formulation."""
    h = 2.0 * half / n
    key_to_node = {}
    coords = []
    conn = []
    for b in range(n):
        for a in range(n):
            p1 = np.array([2 * a, 2 * b, 0])
            el = []
            for p in _quad8_from_corner(p1, np.array([2, 0, 0]), np.array([0, 2, 0])):
                key = (int(p[0]), int(p[1]))
                if key not in key_to_node:
                    key_to_node[key] = len(coords)
                    coords.append([-half + 0.5 * h * p[0], -half + 0.5 * h * p[1], 0.0])
                el.append(key_to_node[key])
            conn.append(el)
    nodes = np.array(coords, dtype=np.float64)
    conn = np.array(conn, dtype=np.int32)
    nn = nodes.shape[0]
    ctype = np.ones((nn, 3), dtype=np.int32)
    cvalue = np.zeros((nn, 3), dtype=np.complex128)
    tol = 1e-9
    loaded = (np.abs(nodes[:, 0]) <= load_half + tol) & (np.abs(nodes[:, 1]) <= load_half + tol)
    cvalue[loaded] = np.asarray(traction, dtype=np.complex128)
    return Deck(f"patch{n}", nodes, conn, ctype, cvalue, np.zeros(len(conn), dtype=np.int32))


# ----------------------------------------------------------------------------
# Half-space decks: the region x3 >= 0 with the traction-free surface x3 = 0
# (outward normal -e3, the only plane the static complementary kernel takes).
# Element normals point out of the soil.
# ----------------------------------------------------------------------------

_Q8_REVERSE = [0, 3, 2, 1, 7, 6, 5, 4]  # same element, opposite normal


def halfspace_footing(a=1.0, n=8, p=1.0):
    """Loaded square [-a,a]^2 on the surface x3 = 0 of the half-space x3 >= 0,
    n x n quad8, uniform pressure p (traction (0, 0, p) on the soil, pushing
    into it) on every node; the rest of the surface is free and not meshed.
    Love's closed form for the settlement of the centre:
    8 ln(1 + sqrt 2) p a (1 - nu^2) / (pi E)."""
    h = 2.0 * a / n
    key_to_node = {}
    coords = []
    conn = []
    for b in range(n):
        for c in range(n):
            p1 = np.array([2 * c, 2 * b, 0])
            el = []
            # xi1 along +x2, xi2 along +x1: T1 x T2 = -e3
            for q in _quad8_from_corner(p1, np.array([0, 2, 0]), np.array([2, 0, 0])):
                key = (int(q[0]), int(q[1]))
                if key not in key_to_node:
                    key_to_node[key] = len(coords)
                    coords.append([-a + 0.5 * h * q[0], -a + 0.5 * h * q[1], 0.0])
                el.append(key_to_node[key])
            conn.append(el)
    nodes = np.array(coords, dtype=np.float64)
    nn = len(nodes)
    ctype = np.ones((nn, 3), dtype=np.int32)
    cvalue = np.zeros((nn, 3), dtype=np.complex128)
    cvalue[:, 2] = p
    return Deck(f"hs_footing{n}", nodes, np.array(conn, dtype=np.int32), ctype, cvalue,
                np.zeros(len(conn), dtype=np.int32))


def _compact(nodes, conn):
    used = np.unique(conn)
    remap = -np.ones(len(nodes), dtype=np.int64)
    remap[used] = np.arange(len(used))
    return nodes[used], remap[conn].astype(np.int32)


def halfspace_excavation(a=0.5, depth=0.5, n=4, p=1.0):
    """Open box [-a,a]^2 x [0,depth] cut into the half-space x3 >= 0: its
    bottom and four walls (no lid; the rim lies on the free surface and its
    nodes get SBIE-MCA), normals into the box. Pressure p on the bottom
    (traction (0, 0, p)), walls traction-free."""
    d = box((2 * a, 2 * a, depth), (n, n, n), split_faces=False, name="hs_excavation")
    keep = d.boundary_of_element != 0  # drop the face x3 = 0
    conn = d.conn[keep][:, _Q8_REVERSE]
    nodes = d.nodes - np.array([a, a, 0.0])
    nodes, conn = _compact(nodes, conn)
    nn = len(nodes)
    ctype = np.ones((nn, 3), dtype=np.int32)
    cvalue = np.zeros((nn, 3), dtype=np.complex128)
    bottom = np.abs(nodes[:, 2] - depth) <= 1e-12
    cvalue[bottom, 2] = p
    return Deck(f"hs_excavation{n}", nodes, conn, ctype, cvalue, d.boundary_of_element[keep])


def halfspace_cavity(a=0.25, top=0.2, n=3, p=1.0):
    """Closed cubic cavity [-a,a]^2 x [top, top+2a] buried in the half-space
    x3 >= 0, normals into the cavity, traction (0, 0, p) on every node."""
    d = box((2 * a, 2 * a, 2 * a), (n, n, n), split_faces=False, name="hs_cavity")
    conn = d.conn[:, _Q8_REVERSE].astype(np.int32)
    nodes = d.nodes - np.array([a, a, -top])
    nn = len(nodes)
    ctype = np.ones((nn, 3), dtype=np.int32)
    cvalue = np.zeros((nn, 3), dtype=np.complex128)
    cvalue[:, 2] = p
    return Deck(f"hs_cavity{n}", nodes, conn, ctype, cvalue, d.boundary_of_element)


def penny_crack(a=1.0, m=2, k=2, p=1.0):
    """Penny-shaped crack of radius a in the plane z = 0 of a full space,
    quad8, an O-grid: an m x m central square of half-width a/2 and four
    blocks of m x k elements out to the circle (mid-side nodes on the mapped
    curves). Element normals +z. Both faces loaded by the crack pressure p:
    face 1 (outward normal +z) t = -p e_z, face 2 t = +p e_z. Returns the
    deck (face 1 conditions) and (crack_el, ctype2, cvalue2).
    Sneddon's opening: u2_z - u1_z = 8 (1 - nu^2) p / (pi E) sqrt(a^2 - r^2)."""
    s0 = 0.5 * a

    def central(u, v):
        return np.array([s0 * u, s0 * v, 0.0])

    def outer(t, rho, rot):
        p0 = np.array([s0, s0 * t])
        th = t * np.pi / 4.0
        p1 = a * np.array([np.cos(th), np.sin(th)])
        q = (1.0 - rho) * p0 + rho * p1
        c, sn = np.cos(rot), np.sin(rot)
        return np.array([c * q[0] - sn * q[1], sn * q[0] + c * q[1], 0.0])

    loc = [(-1, -1), (1, -1), (1, 1), (-1, 1), (0, -1), (1, 0), (0, 1), (-1, 0)]
    elems = []
    for i in range(m):
        for j in range(m):
            u0, v0 = -1 + 2 * i / m, -1 + 2 * j / m
            elems.append([central(u0 + (1 + xi) / m, v0 + (1 + eta) / m) for xi, eta in loc])
    for b in range(4):
        rot = b * np.pi / 2.0
        for i in range(m):
            for j in range(k):
                t0, r0 = -1 + 2 * i / m, j / k
                # local xi along rho, eta along t (orientation fixed below)
                elems.append([outer(t0 + (1 + eta) / m, r0 + (1 + xi) / (2 * k), rot) for xi, eta in loc])
    coords, conn, index = [], [], {}
    for el in elems:
        row = []
        for x in el:
            key = tuple(np.round(x, 12))
            if key not in index:
                index[key] = len(coords)
                coords.append(x)
            row.append(index[key])
        conn.append(row)
    nodes = np.array(coords)
    conn = np.array(conn, dtype=np.int32)
    # orientation: +z normals (counter-clockwise corners)
    for e in range(len(conn)):
        c = nodes[conn[e, :4]]
        if np.cross(c[1] - c[0], c[3] - c[0])[2] < 0:
            conn[e] = conn[e][[0, 3, 2, 1, 7, 6, 5, 4]]
    nn = len(nodes)
    ctype = np.ones((nn, 3), dtype=np.int32)
    cvalue = np.zeros((nn, 3), dtype=np.complex128)
    cvalue[:, 2] = -p
    cvalue2 = np.zeros((nn, 3), dtype=np.complex128)
    cvalue2[:, 2] = p
    d = Deck(f"penny{m}x{k}", nodes, conn, ctype, cvalue, np.zeros(len(conn), dtype=np.int32))
    return d, (np.ones(len(conn), dtype=bool), np.ones((nn, 3), dtype=np.int32), cvalue2)


def penny_crack_in_box(a=1.0, m=2, k=1, half=2.0, nb=2, p=1.0):
    """The pressurised penny crack of penny_crack inside a clamped cube
    [-half, half]^3 (nb x nb quad8 per face, u = 0): one region with a
    crack-like and an ordinary boundary. The crack's elements come first, so
    the ordinary nodes' rows follow the six-row crack nodes."""
    dc, (ce, ct2, cv2) = penny_crack(a, m, k, p)
    db = box((2 * half,) * 3, (nb, nb, nb), split_faces=False)
    nodes = np.vstack([dc.nodes, db.nodes - half])
    conn = np.vstack([dc.conn, db.conn + dc.n_nodes]).astype(np.int32)
    nb_n = db.n_nodes
    ctype = np.vstack([dc.ctype, np.zeros((nb_n, 3), dtype=np.int32)])
    cvalue = np.vstack([dc.cvalue, np.zeros((nb_n, 3), dtype=np.complex128)])
    ct2 = np.vstack([ct2, np.ones((nb_n, 3), dtype=np.int32)])
    cv2 = np.vstack([cv2, np.zeros((nb_n, 3), dtype=np.complex128)])
    ce = np.concatenate([ce, np.zeros(db.n_elements, dtype=bool)])
    d = Deck(f"penny{m}x{k}_box{nb}", nodes, conn, ctype, cvalue,
             np.concatenate([np.zeros(dc.n_elements, np.int32), 1 + db.boundary_of_element]))
    return d, (ce, ct2, cv2)


def sneddon_opening(r, a, p, E, nu):
    """Opening of a pressurised penny crack (Sneddon 1946)."""
    return 8.0 * (1.0 - nu ** 2) * p / (np.pi * E) * np.sqrt(np.maximum(a * a - r * r, 0.0))


def love_square_centre(a, p, E, nu):
    """Settlement of the centre of a uniformly loaded square 2a x 2a on an
    elastic half-space (Love; four corners of a x a squares)."""
    return 8.0 * np.log(1.0 + np.sqrt(2.0)) * p * a * (1.0 - nu ** 2) / (np.pi * E)


# ----------------------------------------------------------------------------
# Materials
# ----------------------------------------------------------------------------

def elastic(E=1.0, nu=0.25):
    """Static elastic region: (mu, nu) as the staela builder reads them."""
    return {"mu": E / (2.0 * (1.0 + nu)), "nu": nu}


def viscoelastic(E=1.0, nu=0.25, rho=1.0, xi=0.05):
    """Viscoelastic region as src/read_regions.f90:938-948 builds it: complex
    mu* = mu (1 + 2 i xi), lambda* = 2 mu* nu / (1 - 2 nu), complex-typed nu."""
    mu = E / (2.0 * (1.0 + nu))
    muc = mu * (1.0 + 2.0j * xi)
    lam = 2.0 * muc * nu / (1.0 - 2.0 * nu)
    cs = np.sqrt(mu / rho)
    return {"mu": muc, "lambda": lam, "nu": complex(nu), "rho": rho, "mu_real": mu, "c_s": cs}


def omega_from_a0(a0, mat, L=1.0):
    """Dimensionless frequency a0 = omega L / c_s with the undamped c_s."""
    return np.asarray(a0, dtype=np.float64) * mat["c_s"] / L


# ----------------------------------------------------------------------------
# The five workloads of the benchmark definition
# ----------------------------------------------------------------------------

def workload(cfg: int):
    """Deck, material and frequencies (None for static) of workload cfg (1..5)."""
    if cfg == 1:
        return cube_clamped_top_traction(4), elastic(1.0, 0.25), None
    if cfg == 2:
        m = viscoelastic(1.0, 0.25, 1.0, 0.05)
        return cube_clamped_top_traction(8), m, omega_from_a0(np.linspace(0.1, 2.0, 20), m)
    if cfg == 3:
        m = viscoelastic(1.0, 0.33, 1.0, 0.05)
        return surface_patch(10.0, 40, 1.0), m, omega_from_a0([0.5], m)
    if cfg == 5:
        m = viscoelastic(1.0, 0.3, 1.0, 0.02)
        return slab(16, 1), m, omega_from_a0([0.2, 1.0], m)
    raise ValueError(cfg)


def batch_workload():
    """Workload 4: cubes n in {4,5,6,7,8,10} per face x 8 frequencies."""
    m = viscoelastic(1.0, 0.25, 1.0, 0.05)
    om = omega_from_a0(np.linspace(0.2, 1.6, 8), m)
    return [(cube_clamped_top_traction(n), m, om) for n in (4, 5, 6, 7, 8, 10)]
