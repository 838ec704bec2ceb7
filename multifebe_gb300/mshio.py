"""Gmsh *.msh 2.2 meshes for the collocation-BEM path.

read_msh() uses the library's native reader (mfbem_msh_read, the gmsh branch
of fbem_mesh%read_from_file, lib/fbem/src/mesh.f90:104-494). deck_from_msh()
turns the quad8 elements of chosen parts into a Deck with the per-boundary
conditions of an input deck's ``[conditions over be boundaries]`` section:
for every part (boundary) and direction, 0 (displacement known) or 1
(traction known) and the complex value. As in the reference, a node belongs
to one boundary only (the .msh files of its tutorials carry one copy of a
junction node per boundary); nodes keep the file's order, elements too, so
the DOF numbering is the reference's. write_msh() writes a Deck in the same
format (physical part = boundary_of_element + 1).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi
from .meshgen import Deck

QUAD8 = 16  # gmsh element type


@dataclass
class MshMesh:
    parts: list           # [(id, dim, name)]
    node_id: np.ndarray   # (nn,) int32
    x: np.ndarray         # (nn, 3)
    el_id: np.ndarray     # (ne,) int32
    el_type: np.ndarray   # (ne,) gmsh type codes
    el_part: np.ndarray   # (ne,) physical ids
    el_off: np.ndarray    # (ne + 1,)
    el_nodes: np.ndarray  # node ids, gmsh order

    def element_nodes(self, e):
        return self.el_nodes[self.el_off[e]:self.el_off[e + 1]]


def _lib():
    L = _abi.load()
    if not getattr(L, "_msh_set", False):
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)
        L.mfbem_msh_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
        L.mfbem_msh_error.restype = ctypes.c_char_p
        L.mfbem_msh_sizes.argtypes = [vp, ip]
        L.mfbem_msh_parts.argtypes = [vp, ip, ip, ctypes.c_char_p, ctypes.c_int32]
        L.mfbem_msh_nodes.argtypes = [vp, ip, dp]
        L.mfbem_msh_elements.argtypes = [vp, ip, ip, ip, ip, ip]
        L.mfbem_msh_free.argtypes = [vp]
        L.mfbem_msh_free.restype = None
        L._msh_set = True
    return L


def read_msh(path) -> MshMesh:
    L = _lib()
    h = ctypes.c_void_p()
    if L.mfbem_msh_read(str(path).encode(), ctypes.byref(h)) != 0:
        raise ValueError(f"{path}: {L.mfbem_msh_error().decode()}")
    try:
        ip = ctypes.POINTER(ctypes.c_int32)
        c = np.zeros(4, np.int32)
        L.mfbem_msh_sizes(h, c.ctypes.data_as(ip))
        npart, nn, ne, nen = (int(v) for v in c)
        pid, pdim = np.zeros(npart, np.int32), np.zeros(npart, np.int32)
        names = ctypes.create_string_buffer(64 * npart)
        L.mfbem_msh_parts(h, pid.ctypes.data_as(ip), pdim.ctypes.data_as(ip), names, 64)
        parts = [(int(pid[i]), int(pdim[i]), names.raw[64 * i:64 * (i + 1)].split(b"\0")[0].decode())
                 for i in range(npart)]
        nid, x = np.zeros(nn, np.int32), np.zeros((nn, 3))
        L.mfbem_msh_nodes(h, nid.ctypes.data_as(ip), x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        eid, et, ep = np.zeros(ne, np.int32), np.zeros(ne, np.int32), np.zeros(ne, np.int32)
        eo, en = np.zeros(ne + 1, np.int32), np.zeros(nen, np.int32)
        L.mfbem_msh_elements(h, eid.ctypes.data_as(ip), et.ctypes.data_as(ip), ep.ctypes.data_as(ip),
                             eo.ctypes.data_as(ip), en.ctypes.data_as(ip))
    finally:
        L.mfbem_msh_free(h)
    return MshMesh(parts, nid, x, eid, et, ep, eo, en)


def deck_from_msh(mesh: MshMesh, conditions: dict, parts=None, name="msh") -> Deck:
    """Deck of the quad8 elements of `parts` (default: every part holding quad8
    elements). conditions: part id -> three (type, value) pairs, type 0
    displacement known / 1 traction known; parts without an entry are
    traction-free."""
    sel = [e for e in range(len(mesh.el_id)) if mesh.el_type[e] == QUAD8 and (parts is None or mesh.el_part[e] in parts)]
    if not sel:
        raise ValueError("no quad8 elements in the chosen parts")
    used = {}
    for e in sel:
        for v in mesh.element_nodes(e):
            used.setdefault(int(v), None)
    pos = {int(v): i for i, v in enumerate(mesh.node_id)}
    order = sorted(used, key=lambda v: pos[v])  # file order of the used nodes
    local = {v: i for i, v in enumerate(order)}
    nodes = mesh.x[[pos[v] for v in order]]
    conn = np.array([[local[int(v)] for v in mesh.element_nodes(e)] for e in sel], dtype=np.int32)
    nn = len(order)
    ctype = np.ones((nn, 3), np.int32)
    cvalue = np.zeros((nn, 3), np.complex128)
    owner = np.full(nn, -1)
    for row, e in enumerate(sel):
        p = int(mesh.el_part[e])
        bc = conditions.get(p, [(1, 0.0)] * 3)
        for s in conn[row]:
            if owner[s] >= 0 and owner[s] != p:
                raise ValueError(f"node {order[s]} sits in two boundaries ({owner[s]} and {p})")
            owner[s] = p
            for k in range(3):
                ctype[s, k] = int(bc[k][0])
                cvalue[s, k] = complex(bc[k][1])
    return Deck(name, nodes, conn, ctype, cvalue, np.array([mesh.el_part[e] for e in sel], dtype=np.int32))


def write_msh(deck: Deck, path, part_names=None):
    """Write the deck's elements as gmsh 2.2 quad8, one physical part per
    boundary_of_element value (part id = value + 1), nodes numbered from 1."""
    bnd = deck.boundary_of_element if deck.boundary_of_element is not None else np.zeros(deck.n_elements, int)
    pids = sorted(set(int(b) + 1 for b in bnd))
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$PhysicalNames\n%d\n" % len(pids))
        for p in pids:
            nm = (part_names or {}).get(p, f"boundary{p}")
            f.write(f'2 {p} "{nm}"\n')
        f.write("$EndPhysicalNames\n$Nodes\n%d\n" % deck.n_nodes)
        for i, x in enumerate(deck.nodes):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, x[0], x[1], x[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % deck.n_elements)
        for e, c in enumerate(deck.conn):
            p = int(bnd[e]) + 1
            f.write("%d 16 2 %d %d " % (e + 1, p, p) + " ".join(str(int(v) + 1) for v in c) + "\n")
        f.write("$EndElements\n")
