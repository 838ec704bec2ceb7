"""Nodal-solution files (*.nso) of the mechanics problems.

write_nso() writes the boundary-node records of a BE region the way
export_solution_mechanics_{harmonic,static}_nso do
(src/export_solution_mechanics_harmonic_nso.f90,
src/export_solution_mechanics_static_nso.f90): the header (program, version,
input file, description, timestamp, column description, and for the harmonic
file the column-header line), then per boundary (increasing id), per element
of the boundary and per element node, the first appearance of each node. The
records themselves are formatted by the library's native writer
(mfbem_nso_write) with the Fortran edit descriptors the export settings name
(src/read_export.f90): the real format sci_double (E25.16E3), sci_simple,
sci_less, eng_double, eng_simple (the default EN18.8E2) or eng_less, integer
columns I(n + 1) with n the digits of the largest identifier.

read_nso() reads the records back (comment lines skipped).
"""
from __future__ import annotations

import ctypes
import datetime

import numpy as np

from . import _abi

# src/read_export.f90:163-170
REAL_FORMATS = {"sci_double": ("E", 25, 16, 3), "sci_simple": ("E", 16, 8, 2), "sci_less": ("E", 11, 3, 2),
                "eng_double": ("N", 27, 16, 3), "eng_simple": ("N", 18, 8, 2), "eng_less": ("N", 13, 3, 2),
                "auto": ("N", 27, 16, 3)}


def _lib():
    L = _abi.load()
    if not getattr(L, "_nso_set", False):
        vp, i32, dp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_double
        L.mfbem_nso_write.argtypes = [ctypes.c_char_p, i32, ctypes.c_char_p, i32, i32, dp, i32, i32, vp, vp, vp, vp,
                                      i32, ctypes.c_char, i32, i32, i32, i32]
        L.mfbem_nso_error.restype = ctypes.c_char_p
        L.mfbem_fortran_format.argtypes = [ctypes.c_char, i32, i32, i32, dp, ctypes.c_char_p]
        L._nso_set = True
    return L


def fortran_format(kind, w, d, e, v) -> str:
    """One value under the edit descriptor 'I' w, 'E' Ew.dEe or 'N' ENw.dEe."""
    buf = ctypes.create_string_buffer(w + 1)
    if _lib().mfbem_fortran_format(kind.encode(), w, d, e, float(v), buf) != 0:
        raise ValueError("invalid edit descriptor")
    return buf.value.decode()


def int_width(*ids) -> int:
    """fmt_integer of src/read_export.f90:61: digits of max(2, ids...) + 1."""
    return len(str(max([2] + [int(np.max(i)) for i in ids if np.size(i)]))) + 1


def _header(harmonic, int_w, real_w, version, input_file, description, timestamp, complex_notation):
    ts = (timestamp or datetime.datetime.now()).strftime("%Y-%m-%d;%H:%M:%S.%f")[:23]
    h = ["# Program      : multifebe", f"# Version      : {version[:5]:<5}", "# File_format  : nso",
         "# Problem_dim  : 3", f"# Input_file   : {input_file}", f"# Description  : {description}",
         f"# Timestamp    : {ts}", "", "# Columns  Description"]
    if harmonic:
        h += ["# C1-C2    Frequency index and value w (rad/s)."]
    else:
        h += ["# C1-C2    Step index and value."]
    h += ["# C3-C5    Region id, class and type.",
          "# C6-C8    (if C4 == 1) Boundary id, class and face." if harmonic else
          "# C6-C8    (if col C4 == 1) Boundary id, class and face.",
          "# C6-C8    (if C4 == 2) Subregion id, number of DOF and 0." if harmonic else
          "# C6-C8    (if col C4 == 2) Subregion id, number of DOF and 0.",
          "# C9-C12   Node id, x1, x2 and x3.",
          "# >=C13    Node variables. Depend on the region class and type (see documentation).", "#"]
    if harmonic:
        h += ["# Complex notation: " + ("polar" if complex_notation == 1 else "cartesian"), "#"]
        # column-header line: C1 over an integer column, C3..C9 integer, the rest real (44 columns in 3D)
        line = "#" + "_" * (int_w - 3) + "C1"
        for kc in range(2, 45):
            nc = int_w if 3 <= kc <= 9 else real_w
            line += "_" * (nc - len(str(kc)) - 1) + f"C{kc}"
        h.append(line)
    return "\n".join(h) + "\n"


def export_order(deck, boundary_ids=None):
    """(node index, boundary id) of every record: boundaries in increasing id,
    elements in order, element nodes in order, first appearance per boundary."""
    bnd = (deck.boundary_of_element + 1) if deck.boundary_of_element is not None else np.ones(deck.n_elements, int)
    out = []
    for b in (boundary_ids if boundary_ids is not None else sorted(set(int(v) for v in bnd))):
        seen = set()
        for e in np.nonzero(bnd == b)[0]:
            for s in deck.conn[e]:
                if int(s) not in seen:
                    seen.add(int(s))
                    out.append((int(s), int(b)))
    return out


def write_nso(path, deck, u, t, omega=None, kf=1, append=False, header=True, real="eng_simple", node_id=None,
              region_id=1, complex_notation=2, n_frequencies=1, version="2.0.1", input_file="", description="",
              timestamp=None):
    """Write the nodal solution u, t [n_nodes, 3] of a deck (complex with
    omega: harmonic, frequency index kf; real without: static)."""
    harmonic = omega is not None
    kind, w, d, e = REAL_FORMATS[real]
    order = export_order(deck)
    nid = np.asarray(node_id if node_id is not None else np.arange(1, deck.n_nodes + 1), dtype=np.int32)
    idx = np.array([s for s, _ in order], dtype=np.int64)
    bid = np.ascontiguousarray([b for _, b in order], dtype=np.int32)
    ids = np.ascontiguousarray(nid[idx], dtype=np.int32)
    x = np.ascontiguousarray(deck.nodes[idx], dtype=np.float64)
    vals = np.concatenate([np.asarray(u)[idx], np.asarray(t)[idx]], axis=1)
    vals = np.ascontiguousarray(vals.astype(np.complex128 if harmonic else np.float64))
    int_w = int_width(n_frequencies, region_id, bid, deck.n_elements, nid)
    head = _header(harmonic, int_w, w, version, input_file, description, timestamp, complex_notation) \
        if header else None
    L = _lib()
    rc = L.mfbem_nso_write(str(path).encode(), 1 if append else 0, head.encode() if head else None,
                           1 if harmonic else 0, int(kf), float(omega or 0.0), region_id, len(ids), ids.ctypes.data,
                           bid.ctypes.data, x.ctypes.data, vals.view(np.float64).ctypes.data, int_w, kind.encode(), w,
                           d, e, complex_notation)
    if rc != 0:
        raise OSError(L.mfbem_nso_error().decode())
    return order


def read_nso(path):
    """The records of a *.nso file as a float array [n_records, n_columns]."""
    rows = []
    with open(path) as f:
        for line in f:
            if not line.strip() or line.lstrip().startswith("#"):
                continue
            rows.append([float(v.replace("D", "E")) for v in line.split()])
    return np.array(rows)
