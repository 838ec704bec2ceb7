"""Gmsh *.msh 2.2 reader (native, mfbem_msh_*), deck builder and writer.

The reference's own tutorial meshes (docs/examples/*/case_files/*.msh) are read
where the reference sources are present and compared with an independent plain
Python parse of the same files; a quad8 deck survives write -> read -> deck
unchanged; the inputs fbem_mesh%read_from_file refuses are refused."""
import glob
import os

import numpy as np
import pytest

from multifebe_gb300 import meshgen as M, mshio


def _plain_parse(path):
    """Counts and first/last entries of each section, by a plain text scan."""
    lines = open(path).read().splitlines()
    out = {}
    for sec in ("PhysicalNames", "Nodes", "Elements"):
        i = lines.index("$" + sec)
        n = int(lines[i + 1])
        out[sec] = (n, lines[i + 2].split(), lines[i + 1 + n].split())
    return out


def test_reads_the_reference_tutorial_meshes(reference_dir):
    files = sorted(glob.glob(os.path.join(reference_dir, "docs", "examples", "*", "case_files", "*.msh")))
    assert files
    for f in files:
        ref = _plain_parse(f)
        m = mshio.read_msh(f)
        assert len(m.parts) == ref["PhysicalNames"][0]
        assert m.parts[0][:2] == (int(ref["PhysicalNames"][1][1]), int(ref["PhysicalNames"][1][0]))
        assert m.parts[0][2] == ref["PhysicalNames"][1][2].strip('"')
        assert len(m.node_id) == ref["Nodes"][0] and len(m.el_id) == ref["Elements"][0]
        first, last = ref["Nodes"][1], ref["Nodes"][2]
        assert m.node_id[0] == int(first[0]) and np.allclose(m.x[0], [float(v) for v in first[1:4]])
        assert m.node_id[-1] == int(last[0]) and np.allclose(m.x[-1], [float(v) for v in last[1:4]])
        e = ref["Elements"][2]
        ntags = int(e[2])
        assert m.el_type[-1] == int(e[1]) and m.el_part[-1] == int(e[3])
        assert list(m.element_nodes(len(m.el_id) - 1)) == [int(v) for v in e[3 + ntags:]]


def _kat_conditions(P=1.0):
    # docs/examples/ME-ST-EL-002: rollers on five faces, traction P on x = L;
    # parts = faces of meshgen.box + 1
    cond = {}
    for face, (axis, side, _, _) in enumerate(M._BOX_FACES):
        if axis == 0 and side == 1:
            cond[face + 1] = [(1, P), (1, 0.0), (1, 0.0)]
        else:
            bc = [(1, 0.0)] * 3
            bc[axis] = (0, 0.0)
            cond[face + 1] = bc
    return cond


def test_write_read_round_trip(tmp_path):
    d = M.cube_confined_kat(3)
    p = tmp_path / "kat3.msh"
    mshio.write_msh(d, p)
    m = mshio.read_msh(p)
    assert [q[0] for q in m.parts] == [1, 2, 3, 4, 5, 6]
    d2 = mshio.deck_from_msh(m, _kat_conditions())
    assert np.array_equal(d2.nodes, d.nodes) and np.array_equal(d2.conn, d.conn)
    assert np.array_equal(d2.ctype, d.ctype) and np.array_equal(d2.cvalue, d.cvalue)


def _write(tmp_path, text):
    p = tmp_path / "bad.msh"
    p.write_text(text)
    return p


GOOD_HEAD = "$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$PhysicalNames\n1\n2 1 \"s\"\n$EndPhysicalNames\n"
NODES = "$Nodes\n8\n" + "".join(f"{i + 1} {x} {y} 0\n" for i, (x, y) in enumerate(
    [(-1, -1), (1, -1), (1, 1), (-1, 1), (0, -1), (1, 0), (0, 1), (-1, 0)])) + "$EndNodes\n"
ELEM = "$Elements\n1\n1 16 2 1 1 1 2 3 4 5 6 7 8\n$EndElements\n"


def test_refuses_what_the_reference_refuses(tmp_path):
    m = mshio.read_msh(_write(tmp_path, GOOD_HEAD + NODES + ELEM))
    assert len(m.el_id) == 1 and m.el_type[0] == 16
    bad = {
        "version": GOOD_HEAD.replace("2.2 0 8", "4.1 0 8") + NODES + ELEM,
        "no parts": "$MeshFormat\n2.2 0 8\n$EndMeshFormat\n" + NODES + ELEM,
        "undeclared part": GOOD_HEAD + NODES + ELEM.replace("16 2 1 1", "16 2 7 1"),
        "repeated node": GOOD_HEAD + NODES.replace("8 -1 0 0", "7 -1 0 0") + ELEM,
        "unknown type": GOOD_HEAD + NODES + ELEM.replace(" 16 2 ", " 99 2 "),
        "undeclared node": GOOD_HEAD + NODES + ELEM.replace(" 8\n", " 9\n"),
        "zero part id": GOOD_HEAD.replace('2 1 "s"', '2 0 "s"') + NODES + ELEM,
        # a quad8 and a line3 in the same physical group
        "mixed dimensions": GOOD_HEAD + NODES + ELEM.replace("$Elements\n1\n", "$Elements\n2\n").replace(
            "$EndElements", "2 8 2 1 1 1 5 2\n$EndElements"),
        # a declared part without elements
        "empty part": GOOD_HEAD.replace('1\n2 1 "s"', '2\n2 1 "s"\n2 2 "e"') + NODES + ELEM,
    }
    for what, text in bad.items():
        with pytest.raises(ValueError):
            mshio.read_msh(_write(tmp_path, text))


def test_a_node_in_two_boundaries_is_refused(tmp_path):
    d = M.cube_confined_kat(2)
    d.boundary_of_element[0] = 1  # one element of face 0 moved to part 2: its nodes now sit in two parts
    p = tmp_path / "two.msh"
    mshio.write_msh(d, p)
    with pytest.raises(ValueError):
        mshio.deck_from_msh(mshio.read_msh(p), _kat_conditions())
