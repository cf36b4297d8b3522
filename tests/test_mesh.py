"""Structured mesher and Abaqus reader (host-side input generation)."""
import numpy as np
import pytest


@pytest.mark.parametrize("et", [4, 10, 8])
def test_box_mesh_volume_and_orientation(jfem, npo, et):
    m = jfem.mesh.box_mesh(et, 3, 2, 4, 1.5, 1.0, 2.0)
    pts, wts = npo.rule(et)
    vol = 0.0
    for xi, wq in zip(pts, wts):
        _, dN = npo.basis(et, xi)
        J = np.einsum("ak,eab->ekb", dN, m.X[m.conn])
        det = np.linalg.det(J)
        assert (det > 0).all()
        vol += (wq * det).sum()
    assert abs(vol - 3.0) < 1e-12


def test_sizes_of_named_configurations(jfem):
    wl = jfem.workloads
    w = wl.cfg_tet4_cantilever()
    assert (w.mesh.n_elem, w.mesh.n_nodes, w.n_dofs) == (3840, 1025, 3075)
    assert w.fixed_dofs.size == 75 and w.faces.shape == (32, 3)
    m = jfem.mesh.box_mesh(10, 4, 2, 2)
    assert m.n_nodes == 9 * 5 * 5


@pytest.mark.parametrize("et", [4, 10])
def test_tet_split_is_conforming(jfem, et):
    m = jfem.mesh.box_mesh(et, 3, 3, 2)
    faces = {}
    for e in m.conn[:, :4]:
        for f in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
            k = tuple(sorted(e[list(f)]))
            faces[k] = faces.get(k, 0) + 1
    counts = np.array(list(faces.values()))
    assert counts.max() == 2
    # boundary faces = 2 triangles per cube face on the box surface
    nb = (counts == 1).sum()
    assert nb == 2 * 2 * (3 * 3 + 3 * 2 + 3 * 2)


@pytest.mark.parametrize("et", [4, 10, 8])
def test_box_face_matches_volume_faces(jfem, npo, et):
    m = jfem.mesh.box_mesh(et, 3, 2, 2, 1.5, 1.0, 1.0)
    ft, faces = m.face(0, 1)
    f = npo.traction(ft, faces, m.X, [1.0, 0.0, 0.0])
    assert abs(f.reshape(-1, 3)[:, 0].sum() - 1.0) < 1e-12     # area 1
    assert np.allclose(m.X[np.unique(faces), 0], 1.5)


def test_abaqus_reader_synthetic(jfem):
    text = """*HEADING
** a two-element Tet4 mesh
*NODE, NSET=NALL
1, 0.0, 0.0, 0.0
2, 1.0, 0.0, 0.0
3, 0.0, 1.0, 0.0
4, 0.0, 0.0, 1.0
5, 1.0, 1.0, 1.0
*ELEMENT, TYPE=C3D4, ELSET=BODY
1, 1, 2, 3, 4
2, 2, 3,
 4, 5
*NSET, NSET=GEN, GENERATE
1, 5, 2
*ELSET, ELSET=FIRST
1
*SURFACE, TYPE=ELEMENT, NAME=TOP
FIRST, S1
*ELASTIC
2.0e5, 0.25
*BOUNDARY
GEN, 1, 3
4, 2
*DSLOAD
TOP, P, 3.0
"""
    ab = jfem.abaqus.read(text)
    assert len(ab.nodes) == 5 and ab.elements[2] == ("Tet4", [2, 3, 4, 5])
    assert ab.node_sets["GEN"] == [1, 3, 5] and ab.elastic == (2.0e5, 0.25)
    ft, nodes = ab.surface_elements("TOP")[0]
    assert ft == "Tri3" and nodes == [1, 3, 2]
    et, X, conn, index, eids = ab.to_arrays()
    dofs, vals = jfem.abaqus.boundary_dofs(ab, index)
    assert list(dofs) == [0, 1, 2, 6, 7, 8, 10, 12, 13, 14]
    assert ab.dsload == [("TOP", "P", 3.0)]


def test_abaqus_reader_reference_fixture(jfem):
    """The reference's fixture test/testdata/cube_tet4.inp, read from the
    reference tree named by JFEM_REFERENCE_ROOT (skipped when it is unset or
    the file is absent), parses to the mesh stored in the golden fixture."""
    import os
    from pathlib import Path
    root = os.environ.get("JFEM_REFERENCE_ROOT")
    if not root:
        pytest.skip("JFEM_REFERENCE_ROOT (a JuliaFEM.jl source tree) is not set")
    p = Path(root) / "test" / "testdata" / "cube_tet4.inp"
    if not p.exists():
        pytest.skip(f"{p} not found")
    ab = jfem.abaqus.read(str(p))
    et, X, conn, index, eids = ab.to_arrays()
    assert et == "Tet4" and X.shape == (10, 3) and conn.shape == (17, 4)
    import numpy as np
    d = np.load(Path(__file__).parent / "golden" / "cube_tet4.npz")
    assert np.array_equal(d["X"], X) and np.array_equal(d["conn"], conn)


def test_rcm_matches_reference_restatement(jfem, orc):
    """jfem_rcm (C++ in the library) against the Python restatement of the
    reference's symrcm, on a shuffled Tet10 box and a mesh with two parts."""
    m = jfem.mesh.box_mesh(10, 4, 2, 2, 2.0, 1.0, 1.0)
    g = np.random.default_rng(5)
    shuffle = g.permutation(m.n_nodes)
    conn = shuffle[m.conn]                       # scramble the numbering
    perm, b0, b1 = jfem._abi.rcm(conn, m.n_nodes, start=int(shuffle[0]))
    op, ob0, ob1 = orc.rcm(conn, m.n_nodes, start=int(shuffle[0]))
    assert np.array_equal(perm, op) and (b0, b1) == (ob0, ob1)
    assert sorted(perm) == list(range(m.n_nodes)) and b1 < b0 / 2
    two = np.concatenate([m.conn, m.conn + m.n_nodes])
    perm2, _, _ = jfem._abi.rcm(two, 2 * m.n_nodes, start=3)
    op2, _, _ = orc.rcm(two, 2 * m.n_nodes, start=3)
    assert np.array_equal(perm2, op2)
    perm1, _, _ = jfem._abi.rcm(conn + 1, m.n_nodes, start=int(shuffle[0]) + 1, index_base=1)
    assert np.array_equal(perm1, perm + 1)
