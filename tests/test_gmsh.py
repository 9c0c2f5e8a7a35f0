"""gmsh ingest (examples/tutorial/mesh.py:23-62) without meshio: MSH 2.2 and 4.1 give the same
arrays, the interaction layer gets the negated largest physical tag, and the boundary lines become
label-0 elements through the artificial vertex."""
import numpy as np
import pytest

MSH22 = """$MeshFormat
2.2 0 8
$EndMeshFormat
$Nodes
5
1 0 0 0
2 1 0 0
3 1 1 0
4 0 1 0
5 0.5 0.5 0
$EndNodes
$Elements
7
1 15 2 4 1 1
2 1 2 3 1 1 2
3 1 2 3 2 2 3
4 2 2 1 1 1 2 5
5 2 2 1 1 2 3 5
6 2 2 2 2 3 4 5
7 2 2 2 2 4 1 5
$EndElements
"""

MSH41 = """$MeshFormat
4.1 0 8
$EndMeshFormat
$Entities
1 2 2 0
1 0 0 0 1 4
1 0 0 0 1 0 0 1 3 2 1 -2
2 1 0 0 1 1 0 1 3 2 2 -3
1 0 0 0 1 1 0 1 1 2 1 2
2 0 0 0 1 1 0 1 2 2 1 2
$EndEntities
$Nodes
1 5 1 5
2 1 0 5
1
2
3
4
5
0 0 0
1 0 0
1 1 0
0 1 0
0.5 0.5 0
$EndNodes
$Elements
5 7 1 7
0 1 15 1
1 1
1 1 1 1
2 1 2
1 2 1 1
3 2 3
2 1 2 2
4 1 2 5
5 2 3 5
2 2 2 2
6 3 4 5
7 4 1 5
$EndElements
"""


@pytest.mark.parametrize("text", [MSH22, MSH41], ids=["2.2", "4.1"])
def test_read_gmsh(tmp_path, text):
    from nlfem_gb300 import gmsh
    f = tmp_path / "m.msh"
    f.write_text(text)
    v, e, l = gmsh.read_gmsh(str(f))
    assert v.shape == (6, 2) and np.array_equal(v[-1], [0.0, 0.0])
    np.testing.assert_array_equal(e, [[0, 1, 4], [1, 2, 4], [2, 3, 4], [3, 0, 4], [0, 1, 5], [1, 2, 5]])
    np.testing.assert_array_equal(l, [1, 1, -2, -2, 0, 0])
    v2, e2, l2 = gmsh.read_gmsh(str(f), set_art_vertex=False)
    assert v2.shape == (5, 2) and e2.shape == (4, 3)
    np.testing.assert_array_equal(l2, [1, 1, -2, -2])


def test_trim_artificial_vertex(tmp_path):
    from nlfem_gb300 import gmsh
    from nlfem_gb300.meshes import mesh_dict
    f = tmp_path / "m.msh"
    f.write_text(MSH22)
    v, e, l = gmsh.read_gmsh(str(f))
    m = mesh_dict(v, e, l)
    m["solutionLabels"] = m["vertexLabels"].copy()
    u = np.arange(v.shape[0], dtype=float)
    m, u, _ = gmsh.trim_artificial_vertex(m, u)
    assert (m["elementLabels"] != 0).all() and m["elements"].shape[0] == 4
    assert m["vertices"].shape[0] == (m["vertexLabels"] != 0).sum() == u.shape[0]


def test_rejects_binary_and_unknown(tmp_path):
    from nlfem_gb300 import gmsh
    f = tmp_path / "b.msh"
    f.write_text("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(ValueError):
        gmsh.read_msh(str(f))
    f.write_text("no mesh here\n")
    with pytest.raises(ValueError):
        gmsh.read_msh(str(f))
