"""gmsh mesh ingest for the assembly (examples/tutorial/mesh.py:23-62).

The reference reads a gmsh file with meshio and turns it into nlfem's arrays:
* vertices: the points' first two coordinates;
* elements: the triangles;
* element labels: the triangles' physical tags, with the largest tag negated (the interaction
  layer).

With set_art_vertex, one artificial vertex at (0, 0) is appended, and every line cell becomes a
label-0 element (line end points + the artificial vertex). The search passes through label-0
elements but never pairs them, so the boundary lines connect the interaction domain's parts.
trim_artificial_vertex removes them again after the solve.

meshio is not needed: this module parses the ASCII MSH formats 2.2 and 4.1 itself. Points are
numbered in file order, and cells keep their file order per type, as meshio numbers them.
"""
import numpy as np

_NODES_PER_TYPE = {1: 2, 2: 3, 3: 4, 4: 4, 15: 1}   # line, triangle, quad, tetra, point


def _sections(lines):
    """{name: [body lines]} of the $Name ... $EndName sections."""
    out, name, body = {}, None, []
    for ln in lines:
        t = ln.strip()
        if not t:
            continue
        if t.startswith("$"):
            if t.startswith("$End"):
                out[name] = body
                name, body = None, []
            else:
                name, body = t[1:], []
        elif name is not None:
            body.append(t)
    return out


def _read_v2(sec):
    nodes = sec["Nodes"]
    n = int(nodes[0])
    tags, pts = [], []
    for ln in nodes[1:1 + n]:
        f = ln.split()
        tags.append(int(f[0]))
        pts.append([float(f[1]), float(f[2]), float(f[3])])
    index = {t: i for i, t in enumerate(tags)}
    cells = {}   # type -> (connectivity rows, physical tags)
    els = sec["Elements"]
    for ln in els[1:1 + int(els[0])]:
        f = [int(x) for x in ln.split()]
        et, nt = f[1], f[2]
        phys = f[3] if nt > 0 else 0
        nn = _NODES_PER_TYPE.get(et)
        if nn is None:
            raise ValueError(f"unsupported gmsh element type {et}")
        conn = [index[t] for t in f[3 + nt:3 + nt + nn]]
        c, p = cells.setdefault(et, ([], []))
        c.append(conn)
        p.append(phys)
    return np.array(pts), cells


def _read_v4(sec):
    # physical tags of the entities (points, curves, surfaces, volumes)
    ent_phys = {}
    if "Entities" in sec:
        e = sec["Entities"]
        counts = [int(x) for x in e[0].split()]
        row = 1
        for dim, cnt in enumerate(counts):
            for _ in range(cnt):
                f = e[row].split()
                row += 1
                tag = int(f[0])
                # points: tag x y z nPhys phys...; others: tag minx miny minz maxx maxy maxz nPhys phys...
                k = 4 if dim == 0 else 7
                nphys = int(f[k])
                ent_phys[(dim, tag)] = int(f[k + 1]) if nphys > 0 else 0
    nodes = sec["Nodes"]
    nblocks, nnodes = (int(x) for x in nodes[0].split()[:2])
    tags, pts = [], []
    row = 1
    for _ in range(nblocks):
        f = nodes[row].split()
        row += 1
        parametric, nb = int(f[2]), int(f[3])
        if parametric:
            raise ValueError("parametric gmsh nodes are not supported")
        tags.extend(int(nodes[row + i]) for i in range(nb))
        row += nb
        for i in range(nb):
            x = nodes[row + i].split()
            pts.append([float(x[0]), float(x[1]), float(x[2])])
        row += nb
    if len(pts) != nnodes:
        raise ValueError("inconsistent $Nodes section")
    index = {t: i for i, t in enumerate(tags)}
    els = sec["Elements"]
    nblocks = int(els[0].split()[0])
    cells = {}
    row = 1
    for _ in range(nblocks):
        f = els[row].split()
        row += 1
        dim, etag, et, nb = int(f[0]), int(f[1]), int(f[2]), int(f[3])
        nn = _NODES_PER_TYPE.get(et)
        if nn is None:
            raise ValueError(f"unsupported gmsh element type {et}")
        phys = ent_phys.get((dim, etag), 0)
        c, p = cells.setdefault(et, ([], []))
        for i in range(nb):
            x = [int(v) for v in els[row + i].split()]
            c.append([index[t] for t in x[1:1 + nn]])
            p.append(phys)
        row += nb
    return np.array(pts), cells


def read_msh(filename):
    """(points (n, 3), {gmsh element type: (connectivity (m, k) int64, physical tags (m,) int64)})
    of an ASCII MSH 2.2 or 4.1 file."""
    with open(filename) as fh:
        sec = _sections(fh.readlines())
    fmt = sec.get("MeshFormat")
    if not fmt:
        raise ValueError("not a gmsh file: no $MeshFormat")
    version, filetype = fmt[0].split()[:2]
    if int(filetype) != 0:
        raise ValueError("binary gmsh files are not supported (save as ASCII)")
    if version.startswith("2"):
        pts, cells = _read_v2(sec)
    elif version.startswith("4"):
        pts, cells = _read_v4(sec)
    else:
        raise ValueError(f"unsupported gmsh format {version}")
    return pts, {t: (np.array(c, dtype=np.int64), np.array(p, dtype=np.int64)) for t, (c, p) in cells.items()}


def add_artificial_vertex(lines, vertices, elements, elementlabels):
    """Search bridges across a boundary: one extra vertex at the origin and, per line cell (a, b),
    a degenerate element (a, b, extra) labelled 0. Label-0 elements carry no quadrature; they
    only connect the breadth-first pair search (the convention of the reference's gmsh tutorial,
    examples/tutorial/mesh.py:23-33)."""
    lines = np.asarray(lines, dtype=np.int64).reshape(-1, 2)
    extra = vertices.shape[0]
    bridges = np.column_stack([lines, np.full(lines.shape[0], extra, dtype=np.int64)])
    origin = np.zeros((1, vertices.shape[1]))
    return (np.vstack([vertices, origin]), np.vstack([elements, bridges]),
            np.concatenate([elementlabels, np.zeros(lines.shape[0], dtype=np.int64)]))


def trim_artificial_vertex(nlfem_mesh, u=None, f_base=None):
    """Undoes add_artificial_vertex after a solve: the label-0 elements and vertices leave the
    mesh dict (changed in place and returned), and u / f_base keep the entries whose solution
    label is nonzero (examples/tutorial/mesh.py:36-46)."""
    masks = {"element": nlfem_mesh["elementLabels"] != 0, "vertex": nlfem_mesh["vertexLabels"] != 0,
             "solution": nlfem_mesh["solutionLabels"] != 0}
    for key, kind in (("elements", "element"), ("elementLabels", "element"),
                      ("vertices", "vertex"), ("vertexLabels", "vertex"), ("solutionLabels", "solution")):
        nlfem_mesh[key] = nlfem_mesh[key][masks[kind]]
    u, f_base = (None if a is None else a[masks["solution"]] for a in (u, f_base))
    return nlfem_mesh, u, f_base


def read_gmsh(filename, set_art_vertex=True):
    """(vertices (n, 2), elements (m, 3), element labels (m,)) of a 2D gmsh file: the triangles
    with their physical tags as labels, where the largest tag names the interaction layer and
    becomes negative; with set_art_vertex the line cells become label-0 bridges
    (examples/tutorial/mesh.py:49-58)."""
    pts, cells = read_msh(filename)
    if 2 not in cells:
        raise ValueError("the gmsh file holds no triangles")
    elements, tags = cells[2]
    labels = np.where(tags == tags.max(), -tags, tags)
    vertices = np.array(pts[:, :2])
    if not set_art_vertex:
        return vertices, elements, labels
    lines = cells[1][0] if 1 in cells else np.zeros((0, 2), dtype=np.int64)
    return add_artificial_vertex(lines, vertices, elements, labels)
