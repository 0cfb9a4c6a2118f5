"""Mesh input on the host (no GPU): GMSH 2.2 / 4.1 reader (mshReader::
readSections, mshreader.cpp:200-376), the include / exclude selection
(sortOutIncludesAndExcludes / elementIsIncluded, :22-198, :378-428), the
quadrilateral split (global::quadrilateralsToTriangles, global.cpp:841-870) and
the wall-impedance mapping (WallImpedanceSection::setUpValues,
SolvingScript/wallimpedancesection.cpp:308-405).

The files are written here from known geometry, so the expected triangles,
physical and geometric numbers are known exactly."""
import os
import re

import numpy as np
import pytest

NAMES = ["front", "back", "left", "right", "bottom", "top"]
# the reference's Example folder (its example meshes and projects), when a
# copy is at hand: BEM_REFERENCE_EXAMPLES=<path to Example>; skipped otherwise
REF_EXAMPLES = os.environ.get("BEM_REFERENCE_EXAMPLES", "")


def cube_faces(n=3, seed=0):
    """Unit-cube faces as structured grids: faces 0-3 triangulated, faces 4-5
    as quadrilaterals. Node tags are sparse and face-local (shared edges get
    duplicate nodes, which the format allows)."""
    rng = np.random.default_rng(seed)
    frames = [((0, 0, 0), (1, 0, 0), (0, 0, 1)), ((0, 1, 0), (0, 0, 1), (1, 0, 0)),
              ((0, 0, 0), (0, 0, 1), (0, 1, 0)), ((1, 0, 0), (0, 1, 0), (0, 0, 1)),
              ((0, 0, 0), (0, 1, 0), (1, 0, 0)), ((0, 0, 1), (1, 0, 0), (0, 1, 0))]
    faces = []
    tag = 100
    for f, (o, e1, e2) in enumerate(frames):
        o, e1, e2 = map(np.array, (o, e1, e2))
        ids = {}
        nodes = []
        for i in range(n + 1):
            for j in range(n + 1):
                p = o + e1 * i / n + e2 * j / n + rng.uniform(-1e-3, 1e-3, 3) * (0 < i < n) * (0 < j < n)
                ids[i, j] = tag
                nodes.append((tag, p))
                tag += 3
        elems = []
        for i in range(n):
            for j in range(n):
                a, b, c, d = ids[i, j], ids[i + 1, j], ids[i + 1, j + 1], ids[i, j + 1]
                if f < 4:
                    elems += [(2, (a, b, c)), (2, (a, c, d))]
                else:
                    elems.append((3, (a, b, c, d)))
        faces.append({"nodes": nodes, "elems": elems, "phys": 11 + f, "geom": 1 + f,
                      "name": NAMES[f]})
    return faces


def expected(faces, keep=lambda f: True):
    xyz = {t: p for f in faces for t, p in f["nodes"]}
    tri, tp, tg, quad, qp, qg = [], [], [], [], [], []
    for f in faces:
        if not keep(f):
            continue
        for typ, nd in f["elems"]:
            co = np.concatenate([xyz[t] for t in nd])
            (tri if typ == 2 else quad).append(co)
            (tp if typ == 2 else qp).append(f["phys"])
            (tg if typ == 2 else qg).append(f["geom"])
    return (np.array(tri).reshape(-1, 9), np.array(tp), np.array(tg),
            np.array(quad).reshape(-1, 12), np.array(qp), np.array(qg))


def xyz(p):
    """Coordinates as shortest round-trip decimal strings."""
    return " ".join(repr(float(c)) for c in p)


def write_v2(path, faces):
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(faces))]
    lines += [f'2 {f["phys"]} "{f["name"]}"' for f in faces]
    lines += ["$EndPhysicalNames", "$Nodes", str(sum(len(f["nodes"]) for f in faces))]
    lines += [f"{t} {xyz(p)}" for f in faces for t, p in f["nodes"]]
    lines.append("$EndNodes")
    el = []
    first = faces[0]["nodes"]
    el.append(f"1 15 2 0 7 {first[0][0]}")                  # a point element
    el.append(f"2 1 2 0 3 {first[0][0]} {first[1][0]}")    # a line element
    for f in faces:
        for typ, nd in f["elems"]:
            el.append(f'{len(el) + 1} {typ} 2 {f["phys"]} {f["geom"]} ' + " ".join(map(str, nd)))
    lines += ["$Elements", str(len(el))] + el + ["$EndElements"]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def write_v4(path, faces):
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(faces))]
    lines += [f'2 {f["phys"]} "{f["name"]}"' for f in faces]
    lines += ["$EndPhysicalNames", "$Entities", f"0 1 {len(faces)} 0",
              "1 0 0 0 1 0 0 0 0"]                               # one curve, no physical tag
    lines += [f'{f["geom"]} 0 0 0 1 1 1 1 {f["phys"]} 0' for f in faces]
    lines.append("$EndEntities")
    nn = sum(len(f["nodes"]) for f in faces)
    tags = [t for f in faces for t, _ in f["nodes"]]
    lines += ["$Nodes", f"{len(faces)} {nn} {min(tags)} {max(tags)}"]
    for f in faces:
        lines.append(f'2 {f["geom"]} 0 {len(f["nodes"])}')
        lines += [str(t) for t, _ in f["nodes"]]
        lines += [xyz(p) for _, p in f["nodes"]]
    lines.append("$EndNodes")
    blocks, count = [], 0
    first = faces[0]["nodes"]
    blocks += ["1 1 1 1", f"1 {first[0][0]} {first[1][0]}"]   # a line block
    count += 1
    for f in faces:
        for typ in (2, 3):
            els = [nd for t, nd in f["elems"] if t == typ]
            if not els:
                continue
            blocks.append(f'2 {f["geom"]} {typ} {len(els)}')
            for nd in els:
                count += 1
                blocks.append(f"{count} " + " ".join(map(str, nd)))
    nblk = 1 + sum(1 for f in faces for typ in (2, 3) if any(t == typ for t, _ in f["elems"]))
    lines += ["$Elements", f"{nblk} {count} 1 {count}"] + blocks + ["$EndElements"]
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


@pytest.fixture(params=["v2", "v4"])
def cube_file(request, tmp_path):
    faces = cube_faces()
    path = str(tmp_path / f"cube_{request.param}.msh")
    (write_v2 if request.param == "v2" else write_v4)(path, faces)
    return path, faces


def check(sel, exp):
    tri, tp, tg, quad, qp, qg = exp
    assert np.array_equal(sel["tri"], tri) and np.array_equal(sel["quad"], quad)
    assert np.array_equal(sel["tri_phys"], tp) and np.array_equal(sel["tri_geom"], tg)
    assert np.array_equal(sel["quad_phys"], qp) and np.array_equal(sel["quad_geom"], qg)


def test_reads_every_element(bem, cube_file):
    path, faces = cube_file
    m = bem.MshFile(path)
    assert m.physical_names == [(2, 11 + i, n) for i, n in enumerate(NAMES)]
    check(m.select(), expected(faces))
    check(m.select("all", ""), expected(faces))


@pytest.mark.parametrize("include,exclude,keep", [
    ("FRONT back", "", lambda f: f["name"] in ("front", "back")),
    ("1...3", "", lambda f: 1 <= f["geom"] <= 3),
    ("2..5", "3", lambda f: f["geom"] in (2, 4, 5)),
    ("all", "top 1", lambda f: f["name"] != "top" and f["geom"] != 1),
    ("..2", "", lambda f: f["geom"] <= 2),
    ("5...", "", lambda f: f["geom"] >= 5),
    ("all 4", "", lambda f: f["geom"] == 4),          # "all" plus more: include mode
    ("left", "left", lambda f: f["name"] == "left"),  # name excludes act only with "all"
    ("", "2, 3;4", lambda f: f["geom"] not in (2, 3, 4)),
    ("nosuchgroup", "", lambda f: False),
])
def test_selection(bem, cube_file, include, exclude, keep):
    path, faces = cube_file
    m = bem.MshFile(path)
    check(m.select(include, exclude), expected(faces, keep))


def test_quads_to_triangles(bem):
    rng = np.random.default_rng(4)
    q = rng.uniform(-1, 1, (50, 12))
    t = bem.quads_to_triangles(q)
    assert t.shape == (100, 9)
    n = q.reshape(-1, 4, 3)
    for i in range(50):
        d1 = np.linalg.norm(n[i, 0] - n[i, 2])
        d2 = np.linalg.norm(n[i, 1] - n[i, 3])
        order = [(0, 1, 3), (1, 2, 3)] if d1 > d2 else [(3, 0, 2), (0, 1, 2)]
        ref = np.concatenate([n[i, list(o)].ravel() for o in order])
        assert np.array_equal(t[2 * i:2 * i + 2].ravel(), ref)


def test_read_msh_splits_quadrilaterals(bem, cube_file):
    path, faces = cube_file
    tri, phys, geom = bem.read_msh(path)
    t, tp, tg, q, qp, qg = expected(faces)
    assert np.array_equal(tri, np.vstack([t, bem.quads_to_triangles(q)]))
    assert np.array_equal(phys, np.concatenate([tp, np.repeat(qp, 2)]))
    assert np.array_equal(geom, np.concatenate([tg, np.repeat(qg, 2)]))


def test_facade(bem, cube_file):
    path, faces = cube_file
    r = bem.mshReader().readMsh(path, 7, False, ["top"], [])
    t, _, _, q, _, _ = expected(faces, lambda f: f["name"] == "top")
    assert np.array_equal(r.quadrilaterals, q) and r.triangles.shape == (0, 9)
    assert r.physicalGroupsNames == NAMES and r.physicalGroupsNumbers == list(range(11, 17))
    r.readMsh(path)
    assert r.triangles.shape[0] == 4 * 18 and r.quadrilaterals.shape[0] == 2 * 9


def test_bad_files(bem, tmp_path, cube_file):
    path, faces = cube_file
    with pytest.raises(bem.BemError):
        bem.MshFile(str(tmp_path / "missing.msh"))
    text = open(path).read()
    cases = {
        "truncated": text[: text.index("$EndElements") - 20],
        "binary": text.replace(text.splitlines()[1], text.splitlines()[1].replace(" 0 ", " 1 ")),
        "version": text.replace(text.splitlines()[1], "4.0 0 8"),
        "no_nodes": re.sub(r"\$Nodes.*?\$EndNodes\n", "", text, flags=re.S),
    }
    for name, bad in cases.items():
        p = tmp_path / f"{name}.msh"
        p.write_text(bad)
        with pytest.raises(bem.BemError):
            bem.MshFile(str(p))
    # an element that names a node the file does not define
    bad = text.replace(f' {faces[0]["elems"][-1][1][0]} ', " 999999 ", 1) if "4.1" not in text \
        else text.replace(f'\n{faces[1]["nodes"][0][0]}\n', "\n999999\n", 1)
    p = tmp_path / "unknown_node.msh"
    p.write_text(bad)
    with pytest.raises(bem.BemError):
        bem.MshFile(str(p))


def test_wall_beta(bem):
    Zm = 1.2 * 343.0
    assert bem.wall_beta(bem.IMP_REFLECTION, 0.5) == pytest.approx(1 / 3)
    assert bem.wall_beta(bem.IMP_DAMPING, 0.4) == pytest.approx(0.25)
    Z = 2.0 + 1.0j
    assert bem.wall_beta(bem.IMP_IMPEDANCE, Z) == pytest.approx(1 / Z)
    assert bem.wall_beta(bem.IMP_IMPEDANCE, Z, False, Zm) == pytest.approx(Zm / Z)
    assert bem.wall_beta(bem.IMP_ADMITTANCE, 0.3 - 0.1j) == pytest.approx(0.3 - 0.1j)
    assert bem.wall_beta(bem.IMP_ADMITTANCE, 0.3, False, Zm) == pytest.approx(0.3 * Zm)
    with pytest.raises(bem.BemError):
        bem.wall_beta(bem.IMP_ADMITTANCE, 0.3, False, 0.0)  # medium impedance not set
    with pytest.raises(bem.BemError):
        bem.wall_beta(7, 0.3)
    with pytest.raises(bem.BemError):
        bem.wall_beta(bem.IMP_REFLECTION, -1.0)  # 1 + R = 0


@pytest.mark.skipif(not REF_EXAMPLES or not os.path.isdir(REF_EXAMPLES),
                    reason="BEM_REFERENCE_EXAMPLES not set")
@pytest.mark.parametrize("rel", ["Loudspeaker/loudspeaker.msh", "Pensil/Pensil R70.msh",
                                 "Sphere/twoSpheres.msh"])
def test_reference_example_meshes(bem, rel):
    """The reference's own example meshes (GMSH 2.2): per physical group, the
    triangle count equals a plain text count of the $Elements lines."""
    path = os.path.join(REF_EXAMPLES, rel)
    text = open(path).read()
    body = text[text.index("$Elements"):text.index("$EndElements")].splitlines()[2:]
    rows = [list(map(int, l.split())) for l in body if l.strip()]
    tris = [r for r in rows if r[1] == 2]
    m = bem.MshFile(path)
    sel = m.select()
    assert sel["tri"].shape[0] == len(tris)
    assert np.array_equal(sel["tri_phys"], [r[3] if r[2] >= 1 else 0 for r in tris])
    for dim, tag, name in m.physical_names:
        n = sum(1 for r in tris if r[2] >= 1 and r[3] == tag)
        assert m.select(name)["tri"].shape[0] == n
    # areas are positive and finite: the node lookup resolved every triangle
    t = sel["tri"].reshape(-1, 3, 3)
    area = np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1)
    assert np.isfinite(area).all() and (area > 0).all()


def _refine_restated(tri, L):
    """ElementSection::refineTriangles / recursiveRefineTriangle
    (elementSection.cpp:688-800) restated recursively."""
    out, par = [], []

    def length(a, b):
        return np.sqrt((a[0] - b[0]) ** 2 + (a[1] - b[1]) ** 2 + (a[2] - b[2]) ** 2)

    def rec(t, i):
        n1, n2, n3 = t[0:3], t[3:6], t[6:9]
        a, b, c = length(n1, n2), length(n2, n3), length(n3, n1)
        k = (1 if a > c else 3) if a > b else (2 if b > c else 3)
        e = (a, b, c)[k - 1]
        if e <= L:
            out.append(t)
            par.append(i)
            return
        if k == 1:
            m = (n1 + n2) / 2
            h1, h2 = (n1, m, n3), (m, n2, n3)
        elif k == 2:
            m = (n2 + n3) / 2
            h1, h2 = (n1, n2, m), (m, n3, n1)
        else:
            m = (n3 + n1) / 2
            h1, h2 = (n1, n2, m), (m, n2, n3)
        rec(np.concatenate(h1), i)
        rec(np.concatenate(h2), i)

    for i, t in enumerate(np.asarray(tri, float).reshape(-1, 9)):
        rec(t, i)
    return np.array(out).reshape(-1, 9), np.array(par)


def _areas(t):
    t = t.reshape(-1, 3, 3)
    return 0.5 * np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1)


def test_refine_triangles_matches_restatement(bem, meshes):
    rng = np.random.default_rng(3)
    tri = np.vstack([rng.uniform(-1, 1, (40, 9)), meshes.icosphere(1, 2.0),
                     np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0.0]])])  # a right isosceles (ties)
    for L in (0.9, 0.35, 0.12):
        out, par = bem.refine_triangles(tri, L)
        ref, rpar = _refine_restated(tri, L)
        assert np.array_equal(out, ref) and np.array_equal(par, rpar)
        t = out.reshape(-1, 3, 3)
        edges = np.linalg.norm(t - np.roll(t, -1, axis=1), axis=2)
        assert edges.max() <= L
        # halves tile their parent: areas add up, normals keep their direction
        tot = np.bincount(par, weights=_areas(out), minlength=tri.shape[0])
        assert np.allclose(tot, _areas(tri), rtol=1e-12, atol=0)
        def nrm(x):
            x = x.reshape(-1, 3, 3)
            c = np.cross(x[:, 1] - x[:, 0], x[:, 2] - x[:, 0])
            return c / np.linalg.norm(c, axis=1)[:, None]
        assert np.allclose(nrm(out), nrm(tri)[par], atol=1e-12)


def test_refine_by_mesh_frequency_and_errors(bem, meshes):
    tri = meshes.icosphere(2, 1.0)
    out, _ = bem.refine_triangles(tri, mesh_frequency=1000.0, c=343.0)
    ref, _ = _refine_restated(tri, 343.0 / 1000.0 / 2)
    assert np.array_equal(out, ref) and out.shape[0] > tri.shape[0]
    same, par = bem.refine_triangles(tri, 10.0)  # already fine enough: unchanged
    assert np.array_equal(same, tri) and np.array_equal(par, np.arange(tri.shape[0]))
    with pytest.raises(bem.BemError):
        bem.refine_triangles(tri, 0.0)
    with pytest.raises(bem.BemError):
        bem.refine_triangles(tri)
