"""Project / solving-script reader (3d_bem_gb300/project.py, the common subset
of SolvingScriptReader): a synthetic project exercising every supported
section, and the reference's own example projects when present."""
import importlib
import math
import os

import numpy as np
import pytest

from test_msh import cube_faces, write_v2

# the reference's Example folder (its example meshes and projects), when a
# copy is at hand: BEM_REFERENCE_EXAMPLES=<path to Example>; skipped otherwise
REF_EXAMPLES = os.environ.get("BEM_REFERENCE_EXAMPLES", "")


@pytest.fixture(scope="module")
def project():
    return importlib.import_module("3d_bem_gb300.project")


def test_units(project):
    u = project.with_units
    assert u("70mm", "m") == pytest.approx(0.07) and u("mm", "m") == pytest.approx(1e-3)
    assert u("100Hz", "Hz") == 100 and u("1kHz", "Hz") == 1000 and u("344m/s", "m/s") == 344
    assert u("6.1", "m") == 6.1 and u("1m", "m") == 1.0


def test_synthetic_project(bem, project, tmp_path):
    faces = cube_faces(n=2)
    write_v2(str(tmp_path / "cube.msh"), faces)
    (tmp_path / "p.abec").write_text(
        "; test project\n[Solving]\nScriptname_Solving=Solving.txt\n"
        "[MeshFiles]\nC0=cube.msh,CubeAlias\n")
    (tmp_path / "Solving.txt").write_text("""// test
Control_Solver
    f1=100Hz; f2=1kHz;
    NumFrequencies=3;
    Abscissa=log
    c=340m/s

Elements Walls
    Scale=100mm
    Shift=1 0 0
    Rotate=0 0 90
    MeshFileAlias=CubeAlias
    7 Mesh Include front back
    8 Mesh Include left right

Elements Lid
    scale=mm
    MeshFileAlias=CubeAlias
    3 Mesh Include top

off Elements Ignored
    MeshFileAlias=CubeAlias
    9 Mesh Include all

Driving Piston
    RefElements=Walls
    1 8 Weight=2

Wallimpedance W
    RefElements=Lid
    ImpType=admittance
    value=0.5

Infinite_Baffle "Floor"
    Position = 0,0,-1
    Normal = 0,0,1
""")
    P = project.Project.load(str(tmp_path / "p.abec"))
    assert np.allclose(P.frequencies, [100.0, 100.0 * math.sqrt(10), 1000.0])
    assert P.c == 340.0
    assert set(P.section) == {"Walls", "Lid"}
    sel = bem.MshFile(str(tmp_path / "cube.msh"))
    fb = sel.select("front back")["tri"]
    lr = sel.select("left right")["tri"]
    top = bem.quads_to_triangles(sel.select("top")["quad"])
    n_w = fb.shape[0] + lr.shape[0]
    assert P.triangles.shape[0] == n_w + top.shape[0]
    # Walls: scale 0.1, then p' = T(1,0,0) Rz(90) p
    x = fb.reshape(-1, 3) * 0.1
    ref = np.column_stack([-x[:, 1] + 1.0, x[:, 0], x[:, 2]]).reshape(-1, 9)
    assert np.allclose(P.triangles[:fb.shape[0]], ref, atol=1e-14)
    assert np.allclose(P.triangles[n_w:], top * 1e-3)
    assert list(np.unique(P.element_index)) == [3, 7, 8]
    # driving: index 8 of Walls gets g = 2; the lid is an admittance wall 0.5
    assert np.all(P.g[fb.shape[0]:n_w] == 2) and np.all(P.g[:fb.shape[0]] == 0)
    assert np.all(P.beta[n_w:] == 0.5) and np.all(P.beta[:n_w] == 0)
    assert np.allclose(P.plane[0], [0, 0, -1]) and np.allclose(P.plane[1], [0, 0, 1])


def test_refinement_by_mesh_frequency(bem, project, tmp_path):
    faces = cube_faces(n=1)
    write_v2(str(tmp_path / "cube.msh"), faces)
    (tmp_path / "p.abec").write_text("[Solving]\nScriptname_Solving=S.txt\n"
                                     "[MeshFiles]\nC0=cube.msh,A\n")
    (tmp_path / "S.txt").write_text("Control_Solver\n    f1=100\n    c=340\n"
                                    "Elements E\n    MeshFileAlias=A\n    MeshFrequency=600Hz\n"
                                    "    1 Mesh Include front\n")
    P = project.Project.load(str(tmp_path / "p.abec"))
    src = bem.MshFile(str(tmp_path / "cube.msh")).select("front")["tri"]
    ref, _ = bem.refine_triangles(src, (340.0 / 600.0) / 2)
    assert np.array_equal(P.triangles, ref) and ref.shape[0] > src.shape[0]


@pytest.mark.skipif(not REF_EXAMPLES or not os.path.isdir(REF_EXAMPLES),
                    reason="BEM_REFERENCE_EXAMPLES not set")
@pytest.mark.parametrize("rel,sections", [
    ("Loudspeaker/Project.abec", {"Enclosure-Exterior", "Enclosure-Driver", "Enclosure-Driver-rear"}),
    ("Pensil/pensil.abec", {"enclosure-Exterior", "loudspeaker-Driver-front",
                            "loudspeaker-Driver-rear"}),
])
def test_reference_example_projects(bem, project, rel, sections):
    P = project.Project.load(os.path.join(REF_EXAMPLES, rel))
    assert set(P.section) == sections
    n = P.triangles.shape[0]
    assert n > 0 and np.isfinite(P.triangles).all()
    t = P.triangles.reshape(-1, 3, 3)
    area = 0.5 * np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1)
    assert (area > 0).all()
    assert np.abs(P.triangles).max() < 1.0          # millimetre meshes scaled to metres
    front = np.array([s.endswith(("Driver", "Driver-front")) for s in P.section])
    rear = np.array([s.endswith(("Driver-rear",)) for s in P.section])
    assert np.all(P.g[front] == 1) and np.all(P.g[rear] == -1)
    assert np.all(P.g[~(front | rear)] == 0)
    assert P.plane is None and P.beta is None       # their baffles and walls are "off"
    assert len(P.frequencies) >= 1 and P.frequencies.min() > 0


def test_point_sources_from_nodes(bem, project, tmp_path):
    write_v2(str(tmp_path / "cube.msh"), cube_faces(n=1))
    (tmp_path / "p.abec").write_text("[Solving]\nScriptname_Solving=S.txt\n"
                                     "[MeshFiles]\nC0=cube.msh,A\n")
    (tmp_path / "S.txt").write_text("""Control_Solver
    f1=200
Elements E
    MeshFileAlias=A
    1 Mesh Include all
Nodes "Src"
    scale=10mm
    shift=0 0 1
    1  100 0 0
    2  0 50 0
Pressure_Points P
    DrvWeight=3
    RefNodes="Src"
    10  1  Weight=0.5
    11  2
""")
    P = project.Project.load(str(tmp_path / "p.abec"))
    assert np.allclose(P.sources, [[1.0, 0.0, 1.0, 0.5], [0.0, 0.5, 1.0, 3.0]])
    assert np.all(P.g == 0) and P.beta is None and P.plane is None


@pytest.mark.skipif(not REF_EXAMPLES or not os.path.isdir(REF_EXAMPLES),
                    reason="BEM_REFERENCE_EXAMPLES not set")
def test_reference_sphere_project(bem, project):
    """Example/Sphere: a GMSH 4.1 sphere, a point source 20 m away and an
    active rigid baffle."""
    P = project.Project.load(os.path.join(REF_EXAMPLES, "Sphere/sphere.abec"))
    assert P.triangles.shape[0] > 0 and set(P.section) == {"Spere"}
    assert np.allclose(P.sources, [[20.0, 0.0, 0.0, 1.0]])
    assert np.allclose(P.plane[0], [0, 0, -10]) and np.allclose(P.plane[1], [0, 0, 1])
    assert P.c == 344.0 and np.allclose(P.frequencies, [100.0])
    c = P.triangles.reshape(-1, 3, 3).mean(axis=1)
    assert np.allclose(c.mean(axis=0), [6.1, 1.5, 1.5], atol=0.2)  # shift applied


def _one_section_project(tmp_path, control, section_lines, n=1):
    faces = cube_faces(n=n)
    write_v2(str(tmp_path / "cube.msh"), faces)
    (tmp_path / "p.abec").write_text("[Solving]\nScriptname_Solving=S.txt\n"
                                     "[MeshFiles]\nC0=cube.msh,A\n")
    (tmp_path / "S.txt").write_text("Control_Solver\n" + control +
                                    "Elements E\n    MeshFileAlias=A\n" + section_lines +
                                    "    1 Mesh Include front\n")


def test_default_refinement_from_highest_frequency(bem, project, tmp_path):
    """No MeshFrequency anywhere: the global edge length is half the
    wavelength at max(f1, f2) (ControlSolverSection::getEdgelength,
    controlsolversection.cpp:301-313), applied to every section that sets
    neither MeshFrequency nor EdgeLength (solvingscriptreader.cpp:1109-1111)."""
    _one_section_project(tmp_path, "    f1=100\n    f2=600\n    c=340\n", "")
    P = project.Project.load(str(tmp_path / "p.abec"))
    src = bem.MshFile(str(tmp_path / "cube.msh")).select("front")["tri"]
    ref, _ = bem.refine_triangles(src, (340.0 / 600.0) / 2)
    assert ref.shape[0] > src.shape[0]
    assert np.array_equal(P.triangles, ref)


def test_mesh_frequency_wins_over_edge_length(bem, project, tmp_path):
    """A section with both: MeshFrequency sets the edge length
    (solvingscriptreader.cpp:1113-1116)."""
    _one_section_project(tmp_path, "    f1=100\n    c=340\n",
                         "    MeshFrequency=900Hz\n    EdgeLength=1m\n")
    P = project.Project.load(str(tmp_path / "p.abec"))
    src = bem.MshFile(str(tmp_path / "cube.msh")).select("front")["tri"]
    ref, _ = bem.refine_triangles(src, (340.0 / 900.0) / 2)
    assert ref.shape[0] > src.shape[0]
    assert np.array_equal(P.triangles, ref)


def test_zero_scale_component_means_one(bem, project, tmp_path):
    """Scale=0 2 0 scales by (1, 2, 1) (elementSection.cpp:147-149)."""
    _one_section_project(tmp_path, "    f1=1\n    c=340\n", "    Scale=0 2 0\n")
    P = project.Project.load(str(tmp_path / "p.abec"))
    src = bem.MshFile(str(tmp_path / "cube.msh")).select("front")["tri"]
    assert np.allclose(P.triangles, (src.reshape(-1, 3) * [1.0, 2.0, 1.0]).reshape(-1, 9))
