"""A solve driven from a GMSH file: the box written as a 2.2 mesh with one
physical group per face, read back through bem_msh_read, boundary data set
per physical group (driven face: g = 1, a = 0, b = 1 as
ElementSection::setLocalDrivingWeight, elementSection.cpp:1108-1123; admittance
wall: a = i k beta, b = 1 with beta from bem_wall_beta; rigid elsewhere). The
pressures equal those of the same problem built from arrays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FACES = ["bottom", "top", "y0", "y1", "x0", "x1"]


def face_of(tri, L=(0.3, 0.2, 0.4)):
    """Face index of each triangle: z = 0, z = lz, y = 0, y = ly, x = 0, x = lx."""
    c = (tri[:, 0:3] + tri[:, 3:6] + tri[:, 6:9]) / 3.0
    out = np.full(tri.shape[0], -1)
    for k, (axis, val) in enumerate([(2, 0.0), (2, L[2]), (1, 0.0), (1, L[1]), (0, 0.0),
                                     (0, L[0])]):
        out[np.abs(c[:, axis] - val) < 1e-9] = k
    return out


def write_msh(path, tri, face):
    n = tri.shape[0]
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(FACES))]
    lines += [f'2 {21 + i} "{name}"' for i, name in enumerate(FACES)]
    lines += ["$EndPhysicalNames", "$Nodes", str(3 * n)]
    for i in range(n):
        for v in range(3):
            lines.append(f"{3 * i + v + 1} " + " ".join(repr(float(x)) for x in tri[i, 3 * v:3 * v + 3]))
    lines += ["$EndNodes", "$Elements", str(n)]
    for i in range(n):
        lines.append(f"{i + 1} 2 2 {21 + face[i]} {1 + face[i]} {3 * i + 1} {3 * i + 2} {3 * i + 3}")
    lines.append("$EndElements")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def test_solve_from_msh_file(bem, meshes, tmp_path):
    tri = meshes.box(n_target=1200, seed=9)
    face = face_of(tri)
    assert (face >= 0).all()
    path = str(tmp_path / "box.msh")
    write_msh(path, tri, face)

    tri_f, phys, geom = bem.read_msh(path)
    assert np.array_equal(tri_f, tri)
    top = dict((name, tag) for _, tag, name in bem.MshFile(path).physical_names)["top"]
    bottom = bem.MshFile(path).select("bottom")["tri_phys"][0]
    beta_wall = bem.wall_beta(bem.IMP_ADMITTANCE, 0.5 + 0.2j)

    def solve(tri_, beta, g):
        s = bem.Solver(aca_tol=1e-5, gmres_tol=1e-10, precision=1)
        s.set_mesh(tri_)
        s.set_bc_impedance(beta)
        _, _, p, info = s.solve(400.0, g)
        assert info["status"] == 0
        return p

    p_file = solve(tri_f, np.where(phys == bottom, beta_wall, 0.0),
                   (phys == top).astype(np.complex128))
    p_arr = solve(tri, np.where(face == 0, beta_wall, 0.0), (face == 1).astype(np.complex128))
    assert np.array_equal(p_file, p_arr)
    assert np.abs(p_file[face == 1]).mean() > 0


def test_project_sweep_matches_library_calls(bem, tmp_path):
    """3d_bem_gb300/project.py end to end: a project with an admittance wall,
    a driven face, a point source and a baffle sweeps to the same pressures as
    the same library calls made by hand."""
    import importlib
    from test_msh import cube_faces, write_v2
    project = importlib.import_module("3d_bem_gb300.project")
    write_v2(str(tmp_path / "cube.msh"), cube_faces(n=3))
    (tmp_path / "p.abec").write_text("[Solving]\nScriptname_Solving=S.txt\n"
                                     "[MeshFiles]\nC0=cube.msh,A\n")
    (tmp_path / "S.txt").write_text("""Control_Solver
    f1=200Hz; f2=800Hz; NumFrequencies=3; Abscissa=log
Elements Box
    Scale=200mm
    Shift=0 0 0.5
    MeshFileAlias=A
    1 Mesh Include front back left right bottom
Elements Top
    Scale=200mm
    Shift=0 0 0.5
    MeshFileAlias=A
    2 Mesh Include top
Driving D
    RefElements=Top
    1 2 Weight=1
Wallimpedance W
    RefElements=Box
    ImpType=admittance
    value=0.2
Nodes N
    1  0.1 0.1 2.0
Pressure_Points S
    RefNodes=N
    5 1 Weight=0.3
Infinite_Baffle B
    Position = 0,0,0
    Normal = 0,0,1
""")
    P = project.Project.load(str(tmp_path / "p.abec"))
    assert P.beta is not None and P.plane is not None and len(P.sources) == 1
    p, info = P.sweep(precision=1, aca_tol=1e-5, gmres_tol=1e-9)
    assert p.shape == (P.triangles.shape[0], 3) and np.isfinite(p).all()
    assert all(i["status"] == 0 for i in info)
    s = bem.Solver(wave_speed=P.c, density=P.rho, precision=1, aca_tol=1e-5, gmres_tol=1e-9)
    s.set_mesh(P.triangles)
    s.set_bc_impedance(P.beta)
    s.set_impedance_plane(*P.plane)
    s.set_point_sources(P.sources)
    q, _ = s.sweep(P.frequencies, P.g)
    assert np.array_equal(p, q[:, 0, :])
