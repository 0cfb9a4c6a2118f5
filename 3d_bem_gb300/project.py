"""Reader for the common subset of the reference's project (.abec) and solving
script formats, so its example projects run headlessly through the library.

Follows SolvingScriptReader (SolvingScript/solvingscriptreader.cpp) for:

* the project file's ``[Solving] Scriptname_Solving`` and ``[MeshFiles]``
  aliases (``Cn=file,alias``);
* ``Control_Solver``: f1, f2, NumFrequencies, Abscissa (log / lin), c, rho
  (ControlSolverSection::getFrequencies, controlsolversection.cpp:190-235;
  c defaults to 343.2 m/s as :272-277), MeshFrequency;
* ``Elements``: Scale, Shift, Rotate (QMatrix4x4 order: every Shift / Rotate
  line post-multiplies the transform, Rotate = x, y, z degrees), SwapNormals,
  MeshFileAlias, MeshFrequency / EdgeLength refinement (edge = (c / f) / 2,
  solvingscriptreader.cpp:1104-1127), and ``<index> Mesh [MeshFileAlias=a]
  Include ... [Exclude ...]`` lines (mshReader selection, quadrilaterals
  split); scale first, then the transform (scaleAndTransformElements,
  elementSection.cpp:1007-1039), then the refinement;
* ``MeshFile_Properties``: Scale of an alias;
* ``Driving``: RefElements, DrvWeight, ``<n> <index> [Weight=w]`` lines: the
  referenced elements with that index get g = w, a = 0, b = 1
  (setTrianglesDrivingWeight, elementSection.cpp:1082-1094);
* ``Wallimpedance``: RefElements, ImpType, Normalized, Value: the referenced
  section becomes an impedance wall (WallImpedanceSection::setUpValues) with
  the medium impedance rho c;
* ``Infinite_Baffle``: Position, Normal: one impedance plane;
* ``Nodes`` (Scale / Shift / Rotate, ``<index> x y z`` lines) and
  ``Pressure_Points`` (DrvWeight, RefNodes, ``<index> <node> [Weight=w]``):
  point sources of the right-hand side (setupPressurePoints,
  solvingscriptreader.cpp:1016-1050);
* sections prefixed with ``off`` are skipped; ``//`` starts a comment.

Not read: two baffles or distanceToParallelPlane, per-mesh-file swap flags,
interior ElType, the single-precision aspect-ratio pre-split of
quadrilaterals.
"""
from __future__ import annotations

import configparser
import math
import os
import re
from dataclasses import dataclass, field

import numpy as np

SECTIONS = ("control_solver", "elements", "driving", "wallimpedance", "infinite_baffle",
            "pressure_points", "nodes", "meshfile_properties")
_PREFIX = {"n": 1e-9, "µ": 1e-6, "u": 1e-6, "m": 1e-3, "k": 1e3, "K": 1e3, "M": 1e6, "G": 1e9}
IMP_TYPES = {"reflection": 0, "damping": 1, "impedance": 2, "admittance": 3}


def with_units(text: str, unit: str) -> float:
    """global::stringWithUnitsToDouble: a number with an optional SI prefix and
    unit ("70mm", "100Hz", "344m/s"; a bare prefix + unit such as "mm" is 1 of
    it)."""
    t = text.strip().strip("\"'")
    if t.endswith(unit):
        t = t[: -len(unit)]
    factor = 1.0
    if t and t[-1] in _PREFIX and not re.fullmatch(r"[-+]?[0-9.]+[eE]", t):
        factor = _PREFIX[t[-1]]
        t = t[:-1]
    t = t.strip()
    return (float(t) if t else 1.0) * factor


def _values(text: str, unit: str, n: int):
    parts = [p for p in re.split(r"[ \t,]+", text.strip().strip("\"'")) if p]
    vals = [with_units(p, unit) for p in parts][:n]
    return vals


def _rotation(deg: float, axis: int) -> np.ndarray:
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    R = np.eye(4)
    i, j = [(1, 2), (2, 0), (0, 1)][axis]
    R[i, i], R[i, j], R[j, i], R[j, j] = c, -s, s, c
    return R


def _transform(params):
    """Scale (3 factors) and the 4 x 4 transform of a section's Scale / Shift /
    Rotate lines: scale first, then every Shift / Rotate post-multiplies the
    transform in the order written (QMatrix4x4::translate / rotate)."""
    scale = np.ones(3)
    M = np.eye(4)
    for k, v in params:
        if k == "scale":
            vals = _values(v, "m", 3)
            scale = np.array(vals + [1.0] * (3 - len(vals))) if len(vals) > 1 else \
                np.full(3, vals[0])
            # a zero factor means 1 (ElementSection, elementSection.cpp:147-149)
            scale[scale == 0] = 1.0
        elif k == "shift":
            vals = _values(v, "m", 3) + [0.0, 0.0]
            T = np.eye(4)
            T[:3, 3] = vals[:3]
            M = M @ T
        elif k == "rotate":
            vals = [float(x) for x in re.split(r"[ \t,]+", v.strip()) if x] + [0.0, 0.0]
            for ax in range(3):
                M = M @ _rotation(vals[ax], ax)
    return scale, M


def _apply(points, scale, M):
    p = np.asarray(points, float).reshape(-1, 3) * scale
    return (np.hstack([p, np.ones((p.shape[0], 1))]) @ M.T)[:, :3]


@dataclass
class _Section:
    kind: str
    name: str
    params: list = field(default_factory=list)  # (key, value) in order
    lines: list = field(default_factory=list)   # other lines


def parse_script(text: str) -> list:
    sections, cur = [], None
    for raw in text.splitlines():
        line = raw.split("//", 1)[0].rstrip()
        if not line.strip():
            continue
        toks = line.split()
        off = toks[0].lower() == "off"
        head = toks[1] if off and len(toks) > 1 else toks[0]
        if head.lower() in SECTIONS and (off or not raw[:1].isspace() or cur is None):
            rest = line.split(head, 1)[1].strip().strip("\"'")
            cur = None if off else _Section(head.lower(), rest)
            if cur is not None:
                sections.append(cur)
            continue
        if cur is None:
            continue
        m = re.match(r"\s*\d+\s", line)
        if m:
            cur.lines.append(line.strip())
            continue
        for part in line.split(";"):
            kv = re.match(r"\s*([A-Za-z_]\w*)\s*(?:=\s*(.*))?$", part)
            if kv:
                cur.params.append((kv.group(1).lower(), (kv.group(2) or "").strip()))
    return sections


@dataclass
class Project:
    """A project read from disk: triangles (N x 9), per-element Robin data or
    wall admittance ratios, frequencies, impedance plane, element index and
    section of every triangle."""
    triangles: np.ndarray
    g: np.ndarray
    beta: np.ndarray | None
    frequencies: np.ndarray
    c: float
    rho: float
    plane: tuple | None
    element_index: np.ndarray
    section: list
    sources: list = field(default_factory=list)  # rows x, y, z, weight

    @classmethod
    def load(cls, abec_path: str) -> "Project":
        from . import MshFile, quads_to_triangles, refine_triangles, wall_beta
        base = os.path.dirname(os.path.abspath(abec_path))
        cp = configparser.ConfigParser(interpolation=None, strict=False)
        cp.optionxform = str
        with open(abec_path, encoding="utf-8", errors="replace") as fh:
            cp.read_string("\n".join(l for l in fh.read().splitlines() if not l.startswith(";")))
        script = cp.get("Solving", "Scriptname_Solving")
        aliases = {}
        if cp.has_section("MeshFiles"):
            for _, v in cp.items("MeshFiles"):
                f, a = [x.strip() for x in v.split(",", 1)]
                aliases[a.lower()] = os.path.join(base, f)
        with open(os.path.join(base, script), encoding="utf-8", errors="replace") as fh:
            sections = parse_script(fh.read())
        ctrl = {k: v for s in sections if s.kind == "control_solver" for k, v in s.params}
        c = with_units(ctrl["c"], "m/s") if "c" in ctrl else 0.0
        if c == 0:  # ControlSolverSection::getWavespeed (controlsolversection.cpp:293-299)
            c = 343.21
        rho = with_units(ctrl["rho"], "kg/m^3") if "rho" in ctrl else 1.2041
        f1 = with_units(ctrl.get("f1", "0"), "Hz")
        f2 = with_units(ctrl.get("f2", "0"), "Hz")
        nf = int(float(ctrl.get("numfrequencies", "1")))
        lo, hi = (min(f1, f2), max(f1, f2)) if f1 and f2 else (f1, f2)
        if nf <= 1 or hi == 0:
            freqs = np.array([max(f1, f2)])
        elif ctrl.get("abscissa", "log").lower().startswith("log"):
            d = (math.log(hi) - math.log(lo)) / (nf - 1)
            freqs = np.array([math.exp(math.log(lo) + i * d) for i in range(nf)])
        else:
            freqs = np.array([lo + i * (hi - lo) / (nf - 1) for i in range(nf)])
        alias_scale = {}
        for s in sections:
            if s.kind == "meshfile_properties":
                p = dict(s.params)
                if "meshfilealias" in p and "scale" in p:
                    alias_scale[p["meshfilealias"].strip("\"'").lower()] = \
                        _values(p["scale"], "m", 3)[0]
        # global edge length (ControlSolverSection::getEdgelength,
        # controlsolversection.cpp:301-313): half the wavelength at MeshFrequency,
        # else at the highest of f1, f2
        global_mf = with_units(ctrl["meshfrequency"], "Hz") if "meshfrequency" in ctrl else 0.0
        if global_mf == 0:
            global_mf = max(f1, f2)

        tris, idx, sec_of = [], [], []
        by_name = {}
        for s in sections:
            if s.kind != "elements":
                continue
            scale, M = _transform(s.params)
            swap = False
            alias = None
            mf, edge = 0.0, 0.0
            for k, v in s.params:
                if k == "swapnormals":
                    swap = v == "" or v.lower() in ("1", "true")
                elif k == "meshfilealias":
                    alias = v.strip("\"'").lower()
                elif k == "meshfrequency":
                    mf = with_units(v, "Hz")
                elif k == "edgelength":
                    edge = with_units(v, "m")
            first = len(tris)
            for line in s.lines:
                m = re.match(r"(\d+)\s+Mesh\b(.*)$", line, re.I)
                if not m:
                    continue
                index, rest = int(m.group(1)), m.group(2)
                am = re.search(r"MeshFileAlias\s*=\s*(\S+)", rest, re.I)
                a = (am.group(1).strip("\"'").lower() if am else alias)
                rest = re.sub(r"MeshFileAlias\s*=\s*\S+", "", rest, flags=re.I)
                im = re.search(r"Include(.*?)(?:Exclude(.*))?$", rest, re.I)
                inc = im.group(1).strip() if im else "all"
                exc = (im.group(2) or "").strip() if im else ""
                msh = MshFile(aliases[a])
                sel = msh.select(inc or "all", exc)
                msh.close()
                t = np.vstack([sel["tri"], quads_to_triangles(sel["quad"])])
                t = _apply(t, scale * alias_scale.get(a, 1.0), M).reshape(-1, 9)
                if swap:
                    t = np.hstack([t[:, 6:9], t[:, 3:6], t[:, 0:3]])
                # SolvingScriptReader::refineElements (solvingscriptreader.cpp:
                # 1104-1116): a section's MeshFrequency wins over its EdgeLength;
                # with neither, the global edge length
                e = (c / mf) / 2 if mf > 0 else (
                    edge if edge > 0 else ((c / global_mf) / 2 if global_mf > 0 else 0.0))
                if e > 0 and t.shape[0]:
                    t, _ = refine_triangles(t, e)
                tris.append(t)
                idx.append(np.full(t.shape[0], index))
                sec_of += [s.name] * t.shape[0]
            by_name[s.name.lower()] = (first, len(tris))
        tri = np.vstack(tris) if tris else np.zeros((0, 9))
        eidx = np.concatenate(idx) if idx else np.zeros(0, int)
        offsets = np.cumsum([0] + [x.shape[0] for x in tris])
        members = {name: np.arange(offsets[a], offsets[b]) for name, (a, b) in by_name.items()}
        n = tri.shape[0]
        g = np.zeros(n, complex)
        beta = None
        for s in sections:
            if s.kind == "wallimpedance":
                p = dict(s.params)
                ref = p.get("refelements", "").strip("\"'").lower()
                kind = IMP_TYPES[p.get("imptype", "reflection").strip("\"'").lower()]
                norm = p.get("normalized", "true").lower() not in ("false", "0")
                vals = [float(x) for x in re.split(r"[ \t,]+", p.get("value", "0")) if x]
                val = complex(vals[0], vals[1] if len(vals) > 1 else 0.0)
                if beta is None:
                    beta = np.zeros(n, complex)
                beta[members[ref]] = wall_beta(kind, val, norm, rho * c)
        for s in sections:
            if s.kind == "driving":
                p = dict(s.params)
                ref = p.get("refelements", "").strip("\"'").lower()
                dw = float(p.get("drvweight", "1"))
                for line in s.lines:
                    m = re.match(r"(\d+)\s+(\d+)(.*)$", line)
                    if not m:
                        continue
                    wm = re.search(r"Weight\s*=\s*(\S+)", m.group(3), re.I)
                    w = float(wm.group(1)) if wm else dw
                    sel = members[ref][eidx[members[ref]] == int(m.group(2))]
                    g[sel] = w
                    if beta is not None:
                        beta[sel] = 0.0
        # point sources: Pressure_Points lines "<index> <node> [Weight=w]
        # [RefNodes=name]" at the nodes of a Nodes section (setupPressurePoints,
        # solvingscriptreader.cpp:1016-1050; the weight defaults to DrvWeight)
        nodes = {}
        for s in sections:
            if s.kind == "nodes":
                scale_n, M_n = _transform(s.params)
                pts = {}
                for line in s.lines:
                    tok = line.split()
                    if len(tok) >= 4:
                        pts[int(tok[0])] = _apply([float(x) for x in tok[1:4]], scale_n, M_n)[0]
                nodes[s.name.lower()] = pts
        sources = []
        for s in sections:
            if s.kind == "pressure_points":
                p = dict(s.params)
                dw = float(p.get("drvweight", "1"))
                for line in s.lines:
                    m = re.match(r"(\d+)\s+(\d+)(.*)$", line)
                    if not m:
                        continue
                    wm = re.search(r"Weight\s*=\s*(\S+)", m.group(3), re.I)
                    rm = re.search(r"RefNodes\s*=\s*(\S+)", m.group(3), re.I)
                    ref = (rm.group(1) if rm else p.get("refnodes", "")).strip("\"'").lower()
                    if ref in nodes and int(m.group(2)) in nodes[ref]:
                        x = nodes[ref][int(m.group(2))]
                        sources.append([x[0], x[1], x[2], float(wm.group(1)) if wm else dw])
        plane = None
        for s in sections:
            if s.kind == "infinite_baffle":
                p = dict(s.params)
                plane = (np.array(_values(p.get("position", "0 0 0"), "m", 3)),
                         np.array([float(x) for x in re.split(r"[ \t,]+", p["normal"]) if x]))
                break
        return cls(tri, g, beta, freqs, c, rho, plane, eidx, sec_of, sources)

    def solver(self, **cfg):
        """A Solver with this project's mesh, boundary data and plane."""
        from . import Solver
        s = Solver(**{"wave_speed": self.c, "density": self.rho, **cfg})
        s.set_mesh(self.triangles)
        n = self.triangles.shape[0]
        if self.beta is not None:
            s.set_bc_impedance(self.beta)
        else:
            s.set_bc(np.zeros(n), np.ones(n))
        if self.plane is not None:
            s.set_impedance_plane(*self.plane)
        if self.sources:
            s.set_point_sources(self.sources)
        return s

    def sweep(self, **cfg):
        """Sound pressure on the elements at every frequency (n x nf)."""
        s = self.solver(**cfg)
        p, info = s.sweep(self.frequencies, self.g)
        s.close()
        return p[:, 0, :], info
