"""Drop-in job runner for the reference's `asend_run_job <job.yaml>` on the
linear-elastic static, Newmark and modal path.

It reads the reference's input files with the reference's own line grammar
(solverSrc/asend_run_job/src/model_input.rs:34-119, read_input_line: up to
four heading levels tracked by indentation, values split at spaces, commas
and brackets, '#' comments), runs the commands on the GPU library, and
writes the reference's result files (results_io):

  job file        model_input.rs:121-310 (read_job)
  model file      :312-860 nodes, elements (brick8, brickIM, tet4, shell4),
                  node / element sets (labels, [a, b(, step)) ranges with b
                  excluded, as :456-470), sections (solid, shell with one
                  isotropic layer), materials (density, isotropic E, nu, G)
  constraints     :872-970 (terms of nodeSet / dof / coef, rhs)
  loads           :981-1124 (nodalForce, surfaceTraction; activeTime)
  objective       :1298-1375 (displacement / velocity / acceleration with
                  powerNorm, objective_meth.rs:329-337 and :592-663)
  design vars     :1218-1296 (modulus, shearModulus, poissonRatio components
                  over element sets; hex8 / tet4 meshes)
  commands        model_meth.rs:20-140: readModelInput, readConstraints,
                  readLoads, readObjectiveInput, readDesignVarInput, solvePrep,
                  solve (static or dynamic elastic), zeroSolution,
                  modalAnalysis (frequency), setSolnToMode, calcObjective,
                  calcObjGradient
                  (static), writeNodeResults, writeModalResults,
                  writeObjective (with the _grad file).

Anything outside that subset (thermal, fluid, nonlinear geometry, other
design-variable categories, other element or load types) raises
NotImplementedError naming the item, rather than running something else.  Usage:

    python -m asend3d_gb300.job path/to/job.yaml
"""
from __future__ import annotations

import sys
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

ELEMENT_TYPES = {"brick8": 8, "brickIM": 81, "tet4": 4, "tet10": 10, "shell4": 41, "beam2": 2}
OTHER_ELEMENT_TYPES = ("wedge6", "shell3", "frcFld", "mass", "fl4", "fl6", "fl8", "fl10")


# ---------------------------------------------------------------------------
# the reference's line grammar
# ---------------------------------------------------------------------------
class LineReader:
    """read_input_line (model_input.rs:34-119).  feed(line) returns
    (headings, data, is_key_line); headings holds four levels."""

    def __init__(self):
        self.headings = ["", "", "", ""]
        self.space = [0, 0, 0, 0]

    @staticmethod
    def _tokens(s: str) -> list[str]:
        for ch in ",[]\t\n":
            s = s.replace(ch, " ")
        return [t for t in s.split(" ") if t]

    def feed(self, line: str):
        i = line.find("#")
        if i >= 0:
            line = line[:i]
        line = line + " "
        colon = line.find(":")
        if colon >= 0:
            lead = len(line) - len(line.lstrip(" -\n\t"))
            word = line[lead:colon]
            h, sp = self.headings, self.space
            if h[0] == "" or sp[0] == lead:
                h[:] = [word, "", "", ""]
                sp[:] = [lead, 0, 0, 0]
            elif h[1] == "" or sp[1] == lead:
                h[1:] = [word, "", ""]
                sp[1:] = [lead, 0, 0]
            elif h[2] == "" or sp[2] == lead:
                h[2:] = [word, ""]
                sp[2:] = [lead, 0]
            else:
                h[3] = word
                sp[3] = lead
            return tuple(h), self._tokens(line[colon + 1:]), True
        dash = line.find("- ")
        data = self._tokens(line[dash + 1:]) if dash >= 0 else []
        return tuple(self.headings), data, False


def read_records(path):
    r = LineReader()
    with open(path) as fh:
        for line in fh:
            yield r.feed(line.rstrip("\n"))


def _range(data):
    """A set entry: one label, or [start, end(, step)) with end excluded."""
    if len(data) == 1:
        return [int(data[0])]
    a, b = int(data[0]), int(data[1])
    step = int(data[2]) if len(data) == 3 else 1
    return list(range(a, b, step))


# ---------------------------------------------------------------------------
# input files
# ---------------------------------------------------------------------------
def read_job(path) -> list[dict]:
    cmds: list[dict] = []
    yes = lambda d: "yes" in d[0]
    conv = {"fileName": str, "dynamic": yes, "elastic": yes, "thermal": yes, "diffusion": yes, "fluid": yes,
            "nonlinearGeom": yes, "saveSolnHist": yes, "lumpMass": yes, "userUpdate": yes,
            "loadRampSteps": int, "solverBlockDim": int, "solverBandwidth": int, "maxIterations": int,
            "numModes": int, "mode": int, "newmarkBeta": float, "newmarkGamma": float, "simPeriod": float,
            "convergenceTol": float, "timeStep": float, "targetEigenvalue": float, "maxAmplitude": float,
            "solverMethod": str, "type": str, "solnField": str, "nodeSet": str, "elementSet": str,
            "position": str, "solnHistDir": str}
    lists = {"fields", "properties", "include", "staticLoadTime"}
    for h, data, _ in read_records(path):
        key = h[1]
        if key == "command" and len(data) == 1:
            cmds.append({"command": data[0]})
            continue
        if not cmds:
            continue
        c = cmds[-1]
        if key in lists and len(data) == 1:
            c.setdefault(key, []).append(float(data[0]) if key == "staticLoadTime" else data[0])
        elif key in ("writeModes", "writeGradient") and len(data) == 1:
            c[key] = data[0] == "yes"
        elif key == "timeSteps" and data:
            if len(data) == 1 and data[0] in ("all", "last"):
                c["timeStepTag"] = data[0]
            else:
                c.setdefault("timeSteps", []).extend(_range(data))
        elif key in conv and len(data) == 1:
            f = conv[key]
            c[key] = f(data) if f is yes else f(data[0])
    return cmds


@dataclass
class ModelInput:
    node_labels: list = field(default_factory=list)
    coords: list = field(default_factory=list)
    elem_type: int | None = None
    elem_labels: list = field(default_factory=list)
    conn: list = field(default_factory=list)
    node_sets: dict = field(default_factory=dict)
    elem_sets: dict = field(default_factory=dict)
    sections: list = field(default_factory=list)
    materials: dict = field(default_factory=dict)


def read_model(path) -> ModelInput:
    m = ModelInput()
    cur_set = None
    for h, data, key_line in read_records(path):
        h0, h1, h2, h3 = h
        if h0 == "nodes" and len(data) == 4:
            m.node_labels.append(int(data[0]))
            m.coords.append([float(v) for v in data[1:]])
        elif h0 == "elements":
            if h1 == "type" and len(data) == 1:
                if data[0] in OTHER_ELEMENT_TYPES:
                    raise NotImplementedError(f"element type {data[0]} is not on the GPU path")
                if data[0] not in ELEMENT_TYPES:
                    raise ValueError(f"unrecognized element type: {data[0]}")
                t = ELEMENT_TYPES[data[0]]
                if m.elem_type is not None and m.elem_type != t:
                    raise NotImplementedError("one element type per model")
                m.elem_type = t
            elif h1 == "connectivity" and len(data) > 1:
                m.elem_labels.append(int(data[0]))
                m.conn.append([int(v) for v in data[1:]])
        elif h0 == "sets" and h1 in ("node", "element") and h2 != "":
            sets = m.node_sets if h1 == "node" else m.elem_sets
            if key_line:
                cur_set = sets.setdefault(h2, [])
            elif data and cur_set is not None:
                cur_set.extend(_range(data))
        elif h0 == "sections":
            if h1 == "type" and len(data) == 1:
                m.sections.append({"type": data[0], "layers": []})
            elif not m.sections:
                continue
            elif h1 in ("material", "elementSet") and len(data) == 1:
                m.sections[-1][h1] = data[0]
            elif h1 == "orientation" and len(data) == 6:
                m.sections[-1]["orientation"] = [float(v) for v in data]
            elif h1 == "layup":
                if h2 == "zOffset" and len(data) == 1:
                    m.sections[-1]["zOffset"] = float(data[0])
                elif h2 == "layers" and h3 == "material" and len(data) == 1:
                    m.sections[-1]["layers"].append({"material": data[0]})
                elif h2 == "layers" and h3 in ("thickness", "angle") and len(data) == 1:
                    m.sections[-1]["layers"][-1][h3] = float(data[0])
            elif h1 == "beamProps" and data:
                # model_input.rs:561-596 (J is read from its one value; the
                # reference indexes data[1] there)
                if h2 == "area" and len(data) == 1:
                    m.sections[-1]["area"] = float(data[0])
                elif h2 == "I" and len(data) == 5:
                    m.sections[-1]["I"] = [float(v) for v in data]
                elif h2 == "J" and len(data) == 1:
                    m.sections[-1]["J"] = float(data[0])
                elif h2 in ("stiffness", "mass") and len(data) == 3:
                    # (row, column, value), 1-based, symmetric (section_meth.rs:61-71)
                    mat = m.sections[-1].setdefault(h2, [0.0] * 36)
                    r, c = int(data[0]) - 1, int(data[1]) - 1
                    mat[6 * r + c] = mat[6 * c + r] = float(data[2])
                elif h2 in ("damping", "expLoadCoef"):
                    raise NotImplementedError(f"beam section {h2} entries are not on the GPU path")
            elif h1 in ("potField", "dampField", "thermField") and data:
                raise NotImplementedError(f"section {h1} is not on the GPU path")
        elif h0 == "materials" and h1 != "":
            if h2 == "" and key_line:
                m.materials[h1] = {}
            elif h2 == "density" and len(data) == 1:
                m.materials[h1]["density"] = float(data[0])
            elif h2 == "elastic" and h3 in ("E", "nu", "G") and data:
                vals = [float(v) for v in data]
                m.materials[h1][h3] = vals * 3 if len(vals) == 1 else vals
            elif h2 == "elastic" and h3 == "stiffness" and data:
                raise NotImplementedError("anisotropic stiffness matrices are not on the GPU path")
            elif h2 == "damping" and len(data) == 3:
                # (row, column, value), 1-based, symmetric (model_input.rs:719-723)
                d = m.materials[h1].setdefault("damping", [0.0] * 36)
                i, j, v = int(data[0]) - 1, int(data[1]) - 1, float(data[2])
                d[6 * i + j] = v
                d[6 * j + i] = v
    return m


def read_constraints(path) -> list:
    out = []
    for h, data, _ in read_records(path):
        if h[0] != "constraints":
            continue
        if h[1] == "type" and len(data) == 1:
            if data[0] != "displacement":
                raise NotImplementedError(f"{data[0]} constraints are not on the GPU path")
            out.append({"terms": [], "rhs": 0.0})
        elif not out:
            continue
        elif h[1] == "terms":
            if h[2] == "nodeSet" and len(data) == 1:
                out[-1]["terms"].append([data[0], 1, 1.0])
            elif h[2] == "dof" and len(data) == 1:
                out[-1]["terms"][-1][1] = int(data[0])
            elif h[2] == "coef" and len(data) == 1:
                out[-1]["terms"][-1][2] = float(data[0])
        elif h[1] == "rhs" and len(data) == 1:
            out[-1]["rhs"] = float(data[0])
    return out


def read_loads(path) -> list:
    out = []
    for h, data, _ in read_records(path):
        if h[0] != "loads":
            continue
        if h[1] == "type" and len(data) == 1:
            if data[0] not in ("nodalForce", "surfaceTraction", "surfacePressure", "bodyForce", "gravitational",
                               "centrifugal"):
                raise NotImplementedError(f"{data[0]} loads are not on the GPU path")
            out.append({"type": data[0], "load": [0.0] * 6, "activeTime": [0.0, 1e100], "normTolerance": 1.0,
                        "center": [0.0] * 3, "axis": [0.0, 0.0, 1.0], "angularVelocity": 0.0})
        elif not out:
            continue
        elif h[1] == "load" and data:
            vals = [float(v) for v in data]
            out[-1]["load"][:len(vals)] = vals
        elif h[1] in ("nodeSet", "elementSet") and len(data) == 1:
            out[-1][h[1]] = data[0]
        elif h[1] == "normDir" and len(data) == 3:
            out[-1]["normDir"] = [float(v) for v in data]
        elif h[1] == "normTolerance" and len(data) == 1:
            out[-1]["normTolerance"] = float(data[0])
        elif h[1] == "activeTime" and data:
            out[-1]["activeTime"] = [float(data[0]), float(data[1]) if len(data) > 1 else 1e100]
        elif h[1] in ("center", "axis") and len(data) == 3:  # model_input.rs:1103-1112
            out[-1][h[1]] = [float(v) for v in data]
        elif h[1] == "angularVelocity" and data:
            out[-1]["angularVelocity"] = float(data[0])
    return out


DV_CATEGORIES = ("modulus", "shearModulus", "poissonRatio", "area", "areaMoment", "polarMoment")
ELEMENT_CATEGORIES = ("stress", "strain", "strainEnergy")


def read_design_vars(path) -> list:
    """read_des_var_input (model_input.rs:1218-1296)."""
    out = []
    for h, data, _ in read_records(path):
        if h[0] != "designVariables":
            continue
        if h[1] == "category" and len(data) == 1:
            out.append({"category": data[0], "component": 0, "layer": 0, "coefficients": [],
                        "activeTime": [0.0, 1e100]})
        elif not out:
            continue
        elif h[1] in ("elementSet", "nodeSet") and len(data) == 1:
            out[-1][h[1]] = data[0]
        elif h[1] == "component" and len(data) == 1:
            out[-1]["component"] = int(data[0])
        elif h[1] == "component" and len(data) == 2:
            out[-1]["component"] = (int(data[0]), int(data[1]))
        elif h[1] == "layer" and len(data) == 1:
            out[-1]["layer"] = int(data[0])
        elif h[1] == "coefficients" and len(data) == 1:
            out[-1]["coefficients"].append(float(data[0]))
        elif h[1] == "activeTime" and data:
            out[-1]["activeTime"] = [float(data[0]), float(data[1]) if len(data) > 1 else 1e100]
    return out


def read_objective(path) -> list:
    out = []
    for h, data, _ in read_records(path):
        if h[0] != "objectiveTerms":
            continue
        if h[1] == "category" and len(data) == 1:
            # defaults of ObjectiveTerm::new (objective.rs:45-49)
            out.append({"category": data[0], "operator": "", "component": 0, "layer": 0,
                        "coefficient": 0.0, "exponent": 0.0, "activeTime": [0.0, 1e100], "targets": []})
        elif not out:
            continue
        elif h[1] in ("operator", "elementSet", "nodeSet") and len(data) == 1:
            out[-1][h[1]] = data[0]
        elif h[1] in ("component", "layer") and len(data) == 1:
            out[-1][h[1]] = int(data[0])
        elif h[1] in ("coefficient", "exponent") and len(data) == 1:
            out[-1][h[1]] = float(data[0])
        elif h[1] == "activeTime" and data:
            out[-1]["activeTime"] = [float(data[0]), float(data[1]) if len(data) > 1 else 1e100]
        elif h[1] == "targetValue" and data:
            out[-1]["targets"].extend(float(v) for v in data)
    return out


# ---------------------------------------------------------------------------
# the runner
# ---------------------------------------------------------------------------
def _cg_log(iterations, residual):
    """The reference's solver log lines (matrix_functions.rs:358-359), which
    job scripts scrape for "Total CG iterations:"; the second line carries
    this library's final ||f - A u|| / ||f|| (the reference prints g^T M^-1 g)."""
    print(f"Total CG iterations: {int(iterations)}", flush=True)
    print(f"Final residual norm: {residual!r}", flush=True)

class JobRunner:
    def __init__(self, job_path, device=0):
        self.job_path = Path(job_path)
        self.base = self.job_path.parent
        self.cmds = read_job(job_path)
        self.device = device
        self.model = None
        self.constraints: list = []
        self.loads: list = []
        self.objective: list = []
        self.g = None
        self.solve_cmd: dict = {}
        self.state = None          # {"u", "v", "a"} per node [n, dpn]
        self.hist = None           # saved solution history {"dir", "steps", "dt"}
        self.modal = None
        self.obj_values = None
        self.obj_gradient = None
        self.dvs: list = []
        self.log: list = []

    def _path(self, name):
        p = Path(name)
        return p if p.is_absolute() else (Path.cwd() / p if (Path.cwd() / p).exists() else self.base / p)

    # -- model -> Problem ---------------------------------------------------
    def _problem(self):
        from .mesh import BlockMesh
        from .solver import Problem
        m = self.model
        if m.elem_type is None:
            raise ValueError("the model has no elements")
        nidx = {lab: i for i, lab in enumerate(m.node_labels)}
        self.node_index = nidx
        conn = np.array([[nidx[n] for n in row] for row in m.conn], dtype=np.int32)
        coords = np.array(m.coords, dtype=np.float64)
        mesh = BlockMesh(0, 0, 0, 0.0, 0.0, 0.0, coords, conn, elem_type=m.elem_type)
        eidx = {lab: i for i, lab in enumerate(m.elem_labels)}
        ne = len(m.elem_labels)
        E, nu, rho, thk = (np.full(ne, np.nan) for _ in range(4))
        props = np.full((ne, 9), np.nan)  # E1 E2 E3 nu12 nu13 nu23 G12 G13 G23
        damp = np.zeros((ne, 36))
        ortho = False
        shell_secs = []
        beam = np.full((ne, 10), np.nan)  # area, I1..I5, J, xy-plane direction
        beam_cm = np.zeros((ne, 72))      # given section stiffness, mass (section_meth.rs:61-71)
        for sec in m.sections:
            es = sec.get("elementSet")
            if es is None or es not in m.elem_sets:
                raise ValueError(f"section without a valid elementSet: {sec}")
            els = [eidx[e] for e in m.elem_sets[es]]
            if sec["type"] == "solid":
                mat = m.materials[sec["material"]]
                t = np.nan
            elif sec["type"] == "shell":
                # layup: layers of (material, thickness, angle) about zOffset
                # (get_layer_thk_z / get_layer_q / get_abd, element_properties.rs:75-222, :766-876)
                rows = []
                for lay in sec["layers"]:
                    lm = m.materials[lay["material"]]
                    le, ln = lm.get("E", [np.nan] * 3), lm.get("nu", [np.nan] * 3)
                    lg = lm.get("G", [le[0] / (2 * (1 + ln[0]))] * 3)
                    if "damping" in lm:
                        raise NotImplementedError("material damping takes solid sections")
                    rows.append([le[0], le[1], ln[0], lg[0], lm.get("density", 0.0), lay["thickness"],
                                 lay.get("angle", 0.0) + self._shell_frame_angle(sec)])
                if not rows:
                    raise ValueError(f"shell section without layers: {sec}")
                mat = m.materials[sec["layers"][0]["material"]]
                t = float(sum(r[5] for r in rows))
                r0 = rows[0]
                one_iso = (len(rows) == 1 and sec.get("zOffset", 0.0) == 0.0 and r0[0] == r0[1]
                           and abs(r0[3] - r0[0] / (2 * (1 + r0[2]))) <= 1e-9 * abs(r0[3]))
                if not one_iso:
                    shell_secs.append((els, rows, sec.get("zOffset", 0.0)))
                E[els], nu[els], rho[els], thk[els] = r0[0], r0[2], r0[4], t
                continue
            elif sec["type"] == "beam":
                mat = m.materials[sec["material"]]
                if "damping" in mat:
                    raise NotImplementedError("material damping takes solid sections")
                for e in els:
                    beam[e], flip = self._beam_row(sec, coords[conn[e, 1]] - coords[conn[e, 0]])
                    cm = np.asarray(sec.get("stiffness", [0.0] * 36), float).reshape(6, 6)
                    mm = np.asarray(sec.get("mass", [0.0] * 36), float).reshape(6, 6)
                    if flip:  # the half turn about y: strains (1,-1,1,1,-1,1), velocities (-1,1,-1,-1,1,-1)
                        ts, tm = np.array([1, -1, 1, 1, -1, 1.0]), np.array([-1, 1, -1, -1, 1, -1.0])
                        cm, mm = cm * np.outer(ts, ts), mm * np.outer(tm, tm)
                    beam_cm[e, :36], beam_cm[e, 36:] = cm.ravel(), mm.ravel()
                t = np.nan
            else:
                raise NotImplementedError(f"{sec['type']} sections are not on the GPU path")
            Ev, nv = mat.get("E", [np.nan] * 3), mat.get("nu", [np.nan] * 3)
            G = mat.get("G", [Ev[0] / (2 * (1 + nv[0]))] * 3)
            iso = (len(set(Ev)) == 1 and len(set(nv)) == 1 and len(set(G)) == 1
                   and abs(G[0] - Ev[0] / (2 * (1 + nv[0]))) <= 1e-9 * abs(G[0]))
            if not iso:
                # orthotropic constants through the compliance form (element_properties.rs:648-764)
                if sec["type"] != "solid" or "G" not in mat:
                    raise NotImplementedError("orthotropic materials take solid sections with E, nu and G lists")
                ortho = True
            props[els] = list(Ev) + list(nv) + list(G)
            if "damping" in mat:
                if sec["type"] != "solid":
                    raise NotImplementedError("material damping takes solid sections")
                damp[els] = mat["damping"]
            E[els], nu[els], rho[els], thk[els] = Ev[0], nv[0], mat.get("density", 0.0), t
        if np.isnan(E).any():
            raise ValueError("elements without a section")
        p = Problem(mesh, E, nu, rho, thickness=None if np.isnan(thk).all() else thk)
        if shell_secs:
            p.shell_sections = shell_secs
        if m.elem_type == 2:
            if np.isnan(beam).any():
                raise ValueError("beam2 elements need a beam section")
            p.beam_sections = beam
            if np.any(beam_cm[:, 0] > 0.0) or np.any(beam_cm[:, 36] > 0.0):
                p.beam_section_matrices = (beam_cm[:, :36].copy(), beam_cm[:, 36:].copy())
        if ortho:
            if m.elem_type not in (8, 4, 10):
                raise NotImplementedError("orthotropic materials take hex8 / tet4 / tet10 meshes on the GPU path")
            p.ortho = props
        if np.any(damp):
            if m.elem_type not in (8, 4, 10):
                raise NotImplementedError("material damping takes hex8 / tet4 / tet10 meshes on the GPU path")
            p.damping = (0.0, 0.0, damp)
        for name, labs in m.node_sets.items():
            p.add_node_set(name, [nidx[v] for v in labs])
        if "all" not in m.node_sets:
            p.add_node_set("all", np.arange(len(m.node_labels)))
        for name, labs in m.elem_sets.items():
            p.add_elem_set(name, [eidx[v] for v in labs])
        if "all" not in m.elem_sets:
            p.add_elem_set("all", np.arange(ne))
        for c in self.constraints:
            p.constraints.append(([(s, d, cf) for s, d, cf in c["terms"]], c["rhs"]))
        p.objective = ("compliance",)
        return p

    def _static_loads(self, p, time):
        for ld in self.loads:
            if not (ld["activeTime"][0] <= time <= ld["activeTime"][1]):
                continue
            t = ld["type"]
            if t == "nodalForce":
                p.add_nodal_force(ld["nodeSet"], ld["load"])
            elif t == "surfaceTraction":
                p.add_surface_traction(ld["elementSet"], tuple(ld["normDir"]), tuple(ld["load"][:3]),
                                       norm_tol=ld["normTolerance"])
            elif t == "surfacePressure":
                p.add_surface_pressure(ld["elementSet"], tuple(ld["normDir"]), ld["load"][0],
                                       norm_tol=ld["normTolerance"])
            elif t == "bodyForce":
                p.add_body_force(ld["elementSet"], ld["load"][:3])
            elif t == "gravitational":
                p.add_gravity(ld["elementSet"], ld["load"][:3])
            else:
                p.add_centrifugal(ld["elementSet"], ld["angularVelocity"], ld["center"], ld["axis"])

    def _solver(self, time=0.0):
        from .solver import GpuSolver
        if self.g is not None:
            self.g.close()
        self.problem = self._problem()
        self._static_loads(self.problem, time)
        self.g = GpuSolver(self.problem, device=self.device)
        return self.g

    def _opts(self, cmd):
        from . import _lib
        method = cmd.get("solverMethod", "iterative")
        kw = dict(method=_lib.METHOD_FP64, precond=_lib.PC_JACOBI, rel_tol=cmd.get("convergenceTol", 1e-12))
        if method == "direct":
            kw["rel_tol"] = 1e-12  # a direct solve, replaced by PCG to the FP64 floor
        if cmd.get("maxIterations"):
            kw["max_iter"] = cmd["maxIterations"]
        if self.model.elem_type in (8, 81) and self.problem.mesh.nx > 0:
            kw["precond"] = _lib.PC_MG
        return kw

    # -- commands ------------------------------------------------------------
    def run(self):
        for c in self.cmds:
            name = c["command"]
            fn = getattr(self, "cmd_" + name, None)
            if fn is None:
                raise NotImplementedError(f"job command {name} is not on the GPU path")
            fn(c)
            self.log.append(name)
        if self.g is not None:
            self.g.close()
        return self

    def cmd_readModelInput(self, c):
        self.model = read_model(self._path(c["fileName"]))
        self.node_index = {lab: i for i, lab in enumerate(self.model.node_labels)}

    def cmd_readConstraints(self, c):
        self.constraints.extend(read_constraints(self._path(c["fileName"])))

    def cmd_readLoads(self, c):
        self.loads.extend(read_loads(self._path(c["fileName"])))

    def cmd_readObjectiveInput(self, c):
        self.objective.extend(read_objective(self._path(c["fileName"])))

    def cmd_readDesignVarInput(self, c):
        for dv in read_design_vars(self._path(c["fileName"])):
            if dv["category"] not in DV_CATEGORIES:
                raise NotImplementedError(f"design variable category {dv['category']} is not on the GPU path")
            top = {"area": 5, "polarMoment": 5, "areaMoment": 5}.get(dv["category"], 3)
            low = 0 if dv["category"] in ("area", "polarMoment") else 1  # the reference ignores their component
            if not isinstance(dv["component"], int) or not low <= dv["component"] <= top or "elementSet" not in dv:
                raise ValueError(f"design variable needs an element set and a component {low}-{top}: {dv}")
            self.dvs.append(dv)

    def cmd_calcObjGradient(self, c):
        """model_analysis.rs:1544-1706 (static branch): the adjoint of each
        powerNorm displacement term of exponent 1 (its dL/du is then the
        coefficient on the set's component, whatever the targets), summed;
        each DV's gradient from the strain-pair tensors."""
        from . import _lib
        if self.g is None or self.state is None:
            raise RuntimeError("calcObjGradient before a solve")
        if self.solve_cmd.get("dynamic"):
            raise NotImplementedError("transient objective gradients are not on the GPU path")
        grad = np.zeros(len(self.dvs))
        opts = self._opts(self.solve_cmd)
        for t in self.objective:
            element_term = t["category"] in ELEMENT_CATEGORIES
            if not element_term and (t["category"] != "displacement" or t["operator"] != "powerNorm"
                                     or t["exponent"] != 1.0):
                raise NotImplementedError("gradients of displacement powerNorm terms of exponent 1 and of "
                                          "stress / strain / strainEnergy terms only")
            if not (t["activeTime"][0] <= self.state["time"] <= t["activeTime"][1]):
                continue
            if element_term:
                self.g.set_element_objective(self._term_elements(t), t["category"], t["component"], t["operator"],
                                             t["coefficient"], t["exponent"], t["targets"])
                _, _, rc, st = self.g.adjoint_gradient(want_dLdE=False, **opts)
            else:
                self.g.set_objective(("displacement", t["nodeSet"], t["component"], t["coefficient"]))
                _, _, rc, st = self.g.adjoint_gradient(**opts)
            if rc not in (_lib.ASEND_OK, _lib.ASEND_MAX_ITER):
                raise RuntimeError(f"adjoint solve failed: {st}")
            _cg_log(st["iterations"], st["rel_residual"])
            for i, dv in enumerate(self.dvs):
                if dv["activeTime"][0] <= self.state["time"] <= dv["activeTime"][1]:
                    grad[i] += self.g.material_dv_gradient(dv["category"], dv["component"], dv["elementSet"],
                                                           dv["coefficients"])
        self.obj_gradient = grad

    def cmd_solvePrep(self, c):
        self.solve_cmd.update({k: v for k, v in c.items() if k != "command"})

    def cmd_zeroSolution(self, c):
        self.state = None

    def cmd_solve(self, c):
        from . import _lib
        cmd = dict(self.solve_cmd)
        cmd.update({k: v for k, v in c.items() if k != "command"})
        self.solve_cmd = cmd
        for k in ("thermal", "diffusion", "fluid", "nonlinearGeom"):
            if cmd.get(k):
                raise NotImplementedError(f"{k} analysis is not on the GPU path")
        if cmd.get("userUpdate"):
            raise NotImplementedError("user update hooks are not on the GPU path")
        g = self._solver()
        # lumpMass: row-sum lumped mass in dynamic runs (element_equations.rs:950-971)
        g._check(g.lib.asend_set_lumped_mass(g.ctx, 1 if cmd.get("lumpMass") else 0), "set_lumped_mass")
        dpn = self.problem.mesh.dpn
        n = self.problem.mesh.n_nodes
        if not cmd.get("dynamic"):
            if len(cmd.get("staticLoadTime", [0.0])) > 1:
                raise NotImplementedError("several static load times are not on the GPU path")
            g.assemble(precision=64)
            u, rc, st = g.static_solve(**self._opts(cmd))
            if rc not in (_lib.ASEND_OK, _lib.ASEND_MAX_ITER):
                raise RuntimeError(f"static solve failed: {st}")
            _cg_log(st["iterations"], st["rel_residual"])
            self.state = {"u": u[0].reshape(n, dpn), "v": np.zeros((n, dpn)), "a": np.zeros((n, dpn)),
                          "time": cmd.get("staticLoadTime", [0.0])[0]}
        else:
            dt = cmd["timeStep"]
            beta, gamma = cmd.get("newmarkBeta", 0.25), cmd.get("newmarkGamma", 0.5)
            n_steps = int(round(cmd["simPeriod"] / dt))
            for ld in self.loads:
                if ld["activeTime"] != [0.0, 1e100]:
                    raise NotImplementedError("time-windowed loads in dynamic jobs are not on the GPU path")
            g.assemble(precision=64, dynamic=True, dt=dt, beta=beta, gamma=gamma)
            kw = self._opts(cmd)
            kw["precond"] = _lib.PC_JACOBI if kw["precond"] == _lib.PC_MG else kw["precond"]
            save = bool(cmd.get("saveSolnHist"))
            if save and self.model.elem_type not in (8, 4, 10):
                raise NotImplementedError("solution histories of elements with internal DOF are not written by the "
                                          "GPU path")
            g.keep_history(3)  # the last state's velocity and acceleration, and the solnTStep files
            hist, u, rc, st = g.newmark(np.ones(n_steps), **kw)
            if rc not in (_lib.ASEND_OK, _lib.ASEND_MAX_ITER):
                raise RuntimeError(f"Newmark run failed: {st}")
            _cg_log(st["iterations"], st["rel_residual"])
            _, v, a = g.step_state(n_steps, fields=3)
            self.state = {"u": u.reshape(n, dpn), "v": v.reshape(n, dpn), "a": a.reshape(n, dpn),
                          "time": n_steps * dt}
            if save:  # solnTStep0 (the initial state) .. solnTStep<n_steps> (model_analysis.rs:591-622)
                from .results_io import write_time_step_soln
                d = self._out(cmd.get("solnHistDir", cmd.get("fileName", ".")))
                z = np.zeros((n, dpn))
                write_time_step_soln(d, 0, z, z, z)
                for s in range(1, n_steps + 1):
                    us, vs, as_ = g.step_state(s, fields=3)
                    write_time_step_soln(d, s, us.reshape(n, dpn), vs.reshape(n, dpn), as_.reshape(n, dpn))
                self.hist = {"dir": d, "steps": n_steps, "dt": dt}

    def cmd_modalAnalysis(self, c):
        from . import _lib
        if c.get("type", "frequency") != "frequency":
            raise NotImplementedError("buckling analysis is not on the GPU path")
        g = self.g or self._solver()
        kw = self._opts(c)
        kw["rel_tol"] = 1e-10
        kw.setdefault("max_iter", 100000)
        ev, fr, modes, _, rc, st = g.eigen(c.get("numModes", 10), shift=c.get("targetEigenvalue", 0.0), **kw)
        if rc != _lib.ASEND_OK:
            raise RuntimeError(f"eigen solve did not converge: {st}")
        _cg_log(st["inner_iterations"], st["max_rel_residual"])
        dpn = self.problem.mesh.dpn
        self.modal = {"eig": ev, "freq": fr, "modes": modes.reshape(len(ev), -1, dpn)}

    def cmd_setSolnToMode(self, c):
        """set_soln_to_mode (model_analysis.rs:890-933): the field becomes mode
        `mode` (0-based; the job default is 1, job.rs:97-99) scaled so that its
        largest |component| equals maxAmplitude.  Mode signs are those of the
        eigen solve (largest-magnitude component positive)."""
        if self.modal is None:
            raise RuntimeError("setSolnToMode before modalAnalysis")
        field = c.get("solnField", "displacement")
        k = c.get("mode", 1)
        amp = c.get("maxAmplitude", 1.0)
        if field not in ("displacement", "velocity", "acceleration"):
            print(f"Warning: {field} is not a valid field to Set to a mode. Aborting setSolnToMode()")
            return
        if not 0 <= k < len(self.modal["eig"]):
            raise ValueError(f"mode {k} was not computed")
        mode = self.modal["modes"][k]
        shape = mode.shape
        if self.state is None:
            self.state = {"u": np.zeros(shape), "v": np.zeros(shape), "a": np.zeros(shape), "time": 0.0}
        key = {"displacement": "u", "velocity": "v", "acceleration": "a"}[field]
        self.state[key] = (amp / np.abs(mode).max()) * mode

    @staticmethod
    def _beam_row(sec, axis):
        """The section table row of one beam2 element.  The reference takes the
        element frame from the section orientation (xDir, xyVec; default the
        global axes, section.rs:150) and differentiates along xDir, so a beam
        is only consistent there when xDir lies along the element; the GPU
        element takes x from the element itself.  An xDir opposite to the
        element gives the same frame turned half a turn about y: the odd
        moments I1 = int z and I5 = int yz change sign, and so do the given
        matrices' entries that couple an odd number of the flipped strains
        or velocities.  Returns (row, flipped)."""
        ori = sec.get("orientation", [1.0, 0.0, 0.0, 0.0, 1.0, 0.0])
        x = np.asarray(ori[:3], float)
        x = x / np.linalg.norm(x)
        a = np.asarray(axis, float) / np.linalg.norm(axis)
        c = float(x @ a)
        if abs(c) < 1.0 - 1e-9:
            raise NotImplementedError("beam sections whose orientation x direction is not along the element")
        im = list(sec.get("I", [0.0] * 5))
        if c < 0.0:
            im[0], im[4] = -im[0], -im[4]
        return [sec.get("area", 0.0), *im, sec.get("J", 0.0), *ori[3:6]], c < 0.0

    @staticmethod
    def _shell_frame_angle(sec):
        """Angle [deg] of the section's material x axis (orientation xDir,
        xyVec; correct_orient element_properties.rs:2052-2150) from the
        global x axis, for flat shells in a plane z = const whose local z is
        +z; layer angles are measured from that axis."""
        o = sec.get("orientation")
        if o is None:
            return 0.0
        xd, xy = np.asarray(o[:3], float), np.asarray(o[3:], float)
        zl = np.cross(xd, xy)
        if abs(xd[2]) > 1e-12 * np.linalg.norm(xd) or zl[2] <= 0 or np.hypot(zl[0], zl[1]) > 1e-12 * np.linalg.norm(zl):
            raise NotImplementedError("shell orientations with the local z axis along +z only")
        return float(np.degrees(np.arctan2(xd[1], xd[0])))

    def _term_elements(self, t):
        """Element indices of an element-category term's set."""
        name = t.get("elementSet")
        if name is None or name not in self.problem.elem_sets:
            raise ValueError(f"objective terms of category '{t['category']}' need a valid element set")
        return self.problem.elem_sets[name]

    def cmd_calcObjective(self, c):
        if self.state is None:
            raise RuntimeError("calcObjective before a solve")
        if self.solve_cmd.get("dynamic"):
            raise NotImplementedError("time-integrated objectives of dynamic runs are not on the GPU path")
        vals = []
        fields = {"displacement": "u", "velocity": "v", "acceleration": "a"}
        cent = None
        for t in self.objective:
            if t["category"] in ELEMENT_CATEGORIES:
                # stress / strain / strainEnergy at the element centroids
                # (objective_meth.rs:665-720) with the term's operator
                from .objective import element_term
                if not (t["activeTime"][0] <= self.state["time"] <= t["activeTime"][1]):
                    vals.append(0.0)
                    continue
                if cent is None:
                    cent = self.g.element_fields(0)
                L, _, _ = element_term(*cent, self._term_elements(t), t["category"], t["component"], t["operator"],
                                       t["coefficient"], t["exponent"], t["targets"])
                vals.append(L)
                continue
            if t["category"] not in fields or t["operator"] != "powerNorm":
                raise NotImplementedError(f"objective {t['category']}/{t['operator']} is not on the GPU path")
            arr = self.state[fields[t["category"]]]
            if arr is None:
                raise NotImplementedError(f"{t['category']} of a dynamic run is not kept")
            if not (t["activeTime"][0] <= self.state["time"] <= t["activeTime"][1]):
                vals.append(0.0)
                continue
            if t["component"] < 1:
                raise ValueError("objective term without a component")
            idx = [self.node_index[v] for v in self.model.node_sets[t["nodeSet"]]]
            q = arr[idx, t["component"] - 1]
            tg = np.zeros(len(q))
            if t["targets"]:
                tg[:] = t["targets"][0] if len(t["targets"]) == 1 else t["targets"]
            # objective_meth.rs:329-337: coef * (sum (q - tgt)^p)^(1/p)
            p = t["exponent"]
            with np.errstate(invalid="ignore"):
                vals.append(float(t["coefficient"] * np.power(np.sum(np.power(q - tg, p)), 1.0 / p)))
        self.obj_values = vals

    def cmd_writeNodeResults(self, c):
        from .results_io import write_node_results
        if c.get("timeSteps") or c.get("timeStepTag"):
            return self._write_node_history(c)
        if self.state is None:
            raise RuntimeError("writeNodeResults before a solve")
        fields = {}
        for f in c.get("fields", ["displacement"]):
            if f == "displacement":
                fields[f] = self.state["u"]
            elif f == "reactionForce":
                fields[f] = self._reaction()
            elif f in ("velocity", "acceleration") and self.state[f[0]] is not None:
                fields[f] = self.state[f[0]]
            else:
                raise NotImplementedError(f"node field {f} is not written by the GPU path")
        labels = self.model.node_sets.get(c.get("nodeSet", "all"), self.model.node_labels)
        write_node_results(self._out(c["fileName"]), labels, fields, time=-1.0,
                           rows=[self.node_index[v] for v in labels])

    def _write_node_history(self, c):
        """writeNodeResults for saved time steps (model_meth.rs:91-110,
        model_output.rs:84-130): per step the solnTStep file is read back and
        written to <name>_timestep<N><ext>, time = N dt."""
        from .results_io import read_time_step_soln, write_node_results
        h = self.hist
        if h is None:
            raise RuntimeError("writeNodeResults for time steps needs a dynamic solve with saveSolnHist")
        tag = c.get("timeStepTag")
        steps = list(range(h["steps"] + 1)) if tag == "all" else [h["steps"]] if tag == "last" else c["timeSteps"]
        n, dpn = len(self.model.node_labels), self.problem.mesh.dpn
        labels = self.model.node_sets.get(c.get("nodeSet", "all"), self.model.node_labels)
        name = c["fileName"]
        i = name.find(".")
        root, ext = (name[:i], name[i:]) if i >= 0 else (name, "")
        for ts in steps:
            u, v, a, _ = read_time_step_soln(h["dir"], ts, n, dpn)
            fields = {}
            for f in c.get("fields", ["displacement"]):
                if f in ("displacement", "velocity", "acceleration"):
                    fields[f] = {"displacement": u, "velocity": v, "acceleration": a}[f]
                else:
                    raise NotImplementedError(f"node field {f} of a time step is not written by the GPU path")
            write_node_results(self._out(f"{root}_timestep{ts}{ext}"), labels, fields, time=h["dt"] * ts,
                               rows=[self.node_index[v_] for v_ in labels])

    def _reaction(self):
        """R(u) = K u (element internal forces, model_output.rs:207-216 with
        build_elastic_soln_load, model_analysis.rs:179-201): the operator
        product minus its penalty part."""
        from . import _lib
        if self.g is None or self.state is None:
            raise RuntimeError("reaction forces before a solve")
        if self.solve_cmd.get("dynamic"):
            raise NotImplementedError("reaction forces of a dynamic run are not written by the GPU path")
        u = self.state["u"].ravel()
        rp, col, val = self.g.csr(2)
        r = np.add.reduceat(val * u[col], rp[:-1])
        return r.reshape(self.state["u"].shape)

    def _out(self, name):
        p = Path(name)
        return p if p.is_absolute() else Path.cwd() / p

    def cmd_writeModalResults(self, c):
        from .results_io import write_modal_results
        if self.modal is None:
            raise RuntimeError("writeModalResults before modalAnalysis")
        write_modal_results(str(self._out(c["fileName"])), self.modal["eig"], self.modal["freq"],
                            modes=self.modal["modes"] if c.get("writeModes") else None,
                            labels=self.model.node_labels)

    def cmd_writeObjective(self, c):
        from .results_io import write_objective
        if self.obj_values is None:
            raise RuntimeError("writeObjective before calcObjective")
        grad = None
        if c.get("writeGradient"):
            if self.obj_gradient is None:
                raise RuntimeError("writeGradient before calcObjGradient")
            grad = self.obj_gradient
        write_objective(str(self._out(c["fileName"])), self.obj_values, self.objective, c.get("include", ()),
                        gradient=grad)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("usage: python -m asend3d_gb300.job <job.yaml>", file=sys.stderr)
        return 2
    JobRunner(argv[0]).run()
    return 0


if __name__ == "__main__":
    sys.exit(main())
