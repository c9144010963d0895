"""Job-file drop-in: the reference's line grammar (model_input.rs:34-119), its
job / model / constraint / load / objective readers, the Problem built from
them, objective evaluation (objective_meth.rs:329-337) and the result files.
Input files are written here in the layout the reference's Python layer
produces (PyYAML block style, rows as bracketed strings with the quotes
removed, asendUtils/model/Model.py:467-480).  The GPU run of a whole job is
in test_gpu_job.py."""
from pathlib import Path

import numpy as np
import pytest

from asend3d_gb300 import job as J
from asend3d_gb300.mesh import block_hex8


def write_cantilever_job(d: Path, nx=4, ny=1, nz=1, L=4.0, etype="brickIM", modal=True, dvs=False):
    """A cantilever of nx*ny*nz hex elements clamped at x = 0 with a -z tip
    load of 2 spread over the tip nodes, mean tip deflection objective."""
    m = block_hex8(nx, ny, nz, L, 1.0, 0.5)
    lines = ["nodes:"]
    lines += [f"- [{i}, {float(x)!r}, {float(y)!r}, {float(z)!r}]" for i, (x, y, z) in enumerate(m.coords)]
    lines += ["elements:", f"- type: {etype}", "  connectivity:"]
    lines += ["  - [" + ", ".join(str(v) for v in [e, *row]) + "]" for e, row in enumerate(m.conn)]
    xmin = m.nodes_in_range(xr=(-1e-9, 1e-9))
    xmax = m.nodes_in_range(xr=(L - 1e-9, L + 1e-9))
    lines += ["sets:", "  node:", "    xMin:"] + [f"    - {v}" for v in xmin]
    lines += ["    xMax:"] + [f"    - {v}" for v in xmax]
    lines += ["  element:", "    all:", f"    - [0, {m.n_elems}]"]
    lines += ["sections:", "- type: solid", "  material: mat1", "  elementSet: all"]
    lines += ["materials:", "  mat1:   # isotropic", "    density: 1.0", "    elastic:",
              "      E: [1000000.0]", "      nu: 0.0", "      G: 500000.0"]
    (d / "model.yaml").write_text("\n".join(lines) + "\n")
    cons = ["constraints:"]
    for dof in (1, 2, 3):
        cons += ["- type: displacement", "  terms:", "  - nodeSet: xMin", f"    dof: {dof}", "    coef: 1.0",
                 "  rhs: 0.0"]
    (d / "constraints.yaml").write_text("\n".join(cons) + "\n")
    f = float(-2.0 / len(xmax))
    (d / "loads.yaml").write_text("loads:\n- type: nodalForce\n  nodeSet: xMax\n"
                                  f"  load: [0.0, 0.0, {f!r}, 0.0, 0.0, 0.0]\n")
    (d / "objective.yaml").write_text("objectiveTerms:\n- category: displacement\n  operator: powerNorm\n"
                                      f"  nodeSet: xMax\n  component: 3\n  coefficient: {float(1.0 / len(xmax))!r}\n"
                                      "  exponent: 1.0\n")
    (d / "dvars.yaml").write_text(
        "designVariables:\n"
        "- category: modulus\n  component: 1\n  layer: 0\n  elementSet: all\n  coefficients: 1.0\n"
        "- category: shearModulus\n  component: 2\n  elementSet: all\n"
        "- category: poissonRatio\n  component: 3\n  elementSet: all\n  coefficients:\n"
        + "".join(f"  - {v}\n" for v in (2.0, 3.0, 4.0, 5.0)))
    job = ["jobCommands:",
           "- command: readModelInput", "  fileName: model.yaml",
           "- command: readConstraints", "  fileName: constraints.yaml",
           "- command: readLoads", "  fileName: loads.yaml",
           "- command: readObjectiveInput", "  fileName: objective.yaml"]
    if dvs:
        job += ["- command: readDesignVarInput", "  fileName: dvars.yaml"]
    job += ["- command: solve", "  elastic: yes", "  dynamic: no", "  solverMethod: iterative",
           "  convergenceTol: 1.0e-11", "  maxIterations: 20000",
           "- command: calcObjective",
           "- command: writeNodeResults", f"  fileName: {d / 'nodes.csv'}", "  nodeSet: xMax",
           "  fields:", "  - displacement", "  - reactionForce",
    ]
    if dvs:
        job += ["- command: calcObjGradient"]
    job += ["- command: writeObjective", f"  fileName: {d / 'obj.csv'}", "  include:", "  - category",
            "  - coefficient"] + (["  writeGradient: yes"] if dvs else [])
    if modal:
        job += ["- command: modalAnalysis", "  type: frequency", "  numModes: 3",
                "- command: writeModalResults", f"  fileName: {d / 'modal.csv'}", "  writeModes: yes"]
    (d / "job.yaml").write_text("\n".join(job) + "\n")
    return m, xmin, xmax


def test_line_grammar():
    r = J.LineReader()
    assert r.feed("nodes:") == (("nodes", "", "", ""), [], True)
    assert r.feed("- [3, 1.5, -2e-3, 0.0]  # comment") == (("nodes", "", "", ""), ["3", "1.5", "-2e-3", "0.0"], False)
    assert r.feed("sets:")[0] == ("sets", "", "", "")
    assert r.feed("  node:")[0] == ("sets", "node", "", "")
    assert r.feed("    tip:")[0] == ("sets", "node", "tip", "")
    assert r.feed("    - [0, 10, 2]")[1] == ["0", "10", "2"]
    r.feed("sections:")
    assert r.feed("- type: shell")[:2] == (("sections", "type", "", ""), ["shell"])
    assert r.feed("  layup:")[0] == ("sections", "layup", "", "")
    assert r.feed("    layers:")[0] == ("sections", "layup", "layers", "")
    assert r.feed("    - material: al")[:2] == (("sections", "layup", "layers", "material"), ["al"])
    assert r.feed("      thickness: 0.1")[:2] == (("sections", "layup", "layers", "thickness"), ["0.1"])
    assert r.feed("  elementSet: all")[:2] == (("sections", "elementSet", "", ""), ["all"])
    assert J._range(["0", "10", "3"]) == [0, 3, 6, 9]


def test_readers(tmp_path):
    m, xmin, xmax = write_cantilever_job(tmp_path)
    cmds = J.read_job(tmp_path / "job.yaml")
    assert [c["command"] for c in cmds] == ["readModelInput", "readConstraints", "readLoads", "readObjectiveInput",
                                            "solve", "calcObjective", "writeNodeResults", "writeObjective",
                                            "modalAnalysis", "writeModalResults"]
    assert cmds[4]["elastic"] is True and cmds[4]["dynamic"] is False and cmds[4]["convergenceTol"] == 1e-11
    assert cmds[4]["maxIterations"] == 20000
    assert cmds[6]["fields"] == ["displacement", "reactionForce"] and cmds[9]["writeModes"] is True
    mi = J.read_model(tmp_path / "model.yaml")
    assert mi.elem_type == 81 and mi.node_labels == list(range(m.n_nodes))
    np.testing.assert_array_equal(np.array(mi.coords), m.coords)
    np.testing.assert_array_equal(np.array(mi.conn), m.conn)
    assert mi.node_sets["xMin"] == list(xmin) and mi.elem_sets["all"] == list(range(m.n_elems))
    assert mi.materials["mat1"] == {"density": 1.0, "E": [1e6] * 3, "nu": [0.0] * 3, "G": [5e5] * 3}
    assert mi.sections == [{"type": "solid", "layers": [], "material": "mat1", "elementSet": "all"}]
    cons = J.read_constraints(tmp_path / "constraints.yaml")
    assert [c["terms"] for c in cons] == [[["xMin", d, 1.0]] for d in (1, 2, 3)]
    loads = J.read_loads(tmp_path / "loads.yaml")
    assert loads[0]["type"] == "nodalForce" and loads[0]["load"][2] == pytest.approx(-2.0 / len(xmax))
    obj = J.read_objective(tmp_path / "objective.yaml")
    assert obj[0]["component"] == 3 and obj[0]["exponent"] == 1.0 and obj[0]["nodeSet"] == "xMax"


def test_problem_from_job(tmp_path):
    m, xmin, xmax = write_cantilever_job(tmp_path)
    r = J.JobRunner(tmp_path / "job.yaml")
    for c in r.cmds[:4]:
        getattr(r, "cmd_" + c["command"])(c)
    p = r._problem()
    r._static_loads(p, 0.0)
    assert p.mesh.elem_type == 81
    np.testing.assert_array_equal(p.mesh.conn, m.conn)
    assert np.all(p.E == 1e6) and np.all(p.nu == 0.0) and np.all(p.rho == 1.0)
    np.testing.assert_array_equal(p.node_sets["xMin"], xmin)
    assert len(p.constraints) == 3 and p.loads[0][0][0] == "nodalForce"


def test_objective_and_writers(tmp_path):
    m, xmin, xmax = write_cantilever_job(tmp_path)
    r = J.JobRunner(tmp_path / "job.yaml")
    for c in r.cmds[:4]:
        getattr(r, "cmd_" + c["command"])(c)
    r.problem = r._problem()
    n = m.n_nodes
    u = np.zeros((n, 3))
    u[xmax, 2] = -8.0
    r.state = {"u": u, "v": np.zeros((n, 3)), "a": np.zeros((n, 3)), "time": 0.0}
    r.cmd_calcObjective({})
    assert r.obj_values == [pytest.approx(-8.0)]
    r.objective[0]["exponent"] = 2.0
    r.objective[0]["targets"] = [-7.0]
    r.cmd_calcObjective({})
    # coef * (sum (q - t)^2)^(1/2) over the tip nodes
    assert r.obj_values[0] == pytest.approx(np.sqrt(len(xmax)) / len(xmax))
    r.cmd_writeObjective({"fileName": str(tmp_path / "o.csv"), "include": ["category"]})
    assert (tmp_path / "o.csv").read_text().splitlines()[1].startswith("0,")
    with pytest.raises(RuntimeError, match="calcObjGradient"):
        r.cmd_writeObjective({"fileName": str(tmp_path / "o.csv"), "writeGradient": True})
    r.obj_gradient = np.array([-8e-6, 1.0])
    r.cmd_writeObjective({"fileName": str(tmp_path / "o.csv"), "writeGradient": True})
    assert (tmp_path / "o_grad.csv").read_text() == "designVariable,objGrad\n0,-8.000000000000e-6\n1,1.000000000000e0\n"


def test_design_var_reader(tmp_path):
    write_cantilever_job(tmp_path, dvs=True)
    dvs = J.read_design_vars(tmp_path / "dvars.yaml")
    assert dvs == [{"category": "modulus", "component": 1, "layer": 0, "coefficients": [1.0], "activeTime": [0.0, 1e100],
                    "elementSet": "all"},
                   {"category": "shearModulus", "component": 2, "layer": 0, "coefficients": [], "activeTime": [0.0, 1e100],
                    "elementSet": "all"},
                   {"category": "poissonRatio", "component": 3, "layer": 0, "coefficients": [2.0, 3.0, 4.0, 5.0],
                    "activeTime": [0.0, 1e100], "elementSet": "all"}]
    r = J.JobRunner(tmp_path / "job.yaml")
    r.cmd_readDesignVarInput({"fileName": "dvars.yaml"})
    assert len(r.dvs) == 3
    (tmp_path / "bad.yaml").write_text("designVariables:\n- category: nodeCoord\n  component: 1\n  nodeSet: xMax\n")
    with pytest.raises(NotImplementedError, match="nodeCoord"):
        r.cmd_readDesignVarInput({"fileName": "bad.yaml"})


def test_unsupported_inputs(tmp_path):
    (tmp_path / "m.yaml").write_text("elements:\n- type: shell3\n")
    with pytest.raises(NotImplementedError, match="shell3"):
        J.read_model(tmp_path / "m.yaml")
    (tmp_path / "l.yaml").write_text("loads:\n- type: bodyHeatGen\n")
    with pytest.raises(NotImplementedError, match="bodyHeatGen"):
        J.read_loads(tmp_path / "l.yaml")
    (tmp_path / "j.yaml").write_text("jobCommands:\n- command: solve\n  thermal: yes\n")
    r = J.JobRunner(tmp_path / "j.yaml")
    r.model = J.ModelInput()
    with pytest.raises(NotImplementedError, match="thermal"):
        r.cmd_solve(r.cmds[0])
    for key, msg in (("userUpdate", "user update"),):
        (tmp_path / "j.yaml").write_text(f"jobCommands:\n- command: solve\n  dynamic: yes\n  {key}: yes\n")
        r = J.JobRunner(tmp_path / "j.yaml")
        r.model = J.ModelInput()
        with pytest.raises(NotImplementedError, match=msg):
            r.cmd_solve(r.cmds[0])


def test_set_soln_to_mode(tmp_path):
    m, xmin, xmax = write_cantilever_job(tmp_path)
    r = J.JobRunner(tmp_path / "job.yaml")
    for c in r.cmds[:4]:
        getattr(r, "cmd_" + c["command"])(c)
    n = m.n_nodes
    rng = np.random.default_rng(1)
    modes = rng.standard_normal((3, n, 3))
    r.modal = {"eig": np.array([1.0, 2.0, 3.0]), "freq": np.zeros(3), "modes": modes}
    r.cmd_setSolnToMode({})  # defaults: displacement, mode 1, amplitude 1
    np.testing.assert_allclose(r.state["u"], modes[1] / np.abs(modes[1]).max())
    r.cmd_setSolnToMode({"solnField": "velocity", "mode": 2, "maxAmplitude": 0.5})
    assert np.abs(r.state["v"]).max() == pytest.approx(0.5)
    np.testing.assert_allclose(r.state["u"], modes[1] / np.abs(modes[1]).max())
    r.cmd_writeNodeResults({"fileName": str(tmp_path / "m.csv"), "fields": ["displacement", "velocity"]})
    lines = (tmp_path / "m.csv").read_text().splitlines()
    assert len(lines) == n + 1 and lines[0].startswith("node,U1,U2,U3,R1,R2,R3,V1")
    r.cmd_setSolnToMode({"solnField": "stress"})  # the reference warns and leaves the state
    with pytest.raises(ValueError):
        r.cmd_setSolnToMode({"mode": 7})


def test_cg_log_lines(capsys):
    """Job scripts sum the integer after "Total CG iterations:" (the
    reference's matrix_functions.rs:358-359 lines)."""
    J._cg_log(25, 3.5e-9)
    out = capsys.readouterr().out.splitlines()
    assert out == ["Total CG iterations: 25", "Final residual norm: 3.5e-09"]
    assert int(out[0].split(":")[1]) == 25


def write_shell_job(d: Path, nx=3, ny=2, t=0.004, z_offset=0.0, layers=1):
    from asend3d_gb300.mesh import plate_quad4
    m = plate_quad4(nx, ny, 0.6, 0.4)
    lines = ["nodes:"] + [f"- [{i}, {float(x)!r}, {float(y)!r}, {float(z)!r}]" for i, (x, y, z) in enumerate(m.coords)]
    lines += ["elements:", "- type: shell4", "  connectivity:"]
    lines += ["  - [" + ", ".join(str(v) for v in [e, *row]) + "]" for e, row in enumerate(m.conn)]
    lines += ["sets:", "  node:", "    edge:"] + [f"    - {v}" for v in m.nodes_in_range(xr=(-1e-9, 1e-9))]
    lines += ["  element:", "    all:", f"    - [0, {m.n_elems}]"]
    lines += ["sections:", "- type: shell", "  layup:", f"    zOffset: {z_offset}", "    layers:"]
    for _ in range(layers):
        lines += ["    - material: al", f"      thickness: {t}", "      angle: 0.0"]
    lines += ["  elementSet: all", "materials:", "  al:", "    density: 2700.0", "    elastic:",
              "      E: 70000000000.0", "      nu: 0.33"]
    (d / "model.yaml").write_text("\n".join(lines) + "\n")
    (d / "job.yaml").write_text("jobCommands:\n- command: readModelInput\n  fileName: model.yaml\n")
    return m


def test_shell_job_problem(tmp_path):
    m = write_shell_job(tmp_path)
    r = J.JobRunner(tmp_path / "job.yaml")
    r.cmd_readModelInput(r.cmds[0])
    assert r.model.sections[0]["layers"] == [{"material": "al", "thickness": 0.004, "angle": 0.0}]
    p = r._problem()
    assert p.mesh.elem_type == 41 and p.mesh.dpn == 6
    np.testing.assert_array_equal(p.thickness, np.full(m.n_elems, 0.004))
    assert np.all(p.E == 70e9) and np.all(p.rho == 2700.0)
    assert p.shell_sections is None  # one centred isotropic layer: the E, nu, t section
    # several layers or an offset: a layered section per element set
    for kw in (dict(layers=2), dict(z_offset=-1.0)):
        d = tmp_path / f"lay{kw.get('layers', 1)}"
        d.mkdir()
        write_shell_job(d, **kw)
        rb = J.JobRunner(d / "job.yaml")
        rb.cmd_readModelInput(rb.cmds[0])
        pb = rb._problem()
        (els, rows, zoff), = pb.shell_sections
        assert len(els) == m.n_elems and len(rows) == kw.get("layers", 1) and zoff == kw.get("z_offset", 0.0)
        assert rows[0][:6] == [70e9, 70e9, 0.33, 70e9 / 2.66, 2700.0, 0.004]
        np.testing.assert_allclose(pb.thickness, 0.004 * kw.get("layers", 1))


def write_beam_job(d: Path, n=20, reverse=False, x_dir=(1.0, 0.0, 0.0), moments=(0.0, 0.0), given=()):
    """The hexBeam / shellBeam cantilever as a line of beam2 elements (L = 10,
    b = 1, h = 0.1, E = 1e6, nu = 0), clamped at x = 0, Fz = 2 at the tip;
    ``reverse`` numbers every element from its outer node to its inner one."""
    from asend3d_gb300.mesh import line_beam2
    m = line_beam2(n, 10.0)
    if reverse:
        m.conn = m.conn[:, ::-1].copy()
    lines = ["nodes:"] + [f"- [{i}, {float(x)!r}, {float(y)!r}, {float(z)!r}]" for i, (x, y, z) in enumerate(m.coords)]
    lines += ["elements:", "- type: beam2", "  connectivity:"]
    lines += ["  - [" + ", ".join(str(v) for v in [e, *row]) + "]" for e, row in enumerate(m.conn)]
    lines += ["sets:", "  node:", "    root:", "    - 0", "    tip:", f"    - {n}"]
    lines += ["  element:", "    all:", f"    - [0, {n}]"]
    lines += ["sections:", "- type: beam", "  material: mat1", "  elementSet: all",
              "  orientation: [" + ", ".join(repr(float(v)) for v in (*x_dir, 0.0, 1.0, 0.0)) + "]",
              "  beamProps:", "    area: 0.1",
              f"    I: [{moments[0]!r}, 0.0, {1.0 * 0.1**3 / 12!r}, {0.1 * 1.0**3 / 12!r}, {moments[1]!r}]",
              "    J: 0.00028"] + [f"    {kind}: [{r}, {c}, {v!r}]" for kind, r, c, v in given] + [
              "materials:", "  mat1:", "    density: 1.0", "    elastic:", "      E: [1000000.0]", "      nu: 0.0"]
    (d / "model.yaml").write_text("\n".join(lines) + "\n")
    cons = ["constraints:"]
    for dof in range(1, 7):
        cons += ["- type: displacement", "  terms:", "  - nodeSet: root", f"    dof: {dof}", "    coef: 1.0",
                 "  rhs: 0.0"]
    (d / "constraints.yaml").write_text("\n".join(cons) + "\n")
    (d / "loads.yaml").write_text("loads:\n- type: nodalForce\n  nodeSet: tip\n  load: [0.0, 0.0, 2.0, 0.0, 0.0, 0.0]\n")
    (d / "objective.yaml").write_text("objectiveTerms:\n- category: displacement\n  operator: powerNorm\n"
                                      "  nodeSet: tip\n  component: 3\n  coefficient: 1.0\n  exponent: 1.0\n")
    job = ["jobCommands:",
           "- command: readModelInput", "  fileName: model.yaml",
           "- command: readConstraints", "  fileName: constraints.yaml",
           "- command: readLoads", "  fileName: loads.yaml",
           "- command: readObjectiveInput", "  fileName: objective.yaml",
           "- command: solve", "  elastic: yes", "  dynamic: no", "  solverMethod: iterative",
           "  convergenceTol: 1.0e-12", "  maxIterations: 400000",
           "- command: calcObjective",
           "- command: writeNodeResults", f"  fileName: {d / 'nodes.csv'}", "  nodeSet: tip",
           "  fields:", "  - displacement",
           "- command: writeObjective", f"  fileName: {d / 'obj.csv'}"]
    (d / "job.yaml").write_text("\n".join(job) + "\n")
    return m


def test_beam_job_problem(tmp_path):
    """beamProps and orientation reach the section table; an element numbered
    against the section's x direction flips the odd moments I1 and I5."""
    write_beam_job(tmp_path, moments=(1e-3, 2e-5))
    r = J.JobRunner(tmp_path / "job.yaml")
    r.cmd_readModelInput(r.cmds[0])
    sec = r.model.sections[0]
    assert sec["area"] == 0.1 and sec["J"] == 0.00028 and len(sec["I"]) == 5
    p = r._problem()
    assert p.mesh.elem_type == 2 and p.mesh.dpn == 6
    assert p.beam_sections.shape == (20, 10)
    np.testing.assert_allclose(p.beam_sections[0], [0.1, 1e-3, 0.0, 0.1**3 / 12, 0.1 / 12, 2e-5, 0.00028, 0, 1, 0])
    d = tmp_path / "rev"
    d.mkdir()
    write_beam_job(d, reverse=True, moments=(1e-3, 2e-5))
    rb = J.JobRunner(d / "job.yaml")
    rb.cmd_readModelInput(rb.cmds[0])
    pb = rb._problem()
    np.testing.assert_allclose(pb.beam_sections[:, [1, 5]], np.tile([-1e-3, -2e-5], (20, 1)))
    # a section x direction across the element is not a consistent beam
    d2 = tmp_path / "skew"
    d2.mkdir()
    write_beam_job(d2, x_dir=(1.0, 1.0, 0.0))
    rs = J.JobRunner(d2 / "job.yaml")
    rs.cmd_readModelInput(rs.cmds[0])
    with pytest.raises(NotImplementedError, match="along the element"):
        rs._problem()


def test_beam_job_given_matrices(tmp_path):
    """beamProps stiffness / mass entries (1-based, symmetric) become given
    section matrices; an element against the orientation's x direction gets
    them in its own frame (the half turn about y flips the couplings of an odd
    number of flipped components)."""
    given = [("stiffness", 1, 1, 1e5), ("stiffness", 1, 5, 3.0), ("stiffness", 5, 5, 90.0),
             ("mass", 1, 1, 0.1), ("mass", 2, 4, 0.002)]
    write_beam_job(tmp_path, n=4, given=given)
    r = J.JobRunner(tmp_path / "job.yaml")
    r.cmd_readModelInput(r.cmds[0])
    st = np.array(r.model.sections[0]["stiffness"]).reshape(6, 6)
    assert st[0, 0] == 1e5 and st[0, 4] == st[4, 0] == 3.0 and st[4, 4] == 90.0
    p = r._problem()
    C, M = p.beam_section_matrices
    np.testing.assert_array_equal(C[0].reshape(6, 6), st)
    assert M[0].reshape(6, 6)[1, 3] == M[0].reshape(6, 6)[3, 1] == 0.002
    d = tmp_path / "rev"
    d.mkdir()
    write_beam_job(d, n=4, reverse=True, given=given)
    rb = J.JobRunner(d / "job.yaml")
    rb.cmd_readModelInput(rb.cmds[0])
    Cr, Mr = rb._problem().beam_section_matrices
    assert Cr[0].reshape(6, 6)[0, 4] == -3.0 and Cr[0].reshape(6, 6)[4, 4] == 90.0
    assert Mr[0].reshape(6, 6)[1, 3] == -0.002 and Mr[0].reshape(6, 6)[0, 0] == 0.1
