"""A whole job file through the drop-in runner on the GPU: static solve,
objective, node results (displacement and reaction force), modal analysis
and the result files, against the oracle on the same model.

Tolerances: displacements and reactions 1e-8 relative to their largest
entry (PCG to 1e-11 on a 4-element beam); the objective 1e-8; frequencies
1e-5 against the oracle's genuine Ritz pairs (its power-iteration
accuracy); the tip deflection against Euler-Bernoulli FL^3 / 3EI = 4.096e-3
within 3 % (L/h = 8: shear deformation adds about 1 %)."""
import numpy as np
import pytest

from asend3d_gb300 import job as J
from asend3d_gb300.solver import Problem

from eigen_cases import dense_reference, genuine_pairs
from test_job import write_beam_job, write_cantilever_job

pytestmark = pytest.mark.gpu


def read_csv(path):
    lines = path.read_text().splitlines()
    return lines[0].split(","), np.array([[float(v) for v in ln.split(",")] for ln in lines[1:]])


def test_job_static_and_modal(gpu_lib, oracle_lib, tmp_path):
    m, xmin, xmax = write_cantilever_job(tmp_path)
    r = J.JobRunner(tmp_path / "job.yaml").run()
    assert r.log[-1] == "writeModalResults"
    # the same model through the oracle
    m.elem_type = 81
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), np.full(m.n_elems, 1.0))
    p.add_node_set("xMin", xmin)
    p.add_node_set("xMax", xmax)
    p.fix_displacement("xMin")
    p.add_nodal_force("xMax", [0.0, 0.0, -2.0 / len(xmax)])
    o = oracle_lib.Oracle(p)
    uo, rc, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    uo = uo.reshape(-1, 3)
    head, rows = read_csv(tmp_path / "nodes.csv")
    assert head == ["node", "U1", "U2", "U3", "R1", "R2", "R3", "RF1", "RF2", "RF3", "RM1", "RM2", "RM3", "time"]
    np.testing.assert_array_equal(rows[:, 0], xmax)
    assert np.abs(rows[:, 1:4] - uo[xmax]).max() <= 1e-8 * np.abs(uo).max()
    assert np.all(rows[:, 4:7] == 0.0) and np.all(rows[:, -1] == -1.0)
    rp, col, val = o.csr(0)  # K without the penalty terms
    ku = np.add.reduceat(val * uo.ravel()[col], rp[:-1]).reshape(-1, 3)
    assert np.abs(rows[:, 7:10] - ku[xmax]).max() <= 1e-8 * np.abs(ku).max()
    # the tip carries the applied load as its internal force
    np.testing.assert_allclose(rows[:, 9].sum(), -2.0, rtol=1e-8)
    lines = (tmp_path / "obj.csv").read_text().splitlines()
    assert lines[0] == "objectiveTerm,value,category,coefficient"
    w = float(lines[1].split(",")[1])
    assert w == pytest.approx(uo[xmax, 2].mean(), rel=1e-8)
    assert w == pytest.approx(-4.096e-3, rel=0.03)
    # modal results against the oracle's frequency job
    om = oracle_lib.Oracle(p, modal=True)
    evo, fro, _, _ = om.eigen(3)
    ref, _, _, _ = dense_reference(om, 6)
    head, modal = read_csv(tmp_path / "modal.csv")
    assert head == ["mode", "eigenvalue", "frequency"]
    np.testing.assert_allclose(modal[:, 1], ref[:3], rtol=1e-8)
    for k, j in genuine_pairs(evo, ref):
        if j < 3:
            assert modal[j, 1] == pytest.approx(evo[k], rel=1e-5)
    np.testing.assert_allclose(modal[:, 2], np.sqrt(modal[:, 1]) / (2 * np.pi), rtol=1e-12)
    mode0 = (tmp_path / "modal_mode0.csv").read_text().splitlines()
    assert mode0[0] == "Node,U1,U2,U3,R1,R2,R3" and len(mode0) == m.n_nodes + 1


def test_cli_matches_python_runner(gpu_lib, tmp_path):
    """The C++ asend_run_job and the Python runner make the same library calls:
    the same headers and values (1e-12) in every result file."""
    import subprocess

    from asend3d_gb300 import build
    build.build()
    build.build_cli()
    d1, d2 = tmp_path / "py", tmp_path / "cli"
    d1.mkdir()
    d2.mkdir()
    write_cantilever_job(d1, etype="brick8", dvs=True)
    write_cantilever_job(d2, etype="brick8", dvs=True)
    J.JobRunner(d1 / "job.yaml").run()
    out = subprocess.run([str(build.CLI), str(d2 / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    def numbers(lines):
        return np.array([float(v) for ln in lines for v in ln.split(",")[1:] if v[:1].isdigit() or v[:1] in "-."])

    for name in ("nodes.csv", "obj.csv", "obj_grad.csv", "modal.csv", "modal_mode0.csv"):
        a, b = (d1 / name).read_text().splitlines(), (d2 / name).read_text().splitlines()
        assert a[0] == b[0] and len(a) == len(b), name
        assert [ln.split(",")[0] for ln in a] == [ln.split(",")[0] for ln in b], name
        fa, fb = numbers(a[1:]), numbers(b[1:])
        assert fa.shape == fb.shape, name
        # summation order differs (numpy vs the C++ loop) in reactions and sums
        assert np.allclose(fa, fb, rtol=1e-12, atol=1e-12 * np.abs(fa).max()), name


def write_dynamic_job(d):
    """The cantilever with an orthotropic, materially damped material and a
    lumped-mass Newmark run under the constant tip load."""
    m, xmin, xmax = write_cantilever_job(d, etype="brick8", modal=False)
    model = (d / "model.yaml").read_text()
    iso = "      E: [1000000.0]\n      nu: 0.0\n      G: 500000.0"
    assert iso in model
    model = model.replace(iso, "      E: [1000000.0, 500000.0, 400000.0]\n      nu: [0.2, 0.25, 0.3]\n"
                               "      G: [300000.0, 250000.0, 200000.0]\n    damping:\n    - [1, 1, 40.0]\n"
                               "    - [2, 2, 40.0]\n    - [3, 3, 40.0]\n    - [1, 2, 10.0]\n    - [4, 4, 20.0]")
    (d / "model.yaml").write_text(model)
    job = ["jobCommands:",
           "- command: readModelInput", "  fileName: model.yaml",
           "- command: readConstraints", "  fileName: constraints.yaml",
           "- command: readLoads", "  fileName: loads.yaml",
           "- command: solve", "  elastic: yes", "  dynamic: yes", "  timeStep: 0.002", "  simPeriod: 0.08",
           "  newmarkBeta: 0.25", "  newmarkGamma: 0.5", "  lumpMass: yes", "  solverMethod: iterative",
           "  convergenceTol: 1.0e-12",
           "- command: writeNodeResults", f"  fileName: {d / 'nodes.csv'}", "  nodeSet: xMax",
           "  fields:", "  - displacement"]
    (d / "job.yaml").write_text("\n".join(job) + "\n")
    return m, xmin, xmax


def test_job_lumped_mass_orthotropic_damped_dynamics(gpu_lib, oracle_lib, tmp_path):
    """lumpMass, orthotropic constants and material damping from job files:
    the Python runner against the oracle's Newmark run (1e-8 of the largest
    displacement), and the C++ runner against the Python runner (1e-12)."""
    import subprocess

    from asend3d_gb300 import build

    d1, d2 = tmp_path / "py", tmp_path / "cli"
    d1.mkdir()
    d2.mkdir()
    m, xmin, xmax = write_dynamic_job(d1)
    write_dynamic_job(d2)
    J.JobRunner(d1 / "job.yaml").run()
    head, rows = read_csv(d1 / "nodes.csv")
    props = np.tile([1e6, 5e5, 4e5, 0.2, 0.25, 0.3, 3e5, 2.5e5, 2e5], (m.n_elems, 1))
    D = np.zeros(36)
    for i, j, v in ((0, 0, 40.0), (1, 1, 40.0), (2, 2, 40.0), (0, 1, 10.0), (3, 3, 20.0)):
        D[6 * i + j] = D[6 * j + i] = v
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.2), np.full(m.n_elems, 1.0),
                ortho=props, damping=(0.0, 0.0, np.tile(D, (m.n_elems, 1))), lump_mass=True)
    p.add_node_set("xMin", xmin)
    p.add_node_set("xMax", xmax)
    p.fix_displacement("xMin")
    p.add_nodal_force("xMax", [0.0, 0.0, -2.0 / len(xmax)])
    n_steps = 40
    o = oracle_lib.Oracle(p, dynamic=True, dt=0.002, beta=0.25, gamma=0.5)
    _, uo, rc, _ = o.newmark(n_steps, 0.002, 0.25, 0.5, o.loads()[0], np.ones(n_steps), -1,
                             precond=oracle_lib.PC_DIRECT)
    assert rc == 0
    uo = uo.reshape(-1, 3)
    assert np.abs(rows[:, 1:4] - uo[xmax]).max() <= 1e-8 * np.abs(uo).max()
    build.build()
    build.build_cli()
    out = subprocess.run([str(build.CLI), str(d2 / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    _, rows2 = read_csv(d2 / "nodes.csv")
    assert np.allclose(rows2, rows, rtol=1e-12, atol=1e-12 * np.abs(rows).max())


def compliance_dC(E, nu, G, category, comp):
    """dC/dD of the reference's compliance form (element_properties.rs:648-764)
    for an isotropic element: 'modulus' k adds to E_k, 'shearModulus' k to
    G_k, 'poissonRatio' k to nu_k (nu12, nu13, nu23); dC = -C dS C."""
    S = np.zeros((6, 6))
    S[[0, 1, 2], [0, 1, 2]] = 1 / E
    S[0, 1] = S[1, 0] = S[0, 2] = S[2, 0] = S[1, 2] = S[2, 1] = -nu / E
    S[[3, 4, 5], [3, 4, 5]] = 1 / G
    C = np.linalg.inv(S)
    dS = np.zeros((6, 6))
    k = comp - 1
    if category == "modulus":
        dS[k, k] = -1 / E ** 2
        # S[0,1], S[0,2] carry 1/E1 and S[1,2] 1/E2
        for (a, b), ek in (((0, 1), 0), ((0, 2), 0), ((1, 2), 1)):
            if ek == k:
                dS[a, b] = dS[b, a] = nu / E ** 2
    elif category == "shearModulus":
        dS[3 + k, 3 + k] = -1 / G ** 2
    else:
        a, b, ek = ((0, 1, 0), (0, 2, 0), (1, 2, 1))[k]
        dS[a, b] = dS[b, a] = -1 / E
    return -C @ dS @ C


def test_job_element_objective_gradient(gpu_lib, oracle_lib, tmp_path):
    """A strainEnergy volumeIntegral term and a stress powerNorm term through
    calcObjective / calcObjGradient: values and the three material DV
    gradients against the oracle (values 1e-9, gradients 1e-7 relative)."""
    m, xmin, xmax = write_cantilever_job(tmp_path, nx=6, ny=2, nz=2, etype="brick8", modal=False, dvs=True)
    (tmp_path / "objective.yaml").write_text(
        "objectiveTerms:\n- category: strainEnergy\n  operator: volumeIntegral\n  elementSet: all\n"
        "  coefficient: 2.0\n  exponent: 1.0\n"
        "- category: stress\n  operator: powerNorm\n  elementSet: all\n  component: 1\n"
        "  coefficient: 1.0\n  exponent: 2.0\n")
    (tmp_path / "dvars.yaml").write_text(
        "designVariables:\n- category: modulus\n  component: 1\n  elementSet: all\n  coefficients: 1.0\n"
        "- category: shearModulus\n  component: 2\n  elementSet: all\n"
        "- category: poissonRatio\n  component: 3\n  elementSet: all\n  coefficients: 2.0\n")
    r = J.JobRunner(tmp_path / "job.yaml").run()
    assert r.log[-1] == "writeObjective"
    p = Problem(m, np.full(m.n_elems, 1e6), np.full(m.n_elems, 0.0), np.full(m.n_elems, 1.0))
    p.add_node_set("xMin", xmin)
    p.fix_displacement("xMin")
    p.add_node_set("xMax", xmax)
    p.add_nodal_force("xMax", [0.0, 0.0, -2.0 / len(xmax)])
    o = oracle_lib.Oracle(p)
    uo, _, _ = o.solve(o.loads()[0] + o.penalty_rhs(), precond=oracle_lib.PC_DIRECT)
    els = np.arange(m.n_elems)
    terms = [("strainEnergy", 0, "volumeIntegral", 2.0, 1.0), ("stress", 1, "powerNorm", 1.0, 2.0)]
    vals, grads = [], np.zeros(3)
    dvs = [("modulus", 1, np.ones(m.n_elems)), ("shearModulus", 2, np.ones(m.n_elems)),
           ("poissonRatio", 3, np.full(m.n_elems, 2.0))]
    for cat, comp, op, coef, ex in terms:
        L, dLdu, Q, _ = o.element_objective(uo, els, cat, comp, op, coef, ex)
        vals.append(L)
        _, lam, _, _ = o.adjoint(uo, dLdu=dLdu, precond=oracle_lib.PC_DIRECT)
        P = o.strain_pairs(uo, lam) - Q
        for i, (dcat, dcomp, cf) in enumerate(dvs):
            dC = compliance_dC(1e6, 0.0, 5e5, dcat, dcomp)
            grads[i] -= np.sum(cf[:, None, None] * dC[None] * P)
    lines = (tmp_path / "obj.csv").read_text().splitlines()
    got = [float(ln.split(",")[1]) for ln in lines[1:]]
    np.testing.assert_allclose(got, vals, rtol=1e-9)
    g = np.array([float(ln.split(",")[1]) for ln in (tmp_path / "obj_grad.csv").read_text().splitlines()[1:]])
    assert np.linalg.norm(g - grads) <= 1e-7 * np.linalg.norm(grads)


def write_twoply_job(d):
    """The reference's compositePlate [+45 / -45] case as job files: one
    2 x 2 shell4 element, xyMin fully fixed, xMinyMax fixed in x, F = 1 in x
    on each xMax node."""
    coords = [(-1.0, -1.0, 0.0), (1.0, -1.0, 0.0), (1.0, 1.0, 0.0), (-1.0, 1.0, 0.0)]
    lines = ["nodes:"] + [f"- [{i + 1}, {x!r}, {y!r}, {z!r}]" for i, (x, y, z) in enumerate(coords)]
    lines += ["elements:", "- type: shell4", "  connectivity:", "  - [1, 1, 2, 3, 4]"]
    lines += ["sets:", "  node:", "    xyMin:", "    - 1", "    xMinyMax:", "    - 4", "    xMax:", "    - 2", "    - 3",
              "  element:", "    all:", "    - 1"]
    lines += ["sections:", "- type: shell", "  orientation: [1.0, 0.0, 0.0, 0.0, 1.0, 0.0]", "  layup:",
              "    zOffset: 0.0", "    layers:",
              "    - material: cf", "      thickness: 0.05", "      angle: 45.0",
              "    - material: cf", "      thickness: 0.05", "      angle: -45.0",
              "  elementSet: all", "materials:", "  cf:", "    density: 1000.0", "    elastic:",
              "      E: [10000000.0, 1000000.0, 1000000.0]", "      nu: [0.0, 0.0, 0.0]",
              "      G: [5000000.0, 5000000.0, 5000000.0]"]
    (d / "model.yaml").write_text("\n".join(lines) + "\n")
    cons = ["constraints:"]
    for dof in range(1, 7):
        cons += ["- type: displacement", "  terms:", "  - nodeSet: xyMin", f"    dof: {dof}", "    coef: 1.0",
                 "  rhs: 0.0"]
    cons += ["- type: displacement", "  terms:", "  - nodeSet: xMinyMax", "    dof: 1", "    coef: 1.0", "  rhs: 0.0"]
    (d / "constraints.yaml").write_text("\n".join(cons) + "\n")
    (d / "loads.yaml").write_text("loads:\n- type: nodalForce\n  nodeSet: xMax\n  load: [1.0, 0.0, 0.0, 0.0, 0.0, 0.0]\n")
    job = ["jobCommands:", "- command: readModelInput", "  fileName: model.yaml",
           "- command: readConstraints", "  fileName: constraints.yaml",
           "- command: readLoads", "  fileName: loads.yaml",
           "- command: solve", "  elastic: yes", "  dynamic: no", "  solverMethod: iterative",
           "  convergenceTol: 1.0e-14", "  maxIterations: 20000",
           "- command: writeNodeResults", f"  fileName: {d / 'nodes.csv'}", "  nodeSet: xMax",
           "  fields:", "  - displacement"]
    (d / "job.yaml").write_text("\n".join(job) + "\n")


def test_job_layered_shell_known_answers(gpu_lib, tmp_path):
    """A layered shell section through the Python runner and the C++ CLI:
    the compositePlate [+45 / -45] known answers at the (1, 1) corner
    (examples/testCases/compositePlate/notes.txt; 1e-8, ux 1e-5)."""
    import subprocess

    from asend3d_gb300 import build
    build.build_cli()
    for runner in ("python", "cli"):
        d = tmp_path / runner
        d.mkdir()
        write_twoply_job(d)
        if runner == "python":
            J.JobRunner(d / "job.yaml").run()
        else:
            out = subprocess.run([str(build.CLI), str(d / "job.yaml")], capture_output=True, text=True)
            assert out.returncode == 0, out.stderr
        head, rows = read_csv(d / "nodes.csv")
        corner = rows[rows[:, 0] == 3][0]
        assert corner[1] == pytest.approx(4.651452282161358e-06, rel=1e-5), runner
        assert corner[2] == pytest.approx(2.6514522821613584e-06, rel=1e-8), runner
        assert corner[3] == pytest.approx(-1.79253112033e-04, rel=1e-8), runner
        assert corner[4] == pytest.approx(-8.96265560167775e-05, rel=1e-8), runner


def test_beam_job_runners(gpu_lib, tmp_path):
    """The beam2 cantilever job (hexBeam / shellBeam known answer, tip w = 8 at
    the pin's 1e-3) through the Python runner and the C++ CLI (same values to
    1e-12), and with every element numbered against the section's x direction
    (same tip to 1e-8)."""
    import subprocess

    from asend3d_gb300 import build
    build.build()
    build.build_cli()
    d1, d2, d3 = tmp_path / "py", tmp_path / "cli", tmp_path / "rev"
    for d in (d1, d2, d3):
        d.mkdir()
    write_beam_job(d1)
    write_beam_job(d2)
    write_beam_job(d3, reverse=True)
    J.JobRunner(d1 / "job.yaml").run()
    J.JobRunner(d3 / "job.yaml").run()
    out = subprocess.run([str(build.CLI), str(d2 / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    _, r1 = read_csv(d1 / "nodes.csv")
    _, r2 = read_csv(d2 / "nodes.csv")
    _, r3 = read_csv(d3 / "nodes.csv")
    np.testing.assert_allclose(r1, r2, rtol=1e-12, atol=1e-12 * np.abs(r1).max())
    np.testing.assert_allclose(r3[:, 1:4], r1[:, 1:4], rtol=1e-8, atol=1e-8 * np.abs(r1).max())
    assert r1[0, 3] == pytest.approx(8.0, rel=1e-3)
    w = float((d1 / "obj.csv").read_text().splitlines()[1].split(",")[1])
    assert w == pytest.approx(r1[0, 3], rel=1e-12)


def test_beam_job_given_matrices(gpu_lib, tmp_path):
    """A beam job whose section stiffness is given as beamProps entries (with
    an axial-bending coupling): the Python runner and the CLI agree (1e-12),
    and the same job with every element numbered against the orientation's x
    direction (the given matrix turned into its frame) gives the same tip
    (1e-8); with the given diagonal equal to the computed one the tip is the
    pin's 8 (1e-3)."""
    import subprocess

    from asend3d_gb300 import build
    build.build()
    build.build_cli()
    given = [("stiffness", 1, 1, 1e5), ("stiffness", 2, 2, 5e4), ("stiffness", 3, 3, 5e4),
             ("stiffness", 4, 4, 140.0), ("stiffness", 5, 5, 1e6 * 0.1**3 / 12), ("stiffness", 6, 6, 1e6 * 0.1 / 12)]
    coupled = given + [("stiffness", 1, 5, 3.0)]
    dirs = {k: tmp_path / k for k in ("plain", "py", "cli", "rev")}
    for d in dirs.values():
        d.mkdir()
    write_beam_job(dirs["plain"], given=given)
    write_beam_job(dirs["py"], given=coupled)
    write_beam_job(dirs["cli"], given=coupled)
    write_beam_job(dirs["rev"], reverse=True, given=coupled)
    for k in ("plain", "py", "rev"):
        J.JobRunner(dirs[k] / "job.yaml").run()
    out = subprocess.run([str(build.CLI), str(dirs["cli"] / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    rows = {k: read_csv(dirs[k] / "nodes.csv")[1] for k in dirs}
    assert rows["plain"][0, 3] == pytest.approx(8.0, rel=1e-3)
    np.testing.assert_allclose(rows["py"], rows["cli"], rtol=1e-12, atol=1e-12 * np.abs(rows["py"]).max())
    np.testing.assert_allclose(rows["rev"][:, 1:4], rows["py"][:, 1:4], rtol=1e-8,
                               atol=1e-8 * np.abs(rows["py"]).max())
    assert abs(rows["py"][0, 1]) > 1e-9  # the coupling moves the tip axially
