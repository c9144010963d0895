"""Result files in the reference's formats (model_output.rs): exact text of
the node-results, objective (+ _grad) and modal CSVs, Rust "{:.12e}" number
notation, and the big-endian solnTStep<N>.out round trip."""
import struct

import numpy as np
import pytest

from asend3d_gb300 import results_io as rio


@pytest.mark.parametrize("x,s", [(1.5, "1.500000000000e0"), (-2.5e-7, "-2.500000000000e-7"),
                                 (0.0, "0.000000000000e0"), (1e100, "1.000000000000e100"),
                                 (123456.789, "1.234567890000e5"), (-0.0, "-0.000000000000e0"),
                                 (8.0002, "8.000200000000e0"), (float("nan"), "NaN"),
                                 (float("inf"), "inf")])
def test_rust_exp(x, s):
    assert rio.rust_exp(x) == s


def test_node_results_text(tmp_path):
    disp = np.array([[0.0, 0.0, 0.0], [1e-3, -2.5e-7, 8.0]])
    f = tmp_path / "nodes.csv"
    rio.write_node_results(f, [1, 0], {"displacement": disp})
    z = "0.000000000000e0"
    assert f.read_text() == (
        "node,U1,U2,U3,R1,R2,R3,time\n"
        f"1,1.000000000000e-3,-2.500000000000e-7,8.000000000000e0,{z},{z},{z},-1.000000000000e0\n"
        f"0,{z},{z},{z},{z},{z},{z},-1.000000000000e0\n")
    with pytest.raises(ValueError):
        rio.write_node_results(f, [0], {"stress": disp})


def test_node_results_two_fields_shell(tmp_path):
    u = np.arange(12, dtype=float).reshape(2, 6)
    f = tmp_path / "n.csv"
    rio.write_node_results(f, [0], {"displacement": u, "reactionForce": -u}, time=0.5)
    lines = f.read_text().splitlines()
    assert lines[0] == "node,U1,U2,U3,R1,R2,R3,RF1,RF2,RF3,RM1,RM2,RM3,time"
    vals = lines[1].split(",")
    assert vals[0] == "0" and len(vals) == 14 and vals[-1] == "5.000000000000e-1"
    assert [float(v) for v in vals[1:13]] == list(u[0]) + list(-u[0])


def test_objective_and_gradient(tmp_path):
    f = tmp_path / "obj.csv"
    rio.write_objective(str(f), [8.0002], terms=[{"category": "displacement", "coefficient": 1.0}],
                        include=("category", "coefficient"), gradient=[-8e-6, 1.25])
    assert f.read_text() == "objectiveTerm,value,category,coefficient\n0,8.000200000000e0,displacement,1.000000000000e0\n"
    assert (tmp_path / "obj_grad.csv").read_text() == (
        "designVariable,objGrad\n0,-8.000000000000e-6\n1,1.250000000000e0\n")


def test_modal_results_and_modes(tmp_path):
    f = tmp_path / "modal.csv"
    ev = np.array([1.0, 4.0])
    fr = np.sqrt(ev) / (2 * np.pi)
    modes = np.arange(12, dtype=float).reshape(2, 2, 3)
    rio.write_modal_results(str(f), ev, fr, modes=modes)
    lines = f.read_text().splitlines()
    assert lines[0] == "mode,eigenvalue,frequency"
    assert lines[1] == f"0,1.000000000000e0,{rio.rust_exp(fr[0])}"
    m1 = (tmp_path / "modal_mode1.csv").read_text().splitlines()
    assert m1[0] == "Node,U1,U2,U3,R1,R2,R3"
    assert m1[2].split(",")[:4] == ["1", "9.000000000000e0", "1.000000000000e1", "1.100000000000e1"]
    assert m1[2].split(",")[4:] == ["0.000000000000e0"] * 3
    rio.write_modal_results(str(f), ev, [0.5, 0.25], kind="buckling")
    assert f.read_text().splitlines()[0] == "mode,eigenvalue,load_factor"


def test_time_step_soln_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    n, dpn = 5, 6
    d, v, a = (rng.standard_normal((n, dpn)) for _ in range(3))
    internal = rng.standard_normal(16)
    rio.write_time_step_soln(tmp_path, 3, d, v, a, internal)
    raw = (tmp_path / "solnTStep3.out").read_bytes()
    assert len(raw) == 8 * (3 * n * dpn + 16)
    # node 0: its displacement, velocity, acceleration, big-endian
    assert raw[:8] == struct.pack(">d", d[0, 0])
    assert raw[8 * dpn:8 * dpn + 8] == struct.pack(">d", v[0, 0])
    assert raw[8 * 3 * dpn:8 * 3 * dpn + 8] == struct.pack(">d", d[1, 0])
    d2, v2, a2, i2 = rio.read_time_step_soln(tmp_path, 3, n, dpn, 16)
    for x, y in ((d, d2), (v, v2), (a, a2), (internal, i2)):
        np.testing.assert_array_equal(x, y)
    with pytest.raises(ValueError):
        rio.read_time_step_soln(tmp_path, 3, n, 3)
