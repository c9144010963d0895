"""The C++ job CLI (asend_run_job) on the CPU: its --parse mode reads the
same job, model, constraint, load, objective and design-variable files as
the Python readers (job.py) to the same values, prints Rust "{:.12e}"
numbers, and stops with an error naming anything outside the path.  The
GPU run of a whole job is in test_gpu_job.py."""
import json
import subprocess

import numpy as np
import pytest

from asend3d_gb300 import build
from asend3d_gb300 import job as J

from test_job import write_cantilever_job


@pytest.fixture(scope="module")
def cli():
    build.build()
    return str(build.build_cli())  # raises with the compiler's message if the CLI does not build


def test_parse_matches_python_readers(cli, tmp_path):
    m, xmin, xmax = write_cantilever_job(tmp_path, dvs=True)
    out = subprocess.run([cli, "--parse", str(tmp_path / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    j = json.loads(out.stdout)
    assert j["commands"] == [c["command"] for c in J.read_job(tmp_path / "job.yaml")]
    mi = J.read_model(tmp_path / "model.yaml")
    assert j["elem_type"] == mi.elem_type and j["node_labels"] == mi.node_labels
    np.testing.assert_array_equal(np.array(j["coords"]).reshape(-1, 3), np.array(mi.coords))
    assert j["conn"] == mi.conn and j["node_sets"] == mi.node_sets and j["elem_sets"] == mi.elem_sets
    cons = J.read_constraints(tmp_path / "constraints.yaml")
    assert [c["terms"] for c in j["constraints"]] == [c["terms"] for c in cons]
    loads = J.read_loads(tmp_path / "loads.yaml")
    assert [l["load"] for l in j["loads"]] == [l["load"] for l in loads]
    obj = J.read_objective(tmp_path / "objective.yaml")
    assert [(o["component"], o["coefficient"], o["exponent"]) for o in j["objective"]] == \
        [(o["component"], o["coefficient"], o["exponent"]) for o in obj]
    dvs = J.read_design_vars(tmp_path / "dvars.yaml")
    assert [(d["category"], d["component"], d["elementSet"], d["coefficients"]) for d in j["design_vars"]] == \
        [(d["category"], d["component"], d["elementSet"], d["coefficients"]) for d in dvs]
    assert j["rust_exp_samples"] == ["1.500000000000e0", "-2.500000000000e-7", "0.000000000000e0"]


def test_cli_errors(cli, tmp_path):
    (tmp_path / "m.yaml").write_text("elements:\n- type: shell3\n")
    (tmp_path / "job.yaml").write_text("jobCommands:\n- command: readModelInput\n  fileName: m.yaml\n")
    out = subprocess.run([cli, "--parse", str(tmp_path / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 1 and "shell3 is not on the GPU path" in out.stderr
    (tmp_path / "m.yaml").write_text("nodes:\n- [0, 0.0, 0.0, 0.0]\n")
    (tmp_path / "job.yaml").write_text("jobCommands:\n- command: readModelInput\n  fileName: m.yaml\n"
                                       "- command: buildMesh\n")
    out = subprocess.run([cli, str(tmp_path / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 1 and "job command buildMesh is not on the GPU path" in out.stderr
    out = subprocess.run([cli], capture_output=True, text=True)
    assert out.returncode == 2 and "usage" in out.stderr


def test_parse_shell_model(cli, tmp_path):
    from test_job import write_shell_job
    m = write_shell_job(tmp_path)
    out = subprocess.run([cli, "--parse", str(tmp_path / "job.yaml")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    j = json.loads(out.stdout)
    assert j["elem_type"] == 41 and len(j["conn"]) == m.n_elems and all(len(r) == 4 for r in j["conn"])
    assert j["elem_sets"]["all"] == list(range(m.n_elems))
