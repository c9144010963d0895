"""Result files in the reference's formats, so that the reference's
post-processing scripts read this library's results unchanged.

Formats (solverSrc/asend_run_job/src/):
  * solnTStep<N>.out (model_output.rs:14-82 writer, model_input.rs:1468+
    reader): per node in model order, displacement, velocity and acceleration
    (dof-per-node values each) as big-endian f64; then, per element with
    internal DOF, their displacements.  Only the elastic, non-fluid fields are
    written (the path's physics).
  * node results CSV (model_output.rs:84-262): header "node," + six columns
    per field + "time", one row per node of the set, values in Rust's
    "{:.12e}" notation, time -1 for the current state.
  * objective CSV (model_output.rs:556-619): "objectiveTerm,value[,fields]"
    and, with the gradient, <root>_grad<ext> with "designVariable,objGrad".
  * modal results CSV (model_output.rs:495-555): "mode,eigenvalue,frequency"
    (or load_factor for buckling), with <root>_mode<k><ext> per mode when mode
    shapes are asked for.

Rust's LowerExp formatting ("1.500000000000e0", "-2.5e-7" style exponents:
no '+', no zero padding) is reproduced by ``rust_exp``.
"""
from __future__ import annotations

import math
import os
from pathlib import Path

import numpy as np

NODE_FIELD_COLUMNS = {
    "displacement": "U1,U2,U3,R1,R2,R3,",
    "velocity": "V1,V2,V3,RV1,RV2,RV3,",
    "acceleration": "A1,A2,A3,RA1,RA2,RA3,",
    "reactionForce": "RF1,RF2,RF3,RM1,RM2,RM3,",
}


def rust_exp(x: float, prec: int = 12) -> str:
    """Rust's format!("{:.prec$e}", x) for an f64."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    s = f"{x:.{prec}e}"             # C notation: mantissa e[+-]dd
    mant, exp = s.split("e")
    return f"{mant}e{int(exp)}"


def _split_root(file_name: str) -> tuple[str, str]:
    """The reference splits at the FIRST '.' of the whole path (CppStr::find)."""
    i = file_name.find(".")
    return (file_name, "") if i < 0 else (file_name[:i], file_name[i:])


def six(values: np.ndarray) -> np.ndarray:
    """Per-node values widened to the reference's six components (solid nodes
    carry zeros for the rotations, as the node arrays are zero-initialised)."""
    v = np.asarray(values, dtype=np.float64)
    if v.ndim == 1:
        v = v.reshape(-1, 3 if v.size % 6 else 6)
    out = np.zeros((v.shape[0], 6))
    out[:, :v.shape[1]] = v
    return out


def write_node_results(file_name, labels, fields: dict, time: float = -1.0, rows=None):
    """fields: ordered {name: per-node values [n_nodes, 3 or 6]} for names in
    NODE_FIELD_COLUMNS; labels: node labels of the set, in set order; rows:
    the matching positions in the per-node arrays (default: the labels)."""
    for name in fields:
        if name not in NODE_FIELD_COLUMNS:
            raise ValueError(f"unrecognized output field '{name}' for write_node_results")
    data = {k: six(v) for k, v in fields.items()}
    rows = labels if rows is None else rows
    lines = ["node," + "".join(NODE_FIELD_COLUMNS[k] for k in fields) + "time\n"]
    t = rust_exp(time)
    for lab, r in zip(labels, rows):
        row = [f"{int(lab)},"]
        for k in fields:
            row.extend(rust_exp(v) + "," for v in data[k][int(r)])
        row.append(t + "\n")
        lines.append("".join(row))
    Path(file_name).write_text("".join(lines))


def write_objective(file_name, values, terms=None, include=(), gradient=None):
    """values: per objective term; terms: per-term dicts for the include
    fields (category, operator, component, layer, coefficient, exponent,
    elementSet, nodeSet, activeTime); gradient: dL/dD per design variable."""
    lines = ["objectiveTerm,value" + "".join(f",{f}" for f in include) + "\n"]
    num = {"coefficient", "exponent", "activeTime"}
    for i, v in enumerate(values):
        row = f"{i},{rust_exp(v)}"
        for f in include:
            val = (terms[i] if terms else {}).get(f, "")
            row += "," + (rust_exp(val) if f in num else str(val))
        lines.append(row + "\n")
    Path(file_name).write_text("".join(lines))
    if gradient is not None:
        root, ext = _split_root(str(file_name))
        g = ["designVariable,objGrad\n"] + [f"{i},{rust_exp(v)}\n" for i, v in enumerate(gradient)]
        Path(f"{root}_grad{ext}").write_text("".join(g))


def write_modal_results(file_name, eigenvalues, load_factors, kind="frequency", modes=None, labels=None):
    """load_factors: frequencies [Hz] for a frequency job (sqrt(lambda)/(2 pi),
    -1 for lambda < 0); modes: [n_modes, n_nodes, 3 or 6] mode shapes to write
    as <root>_mode<k><ext> (rotations of solid nodes as zeros)."""
    head = "mode,eigenvalue," + ("load_factor\n" if kind == "buckling" else "frequency\n")
    lines = [head] + [f"{i},{rust_exp(e)},{rust_exp(f)}\n"
                      for i, (e, f) in enumerate(zip(eigenvalues, load_factors))]
    Path(file_name).write_text("".join(lines))
    if modes is not None:
        root, ext = _split_root(str(file_name))
        for k, m in enumerate(modes):
            v = six(m)
            labs = range(v.shape[0]) if labels is None else labels
            rows = ["Node,U1,U2,U3,R1,R2,R3\n"]
            rows += [f"{int(lab)}" + "".join("," + rust_exp(x) for x in v[i]) + "\n" for i, lab in enumerate(labs)]
            Path(f"{root}_mode{k}{ext}").write_text("".join(rows))


def write_time_step_soln(directory, step: int, disp, vel, acc, internal=None):
    """disp, vel, acc: [n_nodes, dof per node]; internal: per element with
    internal DOF, its internal displacements (concatenated in element order)."""
    d, v, a = (np.asarray(x, np.float64) for x in (disp, vel, acc))
    per_node = np.concatenate([d, v, a], axis=1)     # node-major: disp, vel, acc
    buf = per_node.astype(">f8").tobytes()
    if internal is not None and len(internal):
        buf += np.asarray(internal, np.float64).astype(">f8").tobytes()
    os.makedirs(directory, exist_ok=True)
    Path(directory, f"solnTStep{step}.out").write_bytes(buf)


def read_time_step_soln(directory, step: int, n_nodes: int, dpn: int, n_internal: int = 0):
    raw = np.frombuffer(Path(directory, f"solnTStep{step}.out").read_bytes(), dtype=">f8").astype(np.float64)
    need = n_nodes * 3 * dpn + n_internal
    if raw.size != need:
        raise ValueError(f"solnTStep{step}.out holds {raw.size} values, expected {need}")
    per_node = raw[:n_nodes * 3 * dpn].reshape(n_nodes, 3, dpn)
    return per_node[:, 0], per_node[:, 1], per_node[:, 2], raw[n_nodes * 3 * dpn:]
