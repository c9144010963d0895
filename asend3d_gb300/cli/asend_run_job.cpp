// asend_run_job -- drop-in for the reference's `asend_run_job <job.yaml>` on
// the linear-elastic static, Newmark and modal path, driving libasend_gpu.so
// through its C ABI (include/asend_gpu.h).
//
// Reference (solverSrc/asend_run_job/src/): main.rs:55-70 (argv), job loop
// model_meth.rs:20-140, input readers model_input.rs (line grammar :34-119,
// job :121-310, model :312-860, constraints :872-970, loads :981-1124,
// design variables :1218-1296, objective :1298-1375), writers
// model_output.rs (node results :84-262, modal :495-555, objective
// :556-619).  The commands, file formats and the subset accepted are those of
// the Python mirror asend3d_gb300/job.py; anything outside the subset stops
// with an error naming it.
//
//   asend_run_job job.yaml            run the job
//   asend_run_job --parse job.yaml    read every input file the job names and
//                                     print a JSON summary (no device use)
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "asend_gpu.h"

namespace {

using Strs = std::vector<std::string>;

struct Fail : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------------------
// the reference's line grammar (model_input.rs:34-119)
// ---------------------------------------------------------------------------
struct Record {
    std::string h[4];
    Strs data;
    bool key = false;
};

Strs tokens(const std::string& s) {
    Strs out;
    std::string cur;
    for (char ch : s) {
        if (ch == ' ' || ch == ',' || ch == '[' || ch == ']' || ch == '\t' || ch == '\n' || ch == '\r') {
            if (!cur.empty()) out.push_back(cur);
            cur.clear();
        } else {
            cur += ch;
        }
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

std::vector<Record> read_records(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw Fail("could not open " + path);
    std::vector<Record> out;
    std::string h[4];
    size_t sp[4] = {0, 0, 0, 0};
    std::string line;
    while (std::getline(f, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        line += " ";
        Record r;
        const size_t colon = line.find(':');
        if (colon != std::string::npos) {
            size_t lead = line.find_first_not_of(" -\n\t");
            if (lead == std::string::npos || lead > colon) lead = colon;
            const std::string word = line.substr(lead, colon - lead);
            if (h[0].empty() || sp[0] == lead) {
                h[0] = word; sp[0] = lead;
                h[1] = h[2] = h[3] = ""; sp[1] = sp[2] = sp[3] = 0;
            } else if (h[1].empty() || sp[1] == lead) {
                h[1] = word; sp[1] = lead;
                h[2] = h[3] = ""; sp[2] = sp[3] = 0;
            } else if (h[2].empty() || sp[2] == lead) {
                h[2] = word; sp[2] = lead;
                h[3] = ""; sp[3] = 0;
            } else {
                h[3] = word; sp[3] = lead;
            }
            r.data = tokens(line.substr(colon + 1));
            r.key = true;
        } else {
            const size_t dash = line.find("- ");
            if (dash != std::string::npos) r.data = tokens(line.substr(dash + 1));
        }
        for (int i = 0; i < 4; ++i) r.h[i] = h[i];
        out.push_back(r);
    }
    return out;
}

double num(const std::string& s) {
    char* end = nullptr;
    const double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str()) throw Fail("not a number: " + s);
    return v;
}
int inum(const std::string& s) { return (int)std::lround(num(s)); }

std::vector<int> label_range(const Strs& d) {  // one label, or [a, b(, step)) with b excluded
    if (d.size() == 1) return {inum(d[0])};
    const int a = inum(d[0]), b = inum(d[1]), st = d.size() == 3 ? inum(d[2]) : 1;
    std::vector<int> out;
    for (int i = a; i < b; i += st) out.push_back(i);
    return out;
}

// ---------------------------------------------------------------------------
// input files
// ---------------------------------------------------------------------------
struct Command {
    std::string name;
    std::map<std::string, std::string> kv;
    std::map<std::string, Strs> lists;
    std::string get(const std::string& k, const std::string& def = "") const {
        auto it = kv.find(k);
        return it == kv.end() ? def : it->second;
    }
    bool yes(const std::string& k) const { return get(k).find("yes") != std::string::npos; }
};

std::vector<Command> read_job(const std::string& path) {
    std::vector<Command> cmds;
    for (const Record& r : read_records(path)) {
        const std::string& k = r.h[1];
        if (k == "command" && r.data.size() == 1) {
            cmds.push_back(Command{r.data[0], {}, {}});
            continue;
        }
        if (cmds.empty() || k.empty()) continue;
        if ((k == "fields" || k == "include" || k == "properties" || k == "staticLoadTime") && r.data.size() == 1)
            cmds.back().lists[k].push_back(r.data[0]);
        else if (k == "timeSteps" && !r.data.empty())
            for (const auto& d : r.data) cmds.back().lists[k].push_back(d);
        else if (r.data.size() == 1)
            cmds.back().kv[k] = r.data[0];
    }
    return cmds;
}

struct Layer {
    std::string material;
    double thickness = 0.0, angle = 0.0;
};
struct Section {
    std::string type, material, elset;
    std::vector<Layer> layers;
    double z_offset = 0.0;
    std::vector<double> orientation;  // xDir, xyVec
    // beamProps (model_input.rs:561-596): area, I[5], J, given stiffness / mass
    // matrices (symmetric, section_meth.rs:61-71; empty when not given)
    double area = 0.0, J = 0.0;
    std::vector<double> I, stiffness, mass;
};
struct Material {
    double density = 0.0;
    std::vector<double> E, nu, G;
    std::vector<double> damping;  // 6 x 6 symmetric, empty when none
};
struct Model {
    std::vector<int> node_labels, elem_labels;
    std::vector<double> coords;
    std::vector<std::vector<int>> conn;
    int elem_type = -1;
    std::map<std::string, std::vector<int>> node_sets, elem_sets;
    std::vector<std::string> node_set_order, elem_set_order;
    std::vector<Section> sections;
    std::map<std::string, Material> materials;
};

// Angle [deg] of a shell section's material x axis (orientation xDir,
// xyVec) from the global x axis, for flat shells in a plane z = const whose
// local z is +z (correct_orient, element_properties.rs:2052-2150).
double shell_frame_angle(const Section& s) {
    if (s.orientation.empty()) return 0.0;
    const double* x = s.orientation.data();
    const double* y = x + 3;
    const double z[3] = {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
    const double nx = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    const double nz = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
    if (std::fabs(x[2]) > 1e-12 * nx || z[2] <= 0.0 || std::hypot(z[0], z[1]) > 1e-12 * nz)
        throw Fail("shell orientations with the local z axis along +z only");
    return std::atan2(x[1], x[0]) * 180.0 / M_PI;
}

int element_type(const std::string& t) {
    if (t == "brick8") return 8;
    if (t == "brickIM") return 81;
    if (t == "tet4") return 4;
    if (t == "tet10") return 10;
    if (t == "shell4") return 41;
    if (t == "beam2") return 2;
    for (const char* o : {"wedge6", "shell3", "frcFld", "mass", "fl4", "fl6", "fl8", "fl10"})
        if (t == o) throw Fail("element type " + t + " is not on the GPU path");
    throw Fail("unrecognized element type: " + t);
}

Model read_model(const std::string& path) {
    Model m;
    std::vector<int>* cur = nullptr;
    for (const Record& r : read_records(path)) {
        const auto& h = r.h;
        const auto& d = r.data;
        if (h[0] == "nodes" && d.size() == 4) {
            m.node_labels.push_back(inum(d[0]));
            for (int j = 1; j < 4; ++j) m.coords.push_back(num(d[j]));
        } else if (h[0] == "elements") {
            if (h[1] == "type" && d.size() == 1) {
                const int t = element_type(d[0]);
                if (m.elem_type >= 0 && m.elem_type != t) throw Fail("one element type per model");
                m.elem_type = t;
            } else if (h[1] == "connectivity" && d.size() > 1) {
                m.elem_labels.push_back(inum(d[0]));
                std::vector<int> row;
                for (size_t i = 1; i < d.size(); ++i) row.push_back(inum(d[i]));
                m.conn.push_back(row);
            }
        } else if (h[0] == "sets" && (h[1] == "node" || h[1] == "element") && !h[2].empty()) {
            auto& sets = h[1] == "node" ? m.node_sets : m.elem_sets;
            auto& order = h[1] == "node" ? m.node_set_order : m.elem_set_order;
            if (r.key) {
                if (!sets.count(h[2])) order.push_back(h[2]);
                cur = &sets[h[2]];
            } else if (!d.empty() && cur) {
                for (int v : label_range(d)) cur->push_back(v);
            }
        } else if (h[0] == "sections") {
            if (h[1] == "type" && d.size() == 1) {
                m.sections.push_back(Section{d[0], "", "", {}, 0.0, {}, 0.0, 0.0, {}, {}, {}});
            } else if (m.sections.empty()) {
                continue;
            } else if (h[1] == "material" && d.size() == 1) {
                m.sections.back().material = d[0];
            } else if (h[1] == "elementSet" && d.size() == 1) {
                m.sections.back().elset = d[0];
            } else if (h[1] == "orientation" && d.size() == 6) {
                for (const auto& x : d) m.sections.back().orientation.push_back(num(x));
            } else if (h[1] == "layup") {
                auto& lay = m.sections.back().layers;
                if (h[2] == "zOffset" && d.size() == 1) m.sections.back().z_offset = num(d[0]);
                else if (h[2] == "layers" && h[3] == "material" && d.size() == 1)
                    lay.push_back(Layer{d[0], 0.0, 0.0});
                else if (h[2] == "layers" && h[3] == "thickness" && d.size() == 1 && !lay.empty())
                    lay.back().thickness = num(d[0]);
                else if (h[2] == "layers" && h[3] == "angle" && d.size() == 1 && !lay.empty())
                    lay.back().angle = num(d[0]);
            } else if (h[1] == "beamProps" && !d.empty()) {
                // J is read from its one value (the reference indexes data[1] there)
                Section& s = m.sections.back();
                if (h[2] == "area" && d.size() == 1) s.area = num(d[0]);
                else if (h[2] == "I" && d.size() == 5) {
                    s.I.clear();
                    for (const auto& x : d) s.I.push_back(num(x));
                } else if (h[2] == "J" && d.size() == 1) s.J = num(d[0]);
                else if ((h[2] == "stiffness" || h[2] == "mass") && d.size() == 3) {
                    std::vector<double>& mat = h[2] == "stiffness" ? s.stiffness : s.mass;
                    if (mat.empty()) mat.assign(36, 0.0);
                    const int r = (int)num(d[0]) - 1, c = (int)num(d[1]) - 1;
                    if (r < 0 || r > 5 || c < 0 || c > 5) throw Fail("beam section matrix index out of range");
                    mat[6 * r + c] = mat[6 * c + r] = num(d[2]);
                } else if (h[2] == "damping" || h[2] == "expLoadCoef")
                    throw Fail("beam section " + h[2] + " entries are not on the GPU path");
            } else if ((h[1] == "potField" || h[1] == "dampField" || h[1] == "thermField") && !d.empty()) {
                throw Fail("section " + h[1] + " is not on the GPU path");
            }
        } else if (h[0] == "materials" && !h[1].empty()) {
            Material& mat = m.materials[h[1]];
            if (h[2] == "density" && d.size() == 1) {
                mat.density = num(d[0]);
            } else if (h[2] == "elastic" && (h[3] == "E" || h[3] == "nu" || h[3] == "G") && !d.empty()) {
                std::vector<double> v;
                for (const auto& x : d) v.push_back(num(x));
                if (v.size() == 1) v.assign(3, v[0]);
                (h[3] == "E" ? mat.E : h[3] == "nu" ? mat.nu : mat.G) = v;
            } else if (h[2] == "elastic" && h[3] == "stiffness" && !d.empty()) {
                throw Fail("anisotropic stiffness matrices are not on the GPU path");
            } else if (h[2] == "damping" && d.size() == 3) {
                // (row, column, value), 1-based, symmetric (model_input.rs:719-723)
                if (mat.damping.empty()) mat.damping.assign(36, 0.0);
                const int i = (int)num(d[0]) - 1, j = (int)num(d[1]) - 1;
                if (i < 0 || i > 5 || j < 0 || j > 5) throw Fail("damping index out of range 1..6");
                mat.damping[6 * i + j] = mat.damping[6 * j + i] = num(d[2]);
            }
        }
    }
    return m;
}

struct Constraint {
    std::vector<std::string> sets;
    std::vector<int> dof;
    std::vector<double> coef;
    double rhs = 0.0;
};
std::vector<Constraint> read_constraints(const std::string& path) {
    std::vector<Constraint> out;
    for (const Record& r : read_records(path)) {
        if (r.h[0] != "constraints") continue;
        const auto& d = r.data;
        if (r.h[1] == "type" && d.size() == 1) {
            if (d[0] != "displacement") throw Fail(d[0] + " constraints are not on the GPU path");
            out.emplace_back();
        } else if (out.empty()) {
            continue;
        } else if (r.h[1] == "terms") {
            auto& c = out.back();
            if (r.h[2] == "nodeSet" && d.size() == 1) { c.sets.push_back(d[0]); c.dof.push_back(1); c.coef.push_back(1.0); }
            else if (r.h[2] == "dof" && d.size() == 1 && !c.dof.empty()) c.dof.back() = inum(d[0]);
            else if (r.h[2] == "coef" && d.size() == 1 && !c.coef.empty()) c.coef.back() = num(d[0]);
        } else if (r.h[1] == "rhs" && d.size() == 1) {
            out.back().rhs = num(d[0]);
        }
    }
    return out;
}

struct Load {
    std::string type, node_set, elem_set;
    double load[6] = {0, 0, 0, 0, 0, 0}, norm_dir[3] = {0, 0, 0}, norm_tol = 1.0;
    double t0 = 0.0, t1 = 1e100;
    double center[3] = {0, 0, 0}, axis[3] = {0, 0, 1}, omega = 0.0;  // centrifugal
};
std::vector<Load> read_loads(const std::string& path) {
    std::vector<Load> out;
    for (const Record& r : read_records(path)) {
        if (r.h[0] != "loads") continue;
        const auto& d = r.data;
        const std::string& k = r.h[1];
        if (k == "type" && d.size() == 1) {
            if (d[0] != "nodalForce" && d[0] != "surfaceTraction" && d[0] != "surfacePressure" && d[0] != "bodyForce" &&
                d[0] != "gravitational" && d[0] != "centrifugal")
                throw Fail(d[0] + " loads are not on the GPU path");
            out.emplace_back();
            out.back().type = d[0];
        } else if (out.empty()) {
            continue;
        } else if (k == "load" && !d.empty()) {
            for (size_t i = 0; i < d.size() && i < 6; ++i) out.back().load[i] = num(d[i]);
        } else if (k == "nodeSet" && d.size() == 1) {
            out.back().node_set = d[0];
        } else if (k == "elementSet" && d.size() == 1) {
            out.back().elem_set = d[0];
        } else if (k == "normDir" && d.size() == 3) {
            for (int i = 0; i < 3; ++i) out.back().norm_dir[i] = num(d[i]);
        } else if (k == "normTolerance" && d.size() == 1) {
            out.back().norm_tol = num(d[0]);
        } else if (k == "activeTime" && !d.empty()) {
            out.back().t0 = num(d[0]);
            out.back().t1 = d.size() > 1 ? num(d[1]) : 1e100;
        } else if ((k == "center" || k == "axis") && d.size() == 3) {  // model_input.rs:1103-1112
            for (int i = 0; i < 3; ++i) (k == "center" ? out.back().center : out.back().axis)[i] = num(d[i]);
        } else if (k == "angularVelocity" && !d.empty()) {
            out.back().omega = num(d[0]);
        }
    }
    return out;
}

struct ObjTerm {  // defaults of ObjectiveTerm::new (objective.rs:45-49)
    std::string category, optr, node_set, elem_set;
    int component = 0;
    double coef = 0.0, expnt = 0.0, t0 = 0.0, t1 = 1e100;
    std::vector<double> targets;
};
std::vector<ObjTerm> read_objective(const std::string& path) {
    std::vector<ObjTerm> out;
    for (const Record& r : read_records(path)) {
        if (r.h[0] != "objectiveTerms") continue;
        const auto& d = r.data;
        const std::string& k = r.h[1];
        if (k == "category" && d.size() == 1) {
            out.emplace_back();
            out.back().category = d[0];
        } else if (out.empty()) {
            continue;
        } else if (k == "operator" && d.size() == 1) {
            out.back().optr = d[0];
        } else if (k == "nodeSet" && d.size() == 1) {
            out.back().node_set = d[0];
        } else if (k == "elementSet" && d.size() == 1) {
            out.back().elem_set = d[0];
        } else if (k == "component" && d.size() == 1) {
            out.back().component = inum(d[0]);
        } else if (k == "coefficient" && d.size() == 1) {
            out.back().coef = num(d[0]);
        } else if (k == "exponent" && d.size() == 1) {
            out.back().expnt = num(d[0]);
        } else if (k == "activeTime" && !d.empty()) {
            out.back().t0 = num(d[0]);
            out.back().t1 = d.size() > 1 ? num(d[1]) : 1e100;
        } else if (k == "targetValue" && !d.empty()) {
            for (const auto& x : d) out.back().targets.push_back(num(x));
        }
    }
    return out;
}

struct DesignVar {
    std::string category, elem_set;
    int component = 0;
    std::vector<double> coefs;
    double t0 = 0.0, t1 = 1e100;
};
std::vector<DesignVar> read_design_vars(const std::string& path) {
    std::vector<DesignVar> out;
    for (const Record& r : read_records(path)) {
        if (r.h[0] != "designVariables") continue;
        const auto& d = r.data;
        const std::string& k = r.h[1];
        if (k == "category" && d.size() == 1) {
            if (d[0] != "modulus" && d[0] != "shearModulus" && d[0] != "poissonRatio" && d[0] != "area" &&
                d[0] != "areaMoment" && d[0] != "polarMoment")
                throw Fail("design variable category " + d[0] + " is not on the GPU path");
            out.emplace_back();
            out.back().category = d[0];
        } else if (out.empty()) {
            continue;
        } else if (k == "elementSet" && d.size() == 1) {
            out.back().elem_set = d[0];
        } else if (k == "component" && d.size() == 1) {
            out.back().component = inum(d[0]);
        } else if (k == "coefficients" && d.size() == 1) {
            out.back().coefs.push_back(num(d[0]));
        } else if (k == "activeTime" && !d.empty()) {
            out.back().t0 = num(d[0]);
            out.back().t1 = d.size() > 1 ? num(d[1]) : 1e100;
        }
    }
    return out;
}

// ---------------------------------------------------------------------------
// writers (Rust "{:.12e}": no '+', no zero padding in the exponent)
// ---------------------------------------------------------------------------
std::string rust_exp(double x) {
    if (std::isnan(x)) return "NaN";
    if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.12e", x);
    std::string s(buf);
    const size_t e = s.find('e');
    return s.substr(0, e) + "e" + std::to_string(std::atoi(s.c_str() + e + 1));
}

std::pair<std::string, std::string> split_root(const std::string& f) {
    const size_t i = f.find('.');
    return i == std::string::npos ? std::make_pair(f, std::string()) : std::make_pair(f.substr(0, i), f.substr(i));
}

void write_text(const std::string& path, const std::string& s) {
    std::ofstream f(path, std::ios::binary);
    if (!f) throw Fail("could not open file " + path);
    f << s;
}

// ---------------------------------------------------------------------------
// the runner
// ---------------------------------------------------------------------------
// The reference's solver log lines (matrix_functions.rs:358-359), scraped by
// job scripts for "Total CG iterations:"; the second line carries this
// library's final ||f - A u|| / ||f|| (the reference prints g^T M^-1 g).
void cg_log(long long iterations, double residual) {
    std::printf("Total CG iterations: %lld\nFinal residual norm: %.17g\n", iterations, residual);
    std::fflush(stdout);
}

struct Runner {
    std::string base;
    std::vector<Command> cmds;
    Model model;
    std::vector<Constraint> cons;
    std::vector<Load> loads;
    std::vector<ObjTerm> obj;
    std::vector<DesignVar> dvs;
    std::map<int, int> nidx, eidx;
    std::map<std::string, int> set_id, elset_id;
    asend_ctx* ctx = nullptr;
    int dpn = 3, n_nodes = 0;
    bool solved = false, dynamic = false;
    double time = 0.0;
    std::vector<double> u, eig, freq, modes, obj_vals, obj_grad;
    std::map<std::string, std::string> solve_kv;

    ~Runner() {
        if (ctx) asend_destroy(ctx);
    }
    std::string path(const std::string& f) const {
        if (!f.empty() && f[0] == '/') return f;
        std::ifstream probe(f);
        return probe ? f : base + "/" + f;
    }
    void check(int rc, const char* what) {
        if (rc < 0) throw Fail(std::string(what) + " failed: " + asend_last_error(ctx));
    }

    void setup() {
        const Model& m = model;
        if (m.elem_type < 0) throw Fail("the model has no elements");
        for (size_t i = 0; i < m.node_labels.size(); ++i) nidx[m.node_labels[i]] = (int)i;
        for (size_t i = 0; i < m.elem_labels.size(); ++i) eidx[m.elem_labels[i]] = (int)i;
        const int ne = (int)m.elem_labels.size();
        n_nodes = (int)m.node_labels.size();
        dpn = (m.elem_type == 41 || m.elem_type == 2) ? 6 : 3;
        std::vector<int32_t> conn;
        for (const auto& row : m.conn)
            for (int v : row) conn.push_back(nidx.at(v));
        std::vector<double> E(ne, NAN), nu(ne, NAN), rho(ne, NAN), thk(ne, NAN);
        std::vector<double> props((size_t)ne * 9, NAN), damp((size_t)ne * 36, 0.0);
        std::vector<double> sec_abd((size_t)ne * 81, 0.0), sec_ms((size_t)ne * 36, 0.0);
        std::vector<char> has_sec(ne, 0);
        std::vector<double> beam((size_t)ne * 10, NAN);  // area, I1..I5, J, xy-plane direction
        std::vector<double> beam_c((size_t)ne * 36, 0.0), beam_m((size_t)ne * 36, 0.0);  // given matrices
        bool beam_given = false;
        bool ortho = false, damped = false, layered = false;
        for (const Section& s : m.sections) {
            if (!m.elem_sets.count(s.elset)) throw Fail("section without a valid elementSet");
            std::string mat_name = s.material;
            double t = NAN;
            if (s.type == "shell") {
                // layup: layers of (material, thickness, angle) about zOffset
                // (element_properties.rs:75-222, :766-876)
                if (s.layers.empty()) throw Fail("shell section without layers");
                const double phi = shell_frame_angle(s);
                std::vector<double> rows;
                t = 0.0;
                for (const Layer& l : s.layers) {
                    const Material& lm = m.materials.at(l.material);
                    if (lm.E.empty() || lm.nu.empty()) throw Fail("material " + l.material + " needs E and nu");
                    if (!lm.damping.empty()) throw Fail("material damping takes solid sections");
                    const double g12 = lm.G.empty() ? lm.E[0] / (2.0 * (1.0 + lm.nu[0])) : lm.G[0];
                    const double r[7] = {lm.E[0], lm.E[1], lm.nu[0], g12, lm.density, l.thickness, l.angle + phi};
                    rows.insert(rows.end(), r, r + 7);
                    t += l.thickness;
                }
                const bool one_iso = s.layers.size() == 1 && s.z_offset == 0.0 && rows[0] == rows[1] &&
                                     std::fabs(rows[3] - rows[0] / (2.0 * (1.0 + rows[2]))) <= 1e-9 * rows[3];
                double abd[81], ms[36];
                if (!one_iso) {
                    check(asend_shell_section((int)s.layers.size(), rows.data(), s.z_offset, abd, ms), "shell_section");
                    layered = true;
                }
                for (int lab : m.elem_sets.at(s.elset)) {
                    const int e = eidx.at(lab);
                    E[e] = rows[0];
                    nu[e] = rows[2];
                    rho[e] = rows[4];
                    thk[e] = t;
                    if (!one_iso) {
                        std::copy(abd, abd + 81, sec_abd.begin() + (size_t)e * 81);
                        std::copy(ms, ms + 36, sec_ms.begin() + (size_t)e * 36);
                        has_sec[e] = 1;
                    }
                }
                continue;
            } else if (s.type == "beam") {
                // The reference's element frame is the section orientation
                // (default the global axes, section.rs:150) and it
                // differentiates along xDir, so xDir must lie along the
                // element; the GPU element takes x from the element.  An
                // opposite xDir is the same frame turned half a turn about y:
                // I1 = int z and I5 = int yz change sign.
                std::vector<double> ori = s.orientation;
                if (ori.empty()) ori = {1.0, 0.0, 0.0, 0.0, 1.0, 0.0};
                const double xn = std::sqrt(ori[0] * ori[0] + ori[1] * ori[1] + ori[2] * ori[2]);
                for (int lab : m.elem_sets.at(s.elset)) {
                    const int e = eidx.at(lab);
                    const int n0 = nidx.at(m.conn[e][0]), n1 = nidx.at(m.conn[e][1]);
                    double ax[3], an = 0.0, c = 0.0;
                    for (int j = 0; j < 3; ++j) {
                        ax[j] = m.coords[3 * (size_t)n1 + j] - m.coords[3 * (size_t)n0 + j];
                        an += ax[j] * ax[j];
                    }
                    an = std::sqrt(an);
                    for (int j = 0; j < 3; ++j) c += ax[j] * ori[j] / (an * xn);
                    if (std::fabs(c) < 1.0 - 1e-9)
                        throw Fail("beam sections whose orientation x direction is not along the element");
                    double im[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
                    for (size_t k = 0; k < s.I.size() && k < 5; ++k) im[k] = s.I[k];
                    if (c < 0.0) {
                        im[0] = -im[0];
                        im[4] = -im[4];
                    }
                    const double row[10] = {s.area, im[0], im[1], im[2], im[3], im[4], s.J, ori[3], ori[4], ori[5]};
                    std::copy(row, row + 10, beam.begin() + (size_t)e * 10);
                    // given matrices; against x: the half turn about y flips strains 2 and 5
                    // and velocities 1, 3, 4, 6
                    const double ts[6] = {1, -1, 1, 1, -1, 1}, tm[6] = {-1, 1, -1, -1, 1, -1};
                    for (int i = 0; i < 6; ++i)
                        for (int j = 0; j < 6; ++j) {
                            if (!s.stiffness.empty())
                                beam_c[(size_t)e * 36 + 6 * i + j] =
                                    s.stiffness[6 * i + j] * (c < 0.0 ? ts[i] * ts[j] : 1.0);
                            if (!s.mass.empty())
                                beam_m[(size_t)e * 36 + 6 * i + j] = s.mass[6 * i + j] * (c < 0.0 ? tm[i] * tm[j] : 1.0);
                        }
                    beam_given = beam_given || !s.stiffness.empty() || !s.mass.empty();
                }
            } else if (s.type != "solid") {
                throw Fail(s.type + " sections are not on the GPU path");
            }
            const Material& mt = m.materials.at(mat_name);
            if (mt.E.empty() || mt.nu.empty()) throw Fail("material " + mat_name + " needs E and nu");
            const double Giso = mt.E[0] / (2.0 * (1.0 + mt.nu[0]));
            std::vector<double> G = mt.G.empty() ? std::vector<double>(3, Giso) : mt.G;
            const bool iso = mt.E[0] == mt.E[1] && mt.E[0] == mt.E[2] && mt.nu[0] == mt.nu[1] &&
                             mt.nu[0] == mt.nu[2] && G[0] == G[1] && G[0] == G[2] &&
                             std::fabs(G[0] - Giso) <= 1e-9 * std::fabs(G[0]);
            if (!iso) {  // orthotropic constants through the compliance form (element_properties.rs:648-764)
                if (s.type != "solid" || mt.G.empty())
                    throw Fail("orthotropic materials take solid sections with E, nu and G lists");
                ortho = true;
            }
            if (!mt.damping.empty()) {
                if (s.type != "solid") throw Fail("material damping takes solid sections");
                damped = true;
            }
            for (int lab : m.elem_sets.at(s.elset)) {
                const int e = eidx.at(lab);
                E[e] = mt.E[0];
                nu[e] = mt.nu[0];
                rho[e] = mt.density;
                thk[e] = t;
                for (int k = 0; k < 3; ++k) {
                    props[(size_t)e * 9 + k] = mt.E[k];
                    props[(size_t)e * 9 + 3 + k] = mt.nu[k];
                    props[(size_t)e * 9 + 6 + k] = G[k];
                }
                if (!mt.damping.empty()) std::copy(mt.damping.begin(), mt.damping.end(), damp.begin() + (size_t)e * 36);
            }
        }
        for (int e = 0; e < ne; ++e)
            if (std::isnan(E[e])) throw Fail("elements without a section");
        ctx = asend_create(0);
        if (!ctx) throw Fail("asend_create failed");
        check(asend_set_mesh(ctx, m.elem_type, n_nodes, m.coords.data(), ne, conn.data(), E.data(), nu.data(),
                             rho.data(), m.elem_type == 41 ? thk.data() : nullptr),
              "set_mesh");
        if (m.elem_type == 2) {
            for (double v : beam)
                if (std::isnan(v)) throw Fail("beam2 elements need a beam section");
            check(asend_set_beam_sections(ctx, beam.data()), "set_beam_sections");
            if (beam_given)
                check(asend_set_beam_section_matrices(ctx, beam_c.data(), beam_m.data()), "set_beam_section_matrices");
        }
        if (ortho) check(asend_set_orthotropic(ctx, props.data()), "set_orthotropic");
        if (layered) {
            // elements outside the layered sections keep one isotropic layer
            for (int e = 0; e < ne; ++e) {
                if (has_sec[e]) continue;
                const double r[7] = {E[e], E[e], nu[e], E[e] / (2.0 * (1.0 + nu[e])), rho[e], thk[e], 0.0};
                check(asend_shell_section(1, r, 0.0, &sec_abd[(size_t)e * 81], &sec_ms[(size_t)e * 36]),
                      "shell_section");
            }
            check(asend_set_shell_sections(ctx, sec_abd.data(), sec_ms.data()), "set_shell_sections");
        }
        if (damped) check(asend_set_damping(ctx, 0.0, 0.0, damp.data()), "set_damping");
        for (const auto& name : m.node_set_order) {
            std::vector<int32_t> v;
            for (int lab : m.node_sets.at(name)) v.push_back(nidx.at(lab));
            set_id[name] = asend_add_node_set(ctx, (int)v.size(), v.data());
            check(set_id[name], "add_node_set");
        }
        if (!set_id.count("all")) {
            std::vector<int32_t> v(n_nodes);
            for (int i = 0; i < n_nodes; ++i) v[i] = i;
            set_id["all"] = asend_add_node_set(ctx, n_nodes, v.data());
        }
        for (const auto& name : m.elem_set_order) {
            std::vector<int32_t> v;
            for (int lab : m.elem_sets.at(name)) v.push_back(eidx.at(lab));
            elset_id[name] = asend_add_element_set(ctx, (int)v.size(), v.data());
            check(elset_id[name], "add_element_set");
        }
        for (const Constraint& c : cons) {
            std::vector<int32_t> sets, comps(c.dof.begin(), c.dof.end());
            for (const auto& s : c.sets) sets.push_back(set_id.at(s));
            check(asend_add_constraint(ctx, (int)sets.size(), sets.data(), comps.data(), c.coef.data(), c.rhs),
                  "add_constraint");
        }
        for (const Load& l : loads) {
            if (!(l.t0 <= time && time <= l.t1)) continue;
            if (l.type == "nodalForce") {
                check(asend_add_nodal_force(ctx, 0, set_id.at(l.node_set), l.load), "add_nodal_force");
            } else if (l.type == "surfaceTraction") {
                check(asend_add_surface_traction(ctx, 0, elset_id.at(l.elem_set), l.norm_dir, l.norm_tol, l.load),
                      "add_surface_traction");
            } else if (l.type == "surfacePressure") {
                check(asend_add_surface_pressure(ctx, 0, elset_id.at(l.elem_set), l.norm_dir, l.norm_tol, l.load[0]),
                      "add_surface_pressure");
            } else {
                const int kind = l.type == "bodyForce" ? ASEND_LOAD_BODY_FORCE
                                 : l.type == "gravitational" ? ASEND_LOAD_GRAVITY : ASEND_LOAD_CENTRIFUGAL;
                check(asend_add_body_load(ctx, 0, elset_id.at(l.elem_set), kind, l.load, l.omega, l.center, l.axis),
                      "add_body_load");
            }
        }
    }

    asend_solve_opts opts(bool modal) const {
        asend_solve_opts o{};
        o.method = ASEND_METHOD_FP64;
        o.precond = ASEND_PC_JACOBI;
        auto it = solve_kv.find("convergenceTol");
        o.rel_tol = modal ? 1e-10 : (it == solve_kv.end() ? 1e-12 : num(it->second));
        it = solve_kv.find("maxIterations");
        o.max_iter = it == solve_kv.end() ? (modal ? 100000 : 0) : inum(it->second);
        o.graph_iters = 16;
        return o;
    }

    void ensure_ctx() {
        if (!ctx) setup();
    }

    void solve(const Command& c) {
        for (const auto& kv : c.kv) solve_kv[kv.first] = kv.second;
        for (const char* k : {"thermal", "diffusion", "fluid", "nonlinearGeom"})
            if (solve_kv.count(k) && solve_kv[k].find("yes") != std::string::npos)
                throw Fail(std::string(k) + " analysis is not on the GPU path");
        if (solve_kv.count("userUpdate") && solve_kv["userUpdate"].find("yes") != std::string::npos)
            throw Fail("user update hooks are not on the GPU path");
        if (ctx) { asend_destroy(ctx); ctx = nullptr; }
        setup();
        // lumpMass: row-sum lumped mass in dynamic runs (element_equations.rs:950-971)
        const bool lump = solve_kv.count("lumpMass") && solve_kv["lumpMass"].find("yes") != std::string::npos;
        check(asend_set_lumped_mass(ctx, lump ? 1 : 0), "set_lumped_mass");
        const asend_solve_opts o = opts(false);
        asend_solve_stats st{};
        const int n = asend_n_dof(ctx);
        dynamic = solve_kv.count("dynamic") && solve_kv["dynamic"].find("yes") != std::string::npos;
        u.assign(n, 0.0);
        if (!dynamic) {
            check(asend_assemble(ctx, 64, 0, 0.0, 0.0, 0.0), "assemble");
            const int rc = asend_static_solve(ctx, &o, u.data(), &st);
            check(rc, "static_solve");
            if (rc == ASEND_NONFINITE) throw Fail("static solve turned non-finite");
            cg_log(st.iterations, st.rel_residual);
        } else {
            const double dt = num(solve_kv.at("timeStep"));
            const double beta = solve_kv.count("newmarkBeta") ? num(solve_kv["newmarkBeta"]) : 0.25;
            const double gamma = solve_kv.count("newmarkGamma") ? num(solve_kv["newmarkGamma"]) : 0.5;
            const int steps = (int)std::lround(num(solve_kv.at("simPeriod")) / dt);
            for (const Load& l : loads)
                if (l.t0 != 0.0 || l.t1 != 1e100) throw Fail("time-windowed loads in dynamic jobs are not on the GPU path");
            check(asend_assemble(ctx, 64, 1, dt, beta, gamma), "assemble");
            std::vector<double> amp(steps, 1.0);
            const int rc = asend_newmark_run(ctx, &o, steps, amp.data(), -1, nullptr, u.data(), &st);
            check(rc, "newmark_run");
            if (rc == ASEND_NONFINITE) throw Fail("Newmark run turned non-finite");
            cg_log(st.iterations, st.rel_residual);
            time = steps * dt;
        }
        solved = true;
    }

    void modal(const Command& c) {
        if (c.get("type", "frequency") != "frequency") throw Fail("buckling analysis is not on the GPU path");
        ensure_ctx();
        asend_eigen_opts eo{};
        eo.n_modes = c.kv.count("numModes") ? inum(c.get("numModes")) : 10;
        eo.block_size = 2;
        eo.shift = c.kv.count("targetEigenvalue") ? num(c.get("targetEigenvalue")) : 0.0;
        eo.tol = 1e-8;
        eo.inner = opts(true);
        const int n = asend_n_dof(ctx);
        eig.assign(eo.n_modes, 0.0);
        freq.assign(eo.n_modes, 0.0);
        modes.assign((size_t)eo.n_modes * n, 0.0);
        asend_eigen_stats st{};
        const int rc = asend_eigen_solve(ctx, &eo, eig.data(), freq.data(), modes.data(), nullptr, &st);
        check(rc, "eigen_solve");
        if (rc != ASEND_OK) throw Fail("eigen solve did not converge");
        cg_log(st.inner_iterations, st.max_rel_residual);
        eig.resize(st.n_found);
        freq.resize(st.n_found);
    }

    void calc_objective() {
        if (!solved) throw Fail("calcObjective before a solve");
        if (dynamic) throw Fail("time-integrated objectives of dynamic runs are not on the GPU path");
        obj_vals.clear();
        for (const ObjTerm& t : obj) {
            if (t.category != "displacement" || t.optr != "powerNorm")
                throw Fail("objective " + t.category + "/" + t.optr + " is not on the GPU path");
            if (t.component < 1) throw Fail("objective term without a component");
            if (!(t.t0 <= time && time <= t.t1)) { obj_vals.push_back(0.0); continue; }
            const auto& labs = model.node_sets.at(t.node_set);
            double sum = 0.0;
            for (size_t i = 0; i < labs.size(); ++i) {
                const double tg = t.targets.empty() ? 0.0 : (t.targets.size() == 1 ? t.targets[0] : t.targets[i]);
                sum += std::pow(u[(size_t)nidx.at(labs[i]) * dpn + t.component - 1] - tg, t.expnt);
            }
            obj_vals.push_back(t.coef * std::pow(sum, 1.0 / t.expnt));  // objective_meth.rs:329-337
        }
    }

    void calc_gradient() {
        if (!solved) throw Fail("calcObjGradient before a solve");
        if (dynamic) throw Fail("transient objective gradients are not on the GPU path");
        obj_grad.assign(dvs.size(), 0.0);
        const asend_solve_opts o = opts(false);
        for (const ObjTerm& t : obj) {
            if (t.category != "displacement" || t.optr != "powerNorm" || t.expnt != 1.0)
                throw Fail("gradients of displacement powerNorm terms of exponent 1 only");
            if (!(t.t0 <= time && time <= t.t1)) continue;
            check(asend_set_objective(ctx, ASEND_OBJ_DISPLACEMENT, set_id.at(t.node_set), t.component, t.coef),
                  "set_objective");
            double L = 0.0;
            asend_solve_stats st{};
            check(asend_adjoint_gradient(ctx, &o, &L, nullptr, &st), "adjoint_gradient");
            cg_log(st.iterations, st.rel_residual);
            for (size_t i = 0; i < dvs.size(); ++i) {
                const DesignVar& dv = dvs[i];
                if (!(dv.t0 <= time && time <= dv.t1)) continue;
                const int cat = dv.category == "modulus"        ? ASEND_DV_MODULUS
                                : dv.category == "shearModulus" ? ASEND_DV_SHEAR_MODULUS
                                : dv.category == "area"         ? ASEND_DV_AREA
                                : dv.category == "areaMoment"   ? ASEND_DV_AREA_MOMENT
                                : dv.category == "polarMoment"  ? ASEND_DV_POLAR_MOMENT
                                                                : ASEND_DV_POISSON_RATIO;
                double g = 0.0;
                check(asend_material_dv_gradient(ctx, cat, dv.component, elset_id.at(dv.elem_set), (int)dv.coefs.size(),
                                                 dv.coefs.empty() ? nullptr : dv.coefs.data(), &g),
                      "material_dv_gradient");
                obj_grad[i] += g;
            }
        }
    }

    void write_nodes(const Command& c) {
        if (c.lists.count("timeSteps") || c.kv.count("timeSteps")) throw Fail("time-step histories are not written by the GPU path");
        if (!solved) throw Fail("writeNodeResults before a solve");
        Strs fields = c.lists.count("fields") ? c.lists.at("fields") : Strs{"displacement"};
        std::vector<double> rf;
        std::string head = "node,";
        for (const auto& f : fields) {
            if (f == "displacement") head += "U1,U2,U3,R1,R2,R3,";
            else if (f == "reactionForce") head += "RF1,RF2,RF3,RM1,RM2,RM3,";
            else throw Fail("node field " + f + " is not written by the GPU path");
        }
        if (std::find(fields.begin(), fields.end(), "reactionForce") != fields.end()) {
            if (dynamic) throw Fail("reaction forces of a dynamic run are not written by the GPU path");
            // R(u) = K u without the penalty terms (model_output.rs:207-216)
            int64_t nnz = 0;
            check(asend_get_csr(ctx, 2, &nnz, nullptr, nullptr, nullptr), "get_csr");
            const int n = asend_n_dof(ctx);
            std::vector<int64_t> rp(n + 1);
            std::vector<int32_t> col(nnz);
            std::vector<double> val(nnz);
            check(asend_get_csr(ctx, 2, &nnz, rp.data(), col.data(), val.data()), "get_csr");
            rf.assign(n, 0.0);
            for (int i = 0; i < n; ++i)
                for (int64_t k = rp[i]; k < rp[i + 1]; ++k) rf[i] += val[k] * u[col[k]];
        }
        head += "time\n";
        const std::string set = c.get("nodeSet", "all");
        const std::vector<int>& labs = model.node_sets.count(set) ? model.node_sets.at(set) : model.node_labels;
        std::string out = head;
        for (int lab : labs) {
            const int i = nidx.at(lab);
            out += std::to_string(lab) + ",";
            for (const auto& f : fields) {
                const std::vector<double>& v = f == "displacement" ? u : rf;
                for (int q = 0; q < 6; ++q) out += rust_exp(q < dpn ? v[(size_t)i * dpn + q] : 0.0) + ",";
            }
            out += rust_exp(-1.0) + "\n";
        }
        write_text(c.get("fileName"), out);
    }

    void write_modal(const Command& c) {
        if (eig.empty()) throw Fail("writeModalResults before modalAnalysis");
        std::string out = "mode,eigenvalue,frequency\n";
        for (size_t k = 0; k < eig.size(); ++k)
            out += std::to_string(k) + "," + rust_exp(eig[k]) + "," + rust_exp(freq[k]) + "\n";
        const std::string fn = c.get("fileName");
        write_text(fn, out);
        if (c.get("writeModes") == "yes") {
            const auto re = split_root(fn);
            const int n = n_nodes * dpn;
            for (size_t k = 0; k < eig.size(); ++k) {
                std::string s = "Node,U1,U2,U3,R1,R2,R3\n";
                for (int i = 0; i < n_nodes; ++i) {
                    s += std::to_string(model.node_labels[i]);
                    for (int q = 0; q < 6; ++q) s += "," + rust_exp(q < dpn ? modes[k * n + (size_t)i * dpn + q] : 0.0);
                    s += "\n";
                }
                write_text(re.first + "_mode" + std::to_string(k) + re.second, s);
            }
        }
    }

    void write_objective(const Command& c) {
        if (obj_vals.empty() && !obj.empty()) throw Fail("writeObjective before calcObjective");
        const Strs inc = c.lists.count("include") ? c.lists.at("include") : Strs{};
        std::string out = "objectiveTerm,value";
        for (const auto& f : inc) out += "," + f;
        out += "\n";
        for (size_t i = 0; i < obj_vals.size(); ++i) {
            out += std::to_string(i) + "," + rust_exp(obj_vals[i]);
            for (const auto& f : inc) {
                const ObjTerm& t = obj[i];
                if (f == "category") out += "," + t.category;
                else if (f == "operator") out += "," + t.optr;
                else if (f == "component") out += "," + std::to_string(t.component);
                else if (f == "coefficient") out += "," + rust_exp(t.coef);
                else if (f == "exponent") out += "," + rust_exp(t.expnt);
                else if (f == "nodeSet") out += "," + t.node_set;
                else if (f == "elementSet") out += "," + t.elem_set;
                else if (f == "activeTime") out += "," + rust_exp(t.t0);
                else throw Fail("unrecognized field '" + f + "' for writeObjective");
            }
            out += "\n";
        }
        const std::string fn = c.get("fileName");
        write_text(fn, out);
        if (c.get("writeGradient") == "yes") {
            if (obj_grad.size() != dvs.size()) throw Fail("writeGradient before calcObjGradient");
            const auto re = split_root(fn);
            std::string g = "designVariable,objGrad\n";
            for (size_t i = 0; i < obj_grad.size(); ++i) g += std::to_string(i) + "," + rust_exp(obj_grad[i]) + "\n";
            write_text(re.first + "_grad" + re.second, g);
        }
    }

    void run() {
        for (const Command& c : cmds) {
            const std::string& n = c.name;
            if (n == "readModelInput") model = read_model(path(c.get("fileName")));
            else if (n == "readConstraints") { auto v = read_constraints(path(c.get("fileName"))); cons.insert(cons.end(), v.begin(), v.end()); }
            else if (n == "readLoads") { auto v = read_loads(path(c.get("fileName"))); loads.insert(loads.end(), v.begin(), v.end()); }
            else if (n == "readObjectiveInput") { auto v = read_objective(path(c.get("fileName"))); obj.insert(obj.end(), v.begin(), v.end()); }
            else if (n == "readDesignVarInput") { auto v = read_design_vars(path(c.get("fileName"))); dvs.insert(dvs.end(), v.begin(), v.end()); }
            else if (n == "solvePrep") { for (const auto& kv : c.kv) solve_kv[kv.first] = kv.second; }
            else if (n == "solve") solve(c);
            else if (n == "zeroSolution") { std::fill(u.begin(), u.end(), 0.0); }
            else if (n == "modalAnalysis") modal(c);
            else if (n == "calcObjective") calc_objective();
            else if (n == "calcObjGradient") calc_gradient();
            else if (n == "writeNodeResults") write_nodes(c);
            else if (n == "writeModalResults") write_modal(c);
            else if (n == "writeObjective") write_objective(c);
            else throw Fail("job command " + n + " is not on the GPU path");
        }
    }

    // --parse: every input file named by the job, as JSON (no device use)
    std::string summary() {
        for (const Command& c : cmds) {
            const std::string& n = c.name;
            if (n == "readModelInput") model = read_model(path(c.get("fileName")));
            else if (n == "readConstraints") { auto v = read_constraints(path(c.get("fileName"))); cons.insert(cons.end(), v.begin(), v.end()); }
            else if (n == "readLoads") { auto v = read_loads(path(c.get("fileName"))); loads.insert(loads.end(), v.begin(), v.end()); }
            else if (n == "readObjectiveInput") { auto v = read_objective(path(c.get("fileName"))); obj.insert(obj.end(), v.begin(), v.end()); }
            else if (n == "readDesignVarInput") { auto v = read_design_vars(path(c.get("fileName"))); dvs.insert(dvs.end(), v.begin(), v.end()); }
        }
        std::ostringstream j;
        j.precision(17);
        auto ivec = [&](const std::vector<int>& v) {
            std::string s = "[";
            for (size_t i = 0; i < v.size(); ++i) s += (i ? "," : "") + std::to_string(v[i]);
            return s + "]";
        };
        j << "{\"commands\":[";
        for (size_t i = 0; i < cmds.size(); ++i) j << (i ? "," : "") << "\"" << cmds[i].name << "\"";
        j << "],\"elem_type\":" << model.elem_type << ",\"node_labels\":" << ivec(model.node_labels) << ",\"coords\":[";
        for (size_t i = 0; i < model.coords.size(); ++i) j << (i ? "," : "") << model.coords[i];
        j << "],\"conn\":[";
        for (size_t i = 0; i < model.conn.size(); ++i) j << (i ? "," : "") << ivec(model.conn[i]);
        j << "],\"node_sets\":{";
        for (size_t i = 0; i < model.node_set_order.size(); ++i)
            j << (i ? "," : "") << "\"" << model.node_set_order[i] << "\":" << ivec(model.node_sets[model.node_set_order[i]]);
        j << "},\"elem_sets\":{";
        for (size_t i = 0; i < model.elem_set_order.size(); ++i)
            j << (i ? "," : "") << "\"" << model.elem_set_order[i] << "\":" << ivec(model.elem_sets[model.elem_set_order[i]]);
        j << "},\"constraints\":[";
        for (size_t i = 0; i < cons.size(); ++i) {
            j << (i ? "," : "") << "{\"terms\":[";
            for (size_t k = 0; k < cons[i].sets.size(); ++k)
                j << (k ? "," : "") << "[\"" << cons[i].sets[k] << "\"," << cons[i].dof[k] << "," << cons[i].coef[k] << "]";
            j << "],\"rhs\":" << cons[i].rhs << "}";
        }
        j << "],\"loads\":[";
        for (size_t i = 0; i < loads.size(); ++i) {
            j << (i ? "," : "") << "{\"type\":\"" << loads[i].type << "\",\"load\":[";
            for (int q = 0; q < 6; ++q) j << (q ? "," : "") << loads[i].load[q];
            j << "]}";
        }
        j << "],\"objective\":[";
        for (size_t i = 0; i < obj.size(); ++i)
            j << (i ? "," : "") << "{\"category\":\"" << obj[i].category << "\",\"component\":" << obj[i].component
              << ",\"coefficient\":" << obj[i].coef << ",\"exponent\":" << obj[i].expnt << "}";
        j << "],\"design_vars\":[";
        for (size_t i = 0; i < dvs.size(); ++i) {
            j << (i ? "," : "") << "{\"category\":\"" << dvs[i].category << "\",\"component\":" << dvs[i].component
              << ",\"elementSet\":\"" << dvs[i].elem_set << "\",\"coefficients\":[";
            for (size_t k = 0; k < dvs[i].coefs.size(); ++k) j << (k ? "," : "") << dvs[i].coefs[k];
            j << "]}";
        }
        j << "],\"rust_exp_samples\":[\"" << rust_exp(1.5) << "\",\"" << rust_exp(-2.5e-7) << "\",\"" << rust_exp(0.0)
          << "\"]}";
        return j.str();
    }
};

}  // namespace

int main(int argc, char** argv) {
    const bool parse_only = argc == 3 && std::strcmp(argv[1], "--parse") == 0;
    if (argc != 2 && !parse_only) {
        std::fprintf(stderr, "usage: asend_run_job [--parse] <job.yaml>\n");
        return 2;
    }
    const std::string job = argv[argc - 1];
    try {
        Runner r;
        const size_t slash = job.find_last_of('/');
        r.base = slash == std::string::npos ? "." : job.substr(0, slash);
        r.cmds = read_job(job);
        if (parse_only) {
            std::printf("%s\n", r.summary().c_str());
            return 0;
        }
        r.run();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "Error: %s\n", e.what());
        return 1;
    }
    return 0;
}
