// Case-file reader: a small YAML reader for the subset cuIBM case files use
// (block sequences of maps, nested maps, flow sequences [a, b], scalars,
// '#' comments) and the mapping of its tree onto Params with the reference's
// defaults and command-line overrides.
//
// Reference behaviour kept:
//   defaults             src/io/io.cu:145-197 (initialiseDefaultDB) and the local
//                        defaults of io/parseSimulationFile.cu:parseSimulation
//   simParams.yaml       io/parseSimulationFile.cu (unknown SolverType -> NAVIER_STOKES
//                        with a warning; unknown preconditioner -> NONE; startStep is read
//                        but the reference never stores it, so it stays 0 - except with
//                        restart: true, where the library continues from that step's state)
//   flow.yaml            io/parseFlowFile.cu (bad location/type is an error here, where
//                        the reference prints and calls exit(0))
//   domain.yaml          io/parseDomainFile.cu (only the description is read here;
//                        geometry.cpp builds the grid)
//   bodies.yaml          io/parseBodiesFile.cu (circle and points bodies; motion keys)
//   command line         io/io.cu:207-299 (commandLineParse1/2)
#include "config.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace cuibm {
namespace {

struct Node {
    enum Kind { Null, Scalar, Seq, Map } kind = Null;
    std::string text;
    std::vector<std::shared_ptr<Node>> seq;
    std::vector<std::pair<std::string, std::shared_ptr<Node>>> map;

    const Node *get(const std::string &k) const {
        if (kind != Map) return nullptr;
        for (auto &kv : map)
            if (kv.first == k) return kv.second.get();
        return nullptr;
    }
};
using NodeP = std::shared_ptr<Node>;

struct Line {
    int indent;
    std::string text;
    int lineno;
};

std::string trim(const std::string &s)
{
    size_t a = s.find_first_not_of(" \t\r");
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(" \t\r");
    return s.substr(a, b - a + 1);
}

NodeP parse_flow(const std::string &s, size_t &p);

NodeP scalar(const std::string &t)
{
    auto n = std::make_shared<Node>();
    n->kind = Node::Scalar;
    std::string v = trim(t);
    if (v.size() >= 2 && (v[0] == '"' || v[0] == '\'') && v.back() == v[0]) v = v.substr(1, v.size() - 2);
    n->text = v;
    return n;
}

NodeP parse_flow(const std::string &s, size_t &p)
{
    while (p < s.size() && s[p] == ' ') ++p;
    if (p < s.size() && s[p] == '[') {
        auto n = std::make_shared<Node>();
        n->kind = Node::Seq;
        ++p;
        for (;;) {
            while (p < s.size() && (s[p] == ' ' || s[p] == ',')) ++p;
            if (p >= s.size()) throw std::runtime_error("unterminated '['");
            if (s[p] == ']') {
                ++p;
                break;
            }
            n->seq.push_back(parse_flow(s, p));
        }
        return n;
    }
    size_t q = p;
    while (q < s.size() && s[q] != ',' && s[q] != ']') ++q;
    auto n = scalar(s.substr(p, q - p));
    p = q;
    return n;
}

NodeP value_node(const std::string &v)
{
    std::string t = trim(v);
    if (!t.empty() && t[0] == '[') {
        size_t p = 0;
        return parse_flow(t, p);
    }
    return scalar(t);
}

// split "key: value" (value may be empty)
bool split_key(const std::string &t, std::string &key, std::string &val)
{
    size_t c = t.find(':');
    if (c == std::string::npos) return false;
    key = trim(t.substr(0, c));
    val = trim(t.substr(c + 1));
    return !key.empty();
}

NodeP parse_block(const std::vector<Line> &L, size_t &i, int indent);

// a map whose entries start at column `indent`; the first entry may already be
// split off (for "- key: value" sequence items)
NodeP parse_map(const std::vector<Line> &L, size_t &i, int indent, const std::string *first)
{
    auto n = std::make_shared<Node>();
    n->kind = Node::Map;
    auto add_entry = [&](const std::string &text, int lineno) {
        std::string k, v;
        if (!split_key(text, k, v))
            throw std::runtime_error("line " + std::to_string(lineno) + ": expected 'key: value'");
        if (v.empty()) {
            if (i < L.size() && L[i].indent > indent)
                n->map.push_back({k, parse_block(L, i, L[i].indent)});
            else if (i < L.size() && L[i].indent == indent && L[i].text.rfind("- ", 0) == 0)
                n->map.push_back({k, parse_block(L, i, L[i].indent)});  // "key:\n- item" at same indent
            else
                n->map.push_back({k, std::make_shared<Node>()});
        } else {
            n->map.push_back({k, value_node(v)});
        }
    };
    if (first) add_entry(*first, i > 0 ? L[i - 1].lineno : 0);
    while (i < L.size() && L[i].indent == indent && L[i].text.rfind("- ", 0) != 0 && L[i].text != "-") {
        std::string t = L[i].text;
        int ln = L[i].lineno;
        ++i;
        add_entry(t, ln);
    }
    return n;
}

NodeP parse_block(const std::vector<Line> &L, size_t &i, int indent)
{
    if (i >= L.size()) return std::make_shared<Node>();
    if (L[i].text.rfind("- ", 0) == 0 || L[i].text == "-") {
        auto n = std::make_shared<Node>();
        n->kind = Node::Seq;
        while (i < L.size() && L[i].indent == indent && (L[i].text.rfind("- ", 0) == 0 || L[i].text == "-")) {
            std::string rest = L[i].text.size() > 1 ? trim(L[i].text.substr(2)) : "";
            int item_indent = indent + 2 + (int)(L[i].text.size() > 2 ? L[i].text.find_first_not_of(' ', 2) - 2 : 0);
            ++i;
            std::string k, v;
            if (rest.empty()) {
                n->seq.push_back(parse_block(L, i, i < L.size() ? L[i].indent : indent + 2));
            } else if (rest[0] != '[' && split_key(rest, k, v)) {
                n->seq.push_back(parse_map(L, i, item_indent, &rest));
            } else {
                n->seq.push_back(value_node(rest));
            }
        }
        return n;
    }
    return parse_map(L, i, indent, nullptr);
}

NodeP parse_yaml_file(const std::string &path, std::string &err)
{
    std::ifstream f(path);
    if (!f) {
        err = "cannot open " + path;
        return nullptr;
    }
    std::vector<Line> L;
    std::string raw;
    int ln = 0;
    while (std::getline(f, raw)) {
        ++ln;
        size_t h = raw.find('#');
        if (h != std::string::npos) raw = raw.substr(0, h);
        for (auto &c : raw)
            if (c == '\t') c = ' ';
        std::string t = trim(raw);
        if (t.empty() || t == "---") continue;
        int ind = (int)raw.find_first_not_of(' ');
        L.push_back({ind, t, ln});
    }
    if (L.empty()) return std::make_shared<Node>();
    try {
        size_t i = 0;
        auto root = parse_block(L, i, L[0].indent);
        if (i != L.size()) {
            err = path + ":" + std::to_string(L[i].lineno) + ": unexpected indentation";
            return nullptr;
        }
        return root;
    } catch (const std::exception &e) {
        err = path + ": " + e.what();
        return nullptr;
    }
}

// ---- scalar conversion (yaml-cpp 0.2 converts through a stringstream) -----
bool to_double(const Node *n, double &v)
{
    if (!n || n->kind != Node::Scalar) return false;
    const char *s = n->text.c_str();
    char *end = nullptr;
    double d = std::strtod(s, &end);
    if (end == s) return false;
    v = d;
    return true;
}
bool to_int(const Node *n, int &v)
{
    if (!n || n->kind != Node::Scalar) return false;
    const char *s = n->text.c_str();
    char *end = nullptr;
    long d = std::strtol(s, &end, 10);
    if (end == s) return false;
    v = (int)d;
    return true;
}
bool to_bool(const Node *n, bool &v)
{
    if (!n || n->kind != Node::Scalar) return false;
    const std::string &t = n->text;
    v = (t == "true" || t == "True" || t == "TRUE" || t == "yes" || t == "1");
    return true;
}
const Node *item(const Node *n, int k) { return (n && n->kind == Node::Seq && k < (int)n->seq.size()) ? n->seq[k].get() : nullptr; }

int precond_from(const std::string &s)
{
    if (s == "DIAGONAL") return PC_DIAGONAL;
    if (s == "SMOOTHED_AGGREGATION") return PC_SMOOTHED_AGGREGATION;
    if (s == "AINV") return PC_AINV;
    return PC_NONE;  // "NONE" and anything unrecognised (parseSimulationFile.cu:19-31)
}

std::string parse_simulation(const Node *doc, Params &P)
{
    if (!doc || doc->kind != Node::Seq) return "simParams.yaml: expected a list";
    for (auto &np : doc->seq) {
        const Node *n = np.get();
        double d;
        int k;
        bool b;
        if (!to_double(n->get("dt"), d)) return "simParams.yaml: missing dt";
        P.dt = d;
        if (!to_int(n->get("nsave"), k)) return "simParams.yaml: missing nsave";
        P.nsave = k;
        if (!to_int(n->get("nt"), k)) return "simParams.yaml: missing nt";
        P.nt = k;
        std::string st = "NAVIER_STOKES_SOLVER";
        if (n->get("SolverType") && n->get("SolverType")->kind == Node::Scalar) st = n->get("SolverType")->text;
        if (st == "NAVIER_STOKES_SOLVER") P.solverType = ST_NAVIERSTOKES;
        else if (st == "FADLUN") P.solverType = ST_FADLUN;
        else if (st == "OSC_CYLINDER") P.solverType = ST_OSC;
        else if (st == "FSI") P.solverType = ST_FSI;
        else if (st == "LUO") P.solverType = ST_LUO;
        else {
            fprintf(stderr, "\nWARNING: unrecognized solverType\nSeting to default: NavierStokes\n\n");
            P.solverType = ST_NAVIERSTOKES;
        }
        if (to_bool(n->get("restart"), b)) P.restart = b;
        // startStep: the reference reads it and never stores it (the run starts at step
        // 0); with restart: true it is the step whose saved state the run continues from
        if (P.restart && to_int(n->get("startStep"), k)) {
            if (k < 0) return "simParams.yaml: startStep must not be negative";
            P.startStep = k;
        }
        P.scaleCV = 2.0;
        if (to_double(n->get("scaleCV"), d)) P.scaleCV = d;
        P.VIV = 0;
        if (to_int(n->get("VIV"), k)) P.VIV = k;
        P.Ured = 3;
        if (to_int(n->get("Ured"), k)) P.Ured = k;
        if (to_bool(n->get("writeOutput"), b)) P.writeOutput = b;
        // linear solvers: values carry over from one entry to the next, as in the reference loop
        std::string linearSolver = "CG", precond = "DIAGONAL";
        double tol = 1e-5;
        int maxIter = 10000;
        const Node *solvers = n->get("linearSolvers");
        if (solvers && solvers->kind == Node::Seq) {
            for (auto &sp : solvers->seq) {
                const Node *s = sp.get();
                std::string system = "velocity";
                if (s->get("system")) system = s->get("system")->text;
                if (s->get("solver")) linearSolver = s->get("solver")->text;
                if (s->get("preconditioner") && s->get("preconditioner")->kind == Node::Scalar)
                    precond = s->get("preconditioner")->text;
                to_double(s->get("tolerance"), tol);
                to_int(s->get("maxIterations"), maxIter);
                LinearSolve ls;
                ls.solver = linearSolver;
                ls.precond = precond_from(precond);
                ls.tolerance = tol;
                ls.maxIterations = maxIter;
                if (s->get("strengthThreshold")) {
                    if (!to_double(s->get("strengthThreshold"), ls.strength))
                        return "simParams.yaml: strengthThreshold must be a number";
                    if (ls.strength < 0 || ls.strength >= 1)
                        return "simParams.yaml: strengthThreshold must be in [0, 1)";
                }
                if (s->get("precision")) {
                    const std::string &pv = s->get("precision")->text;
                    if (pv == "MIXED") ls.precision = PRECISION_MIXED;
                    else if (pv == "DOUBLE" || pv == "FP64") ls.precision = PRECISION_FP64;
                    else return "simParams.yaml: precision must be DOUBLE (or FP64) or MIXED";
                }
                int kry = KRYLOV_BICGSTAB;
                if (s->get("krylov")) {
                    const std::string &kv = s->get("krylov")->text;
                    if (kv == "CG") kry = KRYLOV_CG;
                    else if (kv == "BICGSTAB") kry = KRYLOV_BICGSTAB;
                    else return "simParams.yaml: krylov must be CG or BICGSTAB";
                }
                if (system == "velocity") {
                    P.velocity = ls;
                    P.krylovVelocity = kry;
                } else if (system == "Poisson") {
                    P.poisson = ls;
                    P.krylovPoisson = kry;
                }
            }
        }
    }
    return "";
}

std::string parse_flow_file(const Node *doc, Params &P)
{
    if (!doc || doc->kind != Node::Seq) return "flow.yaml: expected a list";
    for (auto &np : doc->seq) {
        const Node *n = np.get();
        double d;
        if (!to_double(n->get("nu"), d)) return "flow.yaml: missing nu";
        P.nu = d;
        const Node *iv = n->get("initialVelocity");
        if (!to_double(item(iv, 0), P.uInitial) || !to_double(item(iv, 1), P.vInitial))
            return "flow.yaml: missing initialVelocity";
        P.uPerturb = 0;
        P.vPerturb = 0;
        const Node *ip = n->get("initialPerturbation");
        if (ip) {
            to_double(item(ip, 0), P.uPerturb);
            to_double(item(ip, 1), P.vPerturb);
        }
        const Node *bcs = n->get("boundaryConditions");
        if (!bcs || bcs->kind != Node::Seq) return "flow.yaml: missing boundaryConditions";
        for (auto &bp : bcs->seq) {
            const Node *b = bp.get();
            if (!b->get("location")) return "flow.yaml: boundary condition without location";
            std::string loc = b->get("location")->text;
            int L;
            if (loc == "xMinus") L = XMINUS;
            else if (loc == "xPlus") L = XPLUS;
            else if (loc == "yMinus") L = YMINUS;
            else if (loc == "yPlus") L = YPLUS;
            else return "flow.yaml: invalid boundary condition location " + loc;
            for (int c = 0; c < 2; ++c) {
                const Node *comp = b->get(c == 0 ? "u" : "v");
                const Node *t = item(comp, 0);
                double val;
                if (!t || !to_double(item(comp, 1), val)) return "flow.yaml: bad boundary condition at " + loc;
                const std::string &ts = t->text;
                int type;
                if (ts == "DIRICHLET") type = DIRICHLET;
                else if (ts == "NEUMANN") type = NEUMANN;
                else if (ts == "CONVECTIVE") type = CONVECTIVE;
                else if (ts == "PERIODIC") type = PERIODIC;
                else if (ts == "SPECIAL") type = SPECIAL;
                else return "flow.yaml: invalid boundary condition type " + ts;
                P.bc[L][c].type = type;
                P.bc[L][c].value = val;
            }
        }
    }
    return "";
}

std::string parse_domain(const Node *doc, Params &P)
{
    if (!doc || doc->kind != Node::Seq) return "domain.yaml: expected a list";
    bool seen[2] = {false, false};
    for (auto &np : doc->seq) {
        const Node *n = np.get();
        if (!n->get("direction")) return "domain.yaml: missing direction";
        std::string dir = n->get("direction")->text;
        int a = dir == "x" ? 0 : dir == "y" ? 1 : -1;
        if (a < 0) return "domain.yaml: direction must be x or y";
        AxisDesc ax;
        if (!to_double(n->get("start"), ax.start) || !to_double(n->get("mid_h"), ax.mid_h))
            return "domain.yaml: missing start or mid_h";
        const Node *subs = n->get("subDomains");
        if (!subs || subs->kind != Node::Seq || subs->seq.empty()) return "domain.yaml: missing subDomains";
        for (auto &sp : subs->seq) {
            double e, r;
            if (!to_double(sp->get("end"), e) || !to_double(sp->get("stretchRatio"), r))
                return "domain.yaml: subDomain needs end and stretchRatio";
            ax.ends.push_back(e);
            ax.ratios.push_back(r);
        }
        P.axis[a] = ax;
        P.midH = ax.mid_h;
        seen[a] = true;
    }
    if (!seen[0] || !seen[1]) return "domain.yaml: both x and y directions are required";
    return "";
}

std::string parse_bodies(const Node *doc, Params &P, const std::string &folder)
{
    P.bodies.clear();
    if (!doc || doc->kind == Node::Null) return "";
    if (doc->kind != Node::Seq) return "bodies.yaml: expected a list";
    for (auto &np : doc->seq) {
        const Node *n = np.get();
        BodyDesc B;
        // motion keys: absent keys stay 0 (the reference leaves them unset)
        to_double(n->get("xCoefficient"), B.xCoefficient);
        to_double(n->get("xPhase"), B.xPhase);
        to_double(n->get("yCoefficient"), B.yCoefficient);
        to_double(n->get("yPhase"), B.yPhase);
        to_double(n->get("uCoefficient"), B.uCoefficient);
        to_double(n->get("uPhase"), B.uPhase);
        to_double(n->get("vCoefficient"), B.vCoefficient);
        to_double(n->get("vPhase"), B.vPhase);
        to_double(n->get("xfrequency"), B.xfrequency);
        to_double(n->get("yfrequency"), B.yfrequency);
        if (!n->get("type")) return "bodies.yaml: body without type";
        B.type = n->get("type")->text;
        if (B.type == "circle") {
            const Node *o = n->get("circleOptions");
            if (!to_double(item(o, 0), B.cx) || !to_double(item(o, 1), B.cy) || !to_double(item(o, 2), B.R) ||
                !to_int(item(o, 3), B.numPoints))
                return "bodies.yaml: circleOptions needs [cx, cy, R, numPoints, (selfSize, mid_h)]";
            B.selfSize = false;
            if (item(o, 4) && item(o, 5)) {
                to_bool(item(o, 4), B.selfSize);
                to_double(item(o, 5), B.mid_h);
            }
        } else if (B.type == "points") {
            if (!n->get("pointsFile")) return "bodies.yaml: points body without pointsFile";
            std::string fn = folder + "/bodyFiles/" + n->get("pointsFile")->text;
            std::ifstream pf(fn);
            if (!pf) return "cannot open " + fn;
            int np_ = 0;
            pf >> np_;
            if (np_ <= 0) return fn + ": bad point count";
            B.X.resize(np_);
            B.Y.resize(np_);
            for (int i = 0; i < np_; ++i) pf >> B.X[i] >> B.Y[i];
            if (!pf) return fn + ": truncated";
            B.numPoints = np_;
        } else {
            return "bodies.yaml: unsupported body type " + B.type;
        }
        P.bodies.push_back(B);
    }
    return "";
}

template <class T>
bool cli_value(const char *s, T &v)
{
    std::stringstream ss(s);
    ss >> v;
    return !ss.fail();
}

}  // namespace

std::string load_case(const std::string &folder_in, int argc, const char **argv, Params &P)
{
    P = Params();
    P.caseFolder = folder_in;
    // first pass of the command line (io.cu:207-227)
    for (int i = 0; i < argc; ++i) {
        if (!argv[i]) continue;
        if (!strcmp(argv[i], "-caseFolder") && i + 1 < argc) P.caseFolder = argv[++i];
        else if (!strcmp(argv[i], "-deviceNumber") && i + 1 < argc) {
            if (!cli_value(argv[++i], P.deviceNumber)) return "bad -deviceNumber";
        }
    }
    std::string err;
    const std::string &f = P.caseFolder;
    auto sim = parse_yaml_file(f + "/simParams.yaml", err);
    if (!sim) return err;
    if (!(err = parse_simulation(sim.get(), P)).empty()) return err;
    auto flow = parse_yaml_file(f + "/flow.yaml", err);
    if (!flow) return err;
    if (!(err = parse_flow_file(flow.get(), P)).empty()) return err;
    auto dom = parse_yaml_file(f + "/domain.yaml", err);
    if (!dom) return err;
    if (!(err = parse_domain(dom.get(), P)).empty()) return err;
    auto bod = parse_yaml_file(f + "/bodies.yaml", err);
    if (!bod) return err;
    if (!(err = parse_bodies(bod.get(), P, f)).empty()) return err;
    // second pass: overrides (io.cu:234-299)
    for (int i = 0; i + 1 < argc; ++i) {
        const char *a = argv[i];
        if (!a) continue;
        bool ok = true;
        if (!strcmp(a, "-nu")) ok = cli_value(argv[++i], P.nu);
        else if (!strcmp(a, "-uPerturb")) ok = cli_value(argv[++i], P.uPerturb);
        else if (!strcmp(a, "-vPerturb")) ok = cli_value(argv[++i], P.vPerturb);
        else if (!strcmp(a, "-scaleCV")) ok = cli_value(argv[++i], P.scaleCV);
        else if (!strcmp(a, "-nsave")) ok = cli_value(argv[++i], P.nsave);
        else if (!strcmp(a, "-nt")) ok = cli_value(argv[++i], P.nt);
        else if (!strcmp(a, "-dt")) ok = cli_value(argv[++i], P.dt);
        else if (!strcmp(a, "-velocityTol")) ok = cli_value(argv[++i], P.velocity.tolerance);
        else if (!strcmp(a, "-poissonTol")) ok = cli_value(argv[++i], P.poisson.tolerance);
        // extensions of the reference's flags: the persistent solves' grid (batched instances share the GPU)
        else if (!strcmp(a, "-solverBlocks")) ok = cli_value(argv[++i], P.solverBlocks) && P.solverBlocks >= 0;
        else if (!strcmp(a, "-solverPack"))
            ok = cli_value(argv[++i], P.solverPack) && (P.solverPack == 1 || P.solverPack == 2);
        else if (!strcmp(a, "-saStructured"))
            ok = cli_value(argv[++i], P.saStructured) && P.saStructured >= -1 && P.saStructured <= 1;
        else if (!strcmp(a, "-solverThreads"))
            ok = cli_value(argv[++i], P.solverThreads) && P.solverThreads >= 0 && P.solverThreads <= 512 &&
                 P.solverThreads % 32 == 0;
        if (!ok) return std::string("bad value for ") + a;
    }
    if (!(P.dt > 0) || P.nt < 0 || P.nsave <= 0) return "dt must be > 0, nt >= 0 and nsave > 0";
    return "";
}

}  // namespace cuibm
