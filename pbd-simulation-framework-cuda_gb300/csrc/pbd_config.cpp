// pbd_config.cpp -- config.txt reader/writer, defaults and range checks.
//
// Replaces, for the keys the step reads, the reference's configuration stack:
//   Config::getInstance(file) / getValue<T>("A.B.C")          src/parser/Config.h:21-32
//   ConfigParser<IncludeParser<DefineParser<CommentParser>>>  src/parser/Config.h:124
//     grammar: `Name:` opens a scope, `{ }`, `key = value;`, `[a, b]`, "strings"
//                                                             src/parser/ConfigParser.h:265-330
//     comments // and /* */                                   src/parser/CommentParser.h:24-55
//     #define NAME text / #undef NAME, replaced on word bounds src/parser/DefineParser.h:105-143
//     #include "file" (relative to the including file)        src/parser/IncludeParser.h:206-236
//     predefined true -> 1, false -> 0                        src/parser/Config.h:107-108
//   write-back (sorted keys, two-space indent)                src/parser/ConfigObject.h:70-100
//   per-key setters and their accepted ranges                 kernel/Communication.h:440-624
// Values are read the way `istream >> T` reads them (leading numeric text; "0.0f" -> 0.0).
// Keys that a file does not mention keep the value already in the pbd_params (the
// reference throws on a missing key; here the defaults of config.txt stand in).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/pbd.h"
#include "pbd_internal.h"

namespace {

using Defs = std::map<std::string, std::string>;

bool is_word_char(char c) { return std::isalnum((unsigned char)c) || c == '_'; }

// Replace `name` by `text` where it is not part of a longer word (DefineParser.h:147-169;
// its character class "A-Za-z0-9_ \n" is built with `istream >> char`, which skips the
// blanks, so only [A-Za-z0-9_] neighbours block a replacement).
std::string replace_define(const std::string& s, const std::string& name, const std::string& text) {
    if (name.empty()) return s;
    std::string out;
    size_t i = 0;
    while (i < s.size()) {
        size_t k = s.find(name, i);
        if (k == std::string::npos) { out.append(s, i, std::string::npos); break; }
        bool left_ok = k == 0 || !is_word_char(s[k - 1]);
        size_t e = k + name.size();
        bool right_ok = e >= s.size() || !is_word_char(s[e]);
        out.append(s, i, k - i);
        if (left_ok && right_ok) out += text; else out.append(s, k, name.size());
        i = e;
    }
    return out;
}

struct Parser {
    std::map<std::string, std::string> values;   // dotted path -> raw value text
    Defs defines{{"true", "1"}, {"false", "0"}};
    std::set<std::string> included;
    bool in_comment = false;
    bool in_string = false, in_array = false;
    std::string line;                               // pending characters (ConfigParser::line_)
    std::vector<std::string> scopes;                // open scope names
    std::vector<std::string> pending;               // scopes declared by `Name:` but not opened
    std::string error;

    std::string path_of(const std::string& key) const {
        std::string p;
        for (auto& s : scopes) { p += s; p += '.'; }
        return p + key;
    }

    std::string strip_comments(const std::string& raw) {
        std::string out;
        for (size_t i = 0; i < raw.size(); ++i) {
            char a = raw[i], b = i + 1 < raw.size() ? raw[i + 1] : '\0';
            if (a == '*' && b == '/') { ++i; in_comment = false; continue; }
            if (in_comment) continue;
            if (a == '/' && b == '*') { ++i; in_comment = true; continue; }
            if (a == '/' && b == '/') break;
            out += a;
        }
        return out;
    }

    // DefineParser + IncludeParser: returns the tokens re-joined by single spaces, or
    // handles a directive.
    bool directives(const std::string& in, const std::string& dir, std::string& out) {
        std::string s = in;
        for (auto& d : defines) s = replace_define(s, d.first, d.second);
        std::istringstream is(s);
        std::string tok;
        std::vector<std::string> toks;
        while (is >> tok) {
            if (tok == "#define") {
                std::string name, rest;
                is >> name >> std::ws;
                std::getline(is, rest);
                defines[name] = rest;
                out.clear();
                return true;
            }
            if (tok == "#undef") {
                std::string name;
                is >> name;
                defines.erase(name);
                out.clear();
                return true;
            }
            if (tok == "#include") {
                std::string f;
                is >> f;
                if (f.size() >= 2) f = f.substr(1, f.size() - 2);
                std::string full = dir + f;
                if (!included.count(full)) {
                    included.insert(full);
                    if (!parse_file(full)) return false;
                }
                out.clear();
                return true;
            }
            toks.push_back(tok);
        }
        out.clear();
        for (size_t k = 0; k < toks.size(); ++k) { if (k) out += ' '; out += toks[k]; }
        return true;
    }

    // ConfigParser::actualLineParsing (ConfigParser.h:265-330).
    bool config_line(const std::string& s) {
        for (char c : s) {
            if (c == '"') { in_string = !in_string; line += c; }
            else if (in_string) line += c;
            else if (c == ':') { pending.push_back(line); line.clear(); }
            else if (c == '[') { in_array = true; line += c; }
            else if (c == ']') { in_array = false; line += c; }
            else if (in_array) line += c;
            else if (c == '{') {
                if (!pending.empty()) { scopes.push_back(pending.back()); pending.pop_back(); }
                line.clear();
            } else if (c == '}') {
                if (scopes.empty()) { error = "unbalanced '}'"; return false; }
                scopes.pop_back();
                line.clear();
            } else if (c == ';') {
                size_t eq = line.find('=');
                std::string var = eq == std::string::npos ? line : line.substr(0, eq);
                std::string val = eq == std::string::npos ? "" : line.substr(eq + 1);
                if (!var.empty() && !val.empty()) values[path_of(var)] = val;
                else if (!var.empty()) { error = "uninitialized value for '" + var + "'"; return false; }
                else if (!val.empty()) { error = "invalid statement '" + line + "'"; return false; }
                line.clear();
            } else if (c == ' ' || c == '\t' || c == '\r') {
            } else line += c;
        }
        if (in_string) line += '\n';
        return true;
    }

    bool parse_text(const std::string& text, const std::string& dir) {
        std::istringstream is(text);
        std::string raw;
        while (std::getline(is, raw)) {
            std::string a = strip_comments(raw), b;
            if (!directives(a, dir, b)) return false;
            if (!config_line(b)) return false;
        }
        return true;
    }

    bool parse_file(const std::string& path) {
        std::ifstream f(path);
        if (!f) { error = "cannot open config file '" + path + "'"; return false; }
        std::stringstream ss;
        ss << f.rdbuf();
        size_t slash = path.find_last_of('/');
        std::string dir = slash == std::string::npos ? std::string() : path.substr(0, slash + 1);
        return parse_text(ss.str(), dir);
    }
};

std::string clean(std::string v) {   // ConfigParser.h:47-49
    std::string o;
    for (char c : v) if (c != '"' && c != '[' && c != ']') o += c;
    return o;
}

template <class T>
bool get(const Parser& P, const char* key, T& out) {
    auto it = P.values.find(std::string("Application.") + key);
    if (it == P.values.end()) return false;
    std::istringstream is(clean(it->second));
    T v{};
    if (!(is >> v)) return false;
    out = v;
    return true;
}

bool get_flag(const Parser& P, const char* key, uint32_t& mask, uint32_t bit) {
    int v = 0;
    if (!get(P, key, v)) return false;
    mask = v ? (mask | bit) : (mask & ~bit);
    return true;
}

struct Key {
    const char* path;
    char kind;           // f float, u uint32, i int32
    size_t off;
};

#define OFF(field) offsetof(pbd_params, field)
const Key kKeys[] = {
    {"Cuda.threadsPerBlock", 'u', OFF(threads_per_block)},
    {"Simulation.Particles.particleRadius", 'f', OFF(particle_radius)},
    {"Simulation.Particles.maxNeighboursPerParticle", 'u', OFF(max_neighbours_per_particle)},
    {"Simulation.Forces.deltaT", 'f', OFF(delta_t)},
    {"Simulation.Forces.gravity", 'f', OFF(gravity)},
    {"Simulation.Density.restDensity", 'f', OFF(rest_density)},
    {"Simulation.Density.kernelWidthSpiky", 'f', OFF(kernel_width_spiky)},
    {"Simulation.Density.kSCorr", 'f', OFF(k_scorr)},
    {"Simulation.Density.nSCorr", 'i', OFF(n_scorr)},
    {"Simulation.Density.qSCorr", 'f', OFF(q_scorr)},
    {"Simulation.Viscosity.cViscosity", 'f', OFF(c_viscosity)},
    {"Simulation.Viscosity.kernelWidthPoly", 'f', OFF(kernel_width_poly)},
    {"Simulation.Vorticity.eVorticity", 'f', OFF(e_vorticity)},
    {"Simulation.Collision.collisionType", 'u', OFF(collision_type)},
    {"Simulation.Collision.kernelWidthNeighbours", 'u', OFF(kernel_width_neighbours)},
    {"Simulation.Collision.maxCollisionBatches", 'u', OFF(max_collision_batches)},
    {"Simulation.Collision.stiffness", 'f', OFF(stiffness)},
    {"Simulation.Enclosure.enclosurePositionDamping", 'f', OFF(enclosure_position_damping)},
    {"Simulation.Enclosure.enclosureVelocityDamping", 'f', OFF(enclosure_velocity_damping)},
    {"Simulation.Enclosure.X.min", 'f', OFF(bounds_min[0])},
    {"Simulation.Enclosure.Y.min", 'f', OFF(bounds_min[1])},
    {"Simulation.Enclosure.Z.min", 'f', OFF(bounds_min[2])},
    {"Simulation.Enclosure.X.max", 'f', OFF(bounds_max[0])},
    {"Simulation.Enclosure.Y.max", 'f', OFF(bounds_max[1])},
    {"Simulation.Enclosure.Z.max", 'f', OFF(bounds_max[2])},
    {"Simulation.Iterations.solverIterations", 'u', OFF(solver_iterations)},
    {"Simulation.Iterations.stabilizationIterations", 'u', OFF(stabilization_iterations)},
};
#undef OFF

struct ActiveKey { const char* name; uint32_t bit; };
const ActiveKey kActive[] = {
    {"applyForces", PBD_ACTIVE_APPLY_FORCES},
    {"findContacts", PBD_ACTIVE_FIND_CONTACTS},
    {"findNeighbours", PBD_ACTIVE_FIND_NEIGHBOURS},
    {"computeLambda", PBD_ACTIVE_COMPUTE_LAMBDA},
    {"computeDeltaPositions", PBD_ACTIVE_COMPUTE_DELTA_POSITIONS},
    {"applyDeltaPositions", PBD_ACTIVE_APPLY_DELTA_POSITIONS},
    {"updatePositions", PBD_ACTIVE_UPDATE_POSITIONS},
    {"computeOmegas", PBD_ACTIVE_COMPUTE_OMEGAS},
    {"computeVorticity", PBD_ACTIVE_COMPUTE_VORTICITY},
    {"computeViscosity", PBD_ACTIVE_COMPUTE_VISCOSITY},
};

int apply_values(const Parser& P, pbd_params* p) {
    char* base = reinterpret_cast<char*>(p);
    for (const Key& k : kKeys) {
        switch (k.kind) {
            case 'f': get(P, k.path, *reinterpret_cast<float*>(base + k.off)); break;
            case 'u': {
                long long v;
                if (get(P, k.path, v)) *reinterpret_cast<uint32_t*>(base + k.off) = (uint32_t)v;
                break;
            }
            case 'i': get(P, k.path, *reinterpret_cast<int32_t*>(base + k.off)); break;
        }
    }
    for (const ActiveKey& a : kActive) {
        std::string key = std::string("Simulation.Active.") + a.name;
        get_flag(P, key.c_str(), p->active, a.bit);
    }
    return PBD_OK;
}

int range_error(const char* what) {
    pbd::set_error(std::string("parameter out of range: ") + what);
    return PBD_ERR_RANGE;
}

}  // namespace

extern "C" int pbd_params_default(pbd_params* p) {
    if (!p) { pbd::set_error("pbd_params_default: null"); return PBD_ERR_INVALID_ARG; }
    std::memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(pbd_params);
    p->threads_per_block = 512;              // config.txt:11
    p->particle_radius = 0.5f;               // config.txt:113
    p->max_neighbours_per_particle = 512;    // config.txt:112
    p->delta_t = 0.01f;                      // config.txt:96
    p->gravity = -29.82f;                    // config.txt:97
    p->rest_density = 1200.0f;               // config.txt:72
    p->kernel_width_spiky = 6.1f;            // config.txt:69
    p->k_scorr = 0.2f;                       // config.txt:68
    p->n_scorr = 4;                          // config.txt:70
    p->q_scorr = 0.2f;                       // config.txt:71
    p->c_viscosity = 0.0001f;                // config.txt:126
    p->kernel_width_poly = 4.1f;             // config.txt:127
    p->e_vorticity = 1.0f;                   // config.txt:132
    p->collision_type = 0;                   // config.txt:57
    p->kernel_width_neighbours = 2;          // config.txt:58
    p->max_collision_batches = 16;           // config.txt:59
    p->stiffness = 0.3f;                     // config.txt:60
    p->enclosure_position_damping = 0.0f;    // config.txt:77
    p->enclosure_velocity_damping = 1.0f;    // config.txt:78
    for (int a = 0; a < 3; ++a) { p->bounds_min[a] = 1.5f; p->bounds_max[a] = 62.5f; }   // config.txt:80-93
    p->solver_iterations = 1;                // config.txt:102
    p->stabilization_iterations = 1;         // config.txt:103
    p->active = PBD_ACTIVE_ALL;              // config.txt:40-52
    p->max_grid = 128u * 128u * 128u;        // Particles.cc:8
    p->lambda_epsilon = 0.0001f;             // Density.h:90
    p->flags = PBD_FLAG_CELL_END_QUIRK;
    return PBD_OK;
}

extern "C" int pbd_parse_config(pbd_params* p, const char* text, const char* base_dir) {
    if (!p || !text) { pbd::set_error("pbd_parse_config: null"); return PBD_ERR_INVALID_ARG; }
    Parser P;
    std::string dir = base_dir ? std::string(base_dir) : std::string();
    if (!dir.empty() && dir.back() != '/') dir += '/';
    if (!P.parse_text(text, dir)) { pbd::set_error("config: " + P.error); return PBD_ERR_CONFIG; }
    if (!P.scopes.empty()) { pbd::set_error("config: unclosed scope '" + P.scopes.back() + "'"); return PBD_ERR_CONFIG; }
    return apply_values(P, p);
}

extern "C" int pbd_load_config(pbd_params* p, const char* path) {
    if (!p || !path) { pbd::set_error("pbd_load_config: null"); return PBD_ERR_INVALID_ARG; }
    Parser P;
    P.included.insert(path);
    if (!P.parse_file(path)) { pbd::set_error("config: " + P.error); return PBD_ERR_CONFIG; }
    if (!P.scopes.empty()) { pbd::set_error("config: unclosed scope '" + P.scopes.back() + "'"); return PBD_ERR_CONFIG; }
    return apply_values(P, p);
}

// ConfigObject::write layout: in each scope the values sorted by name, then the child
// scopes sorted by name as "Name:\n{\n  ...\n}" (ConfigObject.h:70-100).
namespace {
struct Node {
    std::map<std::string, std::string> vals;
    std::map<std::string, Node> kids;
};
void write_node(const Node& n, std::ostringstream& os, const std::string& ind) {
    for (auto& kv : n.vals) os << ind << kv.first << " = " << kv.second << ";\n";
    if (!n.vals.empty() && !n.kids.empty()) os << "\n";
    size_t k = 0;
    for (auto& c : n.kids) {
        os << ind << c.first << ":\n" << ind << "{\n";
        write_node(c.second, os, ind + "  ");
        os << ind << "}\n";
        if (++k != n.kids.size()) os << "\n";
    }
}
std::string fmt(float v) {
    std::ostringstream o;
    o << v;
    return o.str();
}
}  // namespace

extern "C" int pbd_write_config(const pbd_params* p, const char* path) {
    if (!p || !path) { pbd::set_error("pbd_write_config: null"); return PBD_ERR_INVALID_ARG; }
    Node root;
    const char* base = reinterpret_cast<const char*>(p);
    for (const Key& k : kKeys) {
        std::string full = std::string("Application.") + k.path;
        Node* n = &root;
        size_t s = 0, d;
        while ((d = full.find('.', s)) != std::string::npos) { n = &n->kids[full.substr(s, d - s)]; s = d + 1; }
        std::string v;
        if (k.kind == 'f') v = fmt(*reinterpret_cast<const float*>(base + k.off));
        else if (k.kind == 'u') v = std::to_string(*reinterpret_cast<const uint32_t*>(base + k.off));
        else v = std::to_string(*reinterpret_cast<const int32_t*>(base + k.off));
        n->vals[full.substr(s)] = v;
    }
    Node& act = root.kids["Application"].kids["Simulation"].kids["Active"];
    for (const ActiveKey& a : kActive) act.vals[a.name] = (p->active & a.bit) ? "1" : "0";
    std::ostringstream os;
    write_node(root, os, "");
    std::ofstream f(path);
    if (!f) { pbd::set_error(std::string("cannot write '") + path + "'"); return PBD_ERR_CONFIG; }
    f << os.str() << "\n";
    return PBD_OK;
}

extern "C" int pbd_validate_params(const pbd_params* p) {
    if (!p) { pbd::set_error("pbd_validate_params: null"); return PBD_ERR_INVALID_ARG; }
    if (p->struct_size != sizeof(pbd_params)) { pbd::set_error("pbd_params.struct_size mismatch"); return PBD_ERR_INVALID_ARG; }
    // Communication.h:440-624
    if (!(p->gravity >= -1000.0f && p->gravity <= 1000.0f)) return range_error("gravity [-1000, 1000]");
    if (!(p->kernel_width_neighbours >= 1 && p->kernel_width_neighbours <= 50)) return range_error("kernelWidthNeighbours [1, 50]");
    if (!(p->c_viscosity >= 0.0f && p->c_viscosity <= 100.0f)) return range_error("cViscosity [0, 100]");
    if (!(p->e_vorticity >= -10000.0f && p->e_vorticity <= 10000.0f)) return range_error("eVorticity [-10000, 10000]");
    if (!(p->rest_density > 0.0f && p->rest_density <= 100000.0f)) return range_error("restDensity ]0, 100000]");
    if (!(p->kernel_width_spiky > 0.0f && p->kernel_width_spiky <= 1000.0f)) return range_error("kernelWidthSpiky ]0, 1000]");
    if (!(p->kernel_width_poly > 0.0f && p->kernel_width_poly <= 1000.0f)) return range_error("kernelWidthPoly ]0, 1000]");
    if (!(p->solver_iterations <= 100)) return range_error("solverIterations [0, 100]");
    if (!(p->stabilization_iterations <= 100)) return range_error("stabilizationIterations [0, 100]");
    if (!(p->delta_t > 0.0f && p->delta_t <= 10.0f)) return range_error("deltaT ]0, 10]");
    if (!(p->collision_type == 0 || p->collision_type == 1)) return range_error("collisionType {0, 1}");
    if (!(p->max_collision_batches >= 1 && p->max_collision_batches <= 512)) return range_error("maxCollisionBatches [1, 512]");
    if (!(p->stiffness >= 0.0f && p->stiffness <= 1.0f)) return range_error("stiffness [0, 1]");
    if (!(p->k_scorr >= -100.0f && p->k_scorr <= 100.0f)) return range_error("kSCorr [-100, 100]");
    if (!(p->n_scorr >= -100 && p->n_scorr <= 100)) return range_error("nSCorr [-100, 100]");
    if (!(p->q_scorr >= -100.0f && p->q_scorr <= 100.0f)) return range_error("qSCorr [-100, 100]");
    for (int a = 0; a < 3; ++a)
        if (!(p->bounds_min[a] < p->bounds_max[a] && p->bounds_min[a] >= 1.5f && p->bounds_max[a] <= 126.5f))
            return range_error("enclosure: min < max, each in [1.5, 126.5]");
    if (!(p->enclosure_position_damping >= 0.0f && p->enclosure_position_damping <= 1.0f)) return range_error("enclosurePositionDamping [0, 1]");
    if (!(p->enclosure_velocity_damping >= 0.0f && p->enclosure_velocity_damping <= 1.0f)) return range_error("enclosureVelocityDamping [0, 1]");
    // not setter-checked in the reference, but the tables and the list need them
    if (!(p->particle_radius > 0.0f && std::isfinite(p->particle_radius))) return range_error("particleRadius > 0");
    if (p->max_grid == 0 || p->max_grid > (1u << 30)) return range_error("max_grid in [1, 2^30]");
    if (!(p->lambda_epsilon >= 0.0f && std::isfinite(p->lambda_epsilon))) return range_error("lambda_epsilon >= 0");
    if (p->active & ~PBD_ACTIVE_ALL) return range_error("active: unknown bits");
    return PBD_OK;
}
