/*
 * Host driver over libpicgb: parameters.h reader, dataDump/timeData text
 * files and the pic class (see pic_host.h).
 */
#include "pic_host.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include "pgb_rng.h"

namespace picgb {

/* ------------------------------------------------------------ macros */
namespace {
/* constants.h:15-37 */
const char* kConstants[][2] = {
    {"UPPER_LIMIT", "(int)10000"},
    {"PI", "(double)3.141592654"},
    {"ELECTRON_CHARGE", "-(double)1.602177e-19"},
    {"ELECTRON_CHARGE2", "(double)2.566971e-38"},
    {"CHARGE", "(double)1.602177e-19"},
    {"ELECTRON_MASS", "(double)9.10939e-31"},
    {"AMU", "(double)1.66054e-27"},
    {"K", "(double)1.38066e-23"},
    {"EPSILON", "(double)8.854e-12"},
    {"PERMEABILITY_FREE_SPACE", "4.0*PI*1.0e-7"},
    {"SEED", "1"}, {"TRUE", "1"}, {"FALSE", "0"}, {"IS_ELECTRON", "1"}, {"IS_ION", "0"},
    {"YES", "1"}, {"NO", "0"},
};

std::string strip_comments(const std::string& s) {
    std::string out;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] == '"') {   /* keep string literals intact */
            size_t j = s.find('"', i + 1);
            if (j == std::string::npos) j = s.size() - 1;
            out += s.substr(i, j - i + 1);
            i = j;
        } else if (s.compare(i, 2, "//") == 0) {
            break;
        } else if (s.compare(i, 2, "/*") == 0) {
            size_t j = s.find("*/", i + 2);
            if (j == std::string::npos) break;
            i = j + 1;
            out += ' ';
        } else {
            out += s[i];
        }
    }
    while (!out.empty() && std::isspace((unsigned char)out.back())) out.pop_back();
    size_t k = 0;
    while (k < out.size() && std::isspace((unsigned char)out[k])) ++k;
    return out.substr(k);
}

struct Val {
    double v = 0.0;
    bool is_int = false;
    bool is_str = false;
    std::string s;
};
}  // namespace

/* recursive-descent evaluation of a macro body with C arithmetic rules:
 * integer operands give integer results (division truncates)            */
struct ExprParser {
    const MacroTable& m;
    std::string src;
    size_t pos = 0;
    int depth;
    ExprParser(const MacroTable& mt, const std::string& s, int d) : m(mt), src(s), depth(d) {}

    void ws() { while (pos < src.size() && std::isspace((unsigned char)src[pos])) ++pos; }
    bool eat(char c) {
        ws();
        if (pos < src.size() && src[pos] == c) { ++pos; return true; }
        return false;
    }
    std::string ident() {
        ws();
        size_t b = pos;
        while (pos < src.size() && (std::isalnum((unsigned char)src[pos]) || src[pos] == '_')) ++pos;
        return src.substr(b, pos - b);
    }
    [[noreturn]] void bad(const std::string& why) { throw std::runtime_error("parameters.h: " + why + " in '" + src + "'"); }

    Val expr() {
        Val a = term();
        for (;;) {
            if (eat('+')) a = arith(a, term(), '+');
            else if (eat('-')) a = arith(a, term(), '-');
            else return a;
        }
    }
    Val term() {
        Val a = unary();
        for (;;) {
            if (eat('*')) a = arith(a, unary(), '*');
            else if (eat('/')) a = arith(a, unary(), '/');
            else return a;
        }
    }
    static Val arith(const Val& a, const Val& b, char op) {
        Val r;
        if (a.is_int && b.is_int) {
            long long x = (long long)a.v, y = (long long)b.v, z = 0;
            switch (op) {
                case '+': z = x + y; break;
                case '-': z = x - y; break;
                case '*': z = x * y; break;
                default: z = y ? x / y : 0; break;
            }
            r.v = (double)z;
            r.is_int = true;
        } else {
            switch (op) {
                case '+': r.v = a.v + b.v; break;
                case '-': r.v = a.v - b.v; break;
                case '*': r.v = a.v * b.v; break;
                default: r.v = a.v / b.v; break;
            }
        }
        return r;
    }
    Val unary() {
        ws();
        if (eat('-')) { Val v = unary(); v.v = -v.v; return v; }
        if (eat('+')) return unary();
        /* cast? */
        size_t save = pos;
        if (eat('(')) {
            ws();
            size_t b = pos;
            std::string t = ident();
            ws();
            while (pos < src.size() && src[pos] == '*') { ++pos; ws(); }
            if ((t == "double" || t == "int" || t == "float" || t == "char" || t == "cl_double" || t == "long") && eat(')')) {
                Val v = unary();
                if (t == "int" || t == "long") { v.v = std::trunc(v.v); v.is_int = true; }
                else if (t == "double" || t == "float" || t == "cl_double") {
                    v.is_int = false;
                    if (t == "float") v.v = (double)(float)v.v;
                }
                return v;
            }
            pos = b;
            (void)save;
            Val v = expr();
            if (!eat(')')) bad("missing )");
            return v;
        }
        return primary();
    }
    Val primary() {
        ws();
        if (pos >= src.size()) bad("unexpected end");
        char c = src[pos];
        if (c == '"') {
            size_t j = src.find('"', pos + 1);
            if (j == std::string::npos) bad("unterminated string");
            Val v;
            v.is_str = true;
            v.s = src.substr(pos + 1, j - pos - 1);
            pos = j + 1;
            return v;
        }
        if (std::isdigit((unsigned char)c) || c == '.') {
            const char* b = src.c_str() + pos;
            char* e = nullptr;
            double d = std::strtod(b, &e);
            std::string lit(b, (size_t)(e - b));
            pos += (size_t)(e - b);
            Val v;
            v.v = d;
            v.is_int = lit.find_first_of(".eE") == std::string::npos;
            return v;
        }
        std::string id = ident();
        if (id.empty()) bad(std::string("unexpected '") + c + "'");
        if (eat('(')) {
            std::vector<Val> args;
            if (!eat(')')) {
                do { args.push_back(expr()); } while (eat(','));
                if (!eat(')')) bad("missing ) after arguments");
            }
            Val v;
            if (id == "sqrt" && args.size() == 1) v.v = std::sqrt(args[0].v);
            else if (id == "cos" && args.size() == 1) v.v = std::cos(args[0].v);
            else if (id == "sin" && args.size() == 1) v.v = std::sin(args[0].v);
            else if ((id == "abs" || id == "fabs") && args.size() == 1) { v = args[0]; v.v = std::fabs(v.v); }
            else if (id == "time") { v.v = 0.0; v.is_int = true; }   /* RAND_SEED time(NULL): the caller seeds */
            else bad("unknown function " + id);
            return v;
        }
        if (id == "true") { Val v; v.v = 1; v.is_int = true; return v; }
        if (id == "false") { Val v; v.v = 0; v.is_int = true; return v; }
        if (id == "NULL") { Val v; v.v = 0; v.is_int = true; return v; }
        if (!m.has(id)) bad("unknown macro " + id);
        if (depth > 64) bad("macro recursion");
        auto it = m.body_.find(id);
        ExprParser sub(m, it->second, depth + 1);
        Val v = sub.expr();
        return v;
    }
};

void MacroTable::define(const std::string& name, const std::string& body) {
    body_[name] = body;
    cache_.clear();
}
bool MacroTable::has(const std::string& name) const {
    if (body_.count(name)) return true;
    for (auto& c : kConstants) if (name == c[0]) return true;
    return false;
}
double MacroTable::number(const std::string& name) const {
    auto c = cache_.find(name);
    if (c != cache_.end()) return c->second;
    if (!has(name)) throw std::runtime_error("parameters.h: " + name + " is not defined");
    ExprParser p(*this, name, 0);
    Val v = p.primary();
    if (v.is_str) throw std::runtime_error("parameters.h: " + name + " is a string");
    cache_[name] = v.v;
    return v.v;
}
std::string MacroTable::text(const std::string& name) const {
    ExprParser p(*this, name, 0);
    Val v = p.primary();
    if (!v.is_str) throw std::runtime_error("parameters.h: " + name + " is not a string");
    return v.s;
}
bool MacroTable::flag(const std::string& name) const {
    ExprParser p(*this, name, 0);
    Val v = p.primary();
    if (v.is_str) return v.s == "YES";
    return v.v != 0.0;
}

MacroTable read_parameters_h(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open " + path);
    MacroTable m;
    for (auto& c : kConstants) m.define(c[0], c[1]);
    std::string line;
    bool in_block = false;
    while (std::getline(in, line)) {
        if (in_block) {
            size_t e = line.find("*/");
            if (e == std::string::npos) continue;
            line = line.substr(e + 2);
            in_block = false;
        }
        size_t b = line.find("/*");
        if (b != std::string::npos && line.find("*/", b) == std::string::npos &&
            line.find('"') == std::string::npos) {
            line = line.substr(0, b);
            in_block = true;
        }
        size_t k = line.find_first_not_of(" \t");
        if (k == std::string::npos || line.compare(k, 7, "#define") != 0) continue;
        std::istringstream ss(line.substr(k + 7));
        std::string name;
        ss >> name;
        if (name.empty() || name.find('(') != std::string::npos) continue;
        std::string rest;
        std::getline(ss, rest);
        rest = strip_comments(rest);
        if (rest.empty()) continue;   /* include guards */
        m.define(name, rest);
    }
    return m;
}

pgb_params params_from_macros(const MacroTable& m, uint64_t seed) {
    pgb_params p;
    pgb_params_default(&p);
    auto num = [&](const char* n) { return m.number(n); };
    p.x_no_of_cells = (int32_t)num("X_NO_OF_CELLS");
    p.y_no_of_cells = (int32_t)num("Y_NO_OF_CELLS");
    p.xlength = num("XLENGTH");
    p.ylength = num("YLENGTH");
    p.dt = num("DT");
    p.dti = num("DTI");
    p.electron_mass = num("ELECTRON_MASS");
    p.ion_mass = num("ION_MASS");
    p.q_over_me = num("Q_OVER_ME");
    p.q_over_mi = num("Q_OVER_MI");
    p.qce = num("QCE");
    p.qci = num("QCI");
    p.vte = num("VTE");
    p.vti = num("VTI");
    p.vtn = num("VTN");
    p.magnetic_field = num("MAGNETIC_FIELD");
    p.angle = num("ANGLE");
    p.phi_left = num("PHI_LEFT");
    p.phi_right = num("PHI_RIGHT");
    p.phi_bottom = num("PHI_BOTTOM");
    p.phi_top = num("PHI_TOP");
    p.phi_period = num("PHI_PERIOD");
    p.neutral_density = num("NEUTRAL_DENSITY");
    p.threshold = num("THRESHOLD");
    p.work_function = num("WORK_FUNCTION");
    p.have_collisions = m.flag("HAVE_COLLISIONS") ? 1 : 0;
    p.species = m.text("SPECIES") == "ARGON" ? PGB_ARGON : PGB_HYDROGEN;
    auto mode = [&](const char* n) { return m.text(n) == "CONSTANT" ? PGB_SIGMA_CONSTANT : PGB_SIGMA_ENERGY_DEPENDENT; };
    p.sigma_cx_mode = mode("SIGMA");
    p.sigma_elastic_mode = mode("SIGMA_ELASTIC");
    p.sigma_ionization_mode = mode("SIGMA_IONIZATION");
    p.sigma_value = num("SIGMA_VALUE");
    p.elastic_sigma_value = num("ELASTIC_SIGMA_VALUE");
    p.ionization_sigma_value = num("IONIZATION_SIGMA_VALUE");
    p.e_impact_see = m.flag("E_IMPACT_SEE");
    p.ion_impact_see = m.flag("ION_IMPACT_SEE");
    p.reflection = m.flag("REFLECTION");
    p.backscatter = m.flag("BACKSCATTER");
    p.steadystate = m.flag("STEADYSTATE");
    p.number_to_inject = (int32_t)num("NUMBER_TO_INJECT");
    p.init_no_neutrals = (int32_t)num("INIT_NO_NEUTRALS");
    /* pic.cpp:257-327 */
    p.no_groups = (int32_t)num("NO_GROUPS");
    const char* ve[3] = {"VE1", "VE2", "UPPER_V_LIMIT"};
    const char* vi[3] = {"VI1", "VI2", "UPPER_V_LIMIT_I"};
    for (int g = 0; g < 3; ++g) {
        p.v_limit_e[g] = num(ve[g]);
        p.v_limit_i[g] = num(vi[g]);
        p.group_limit_e[g] = (int32_t)num("UPPER_GROUP_LIMIT");
        p.new_group_size_e[g] = (int32_t)num("NEW_GROUP_SIZE");
        p.group_limit_i[g] = (int32_t)num(g == 0 ? "UPPER_GROUP_LIMIT" : "UPPER_GROUP_LIMIT2");
        p.new_group_size_i[g] = (int32_t)num(g == 0 ? "NEW_GROUP_SIZE" : "NEW_GROUP_SIZE2");
    }
    p.size_to_check_e = (int64_t)num("SIZE_TO_CHECK_E");
    p.size_to_check_i = (int64_t)num("SIZE_TO_CHECK");
    p.seed = seed;
    return p;
}

/* ---------------------------------------------------------- text files */
std::vector<double> read_datadump(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) throw Error("cannot open " + path, PGB_ERR_IO);
    std::vector<double> out;
    double r[6];
    /* while (in >> x >> y >> vx >> vy >> vz >> weight) (particle.cpp:385) */
    while (std::fscanf(f, "%lf %lf %lf %lf %lf %lf", &r[0], &r[1], &r[2], &r[3], &r[4], &r[5]) == 6)
        out.insert(out.end(), r, r + 6);
    std::fclose(f);
    return out;
}

/* `ofstream << double` at the default precision: %g with 6 digits */
static void put(std::string& s, double v) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%g", v);
    s += buf;
}

void write_datadump(const std::string& path, const std::vector<double>& a) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) throw Error("cannot write " + path, PGB_ERR_IO);
    std::string line;
    for (size_t i = 0; i + 5 < a.size(); i += 6) {
        line.clear();
        for (int k = 0; k < 6; ++k) {
            if (k) line += ' ';
            put(line, a[i + k]);
        }
        line += '\n';
        std::fwrite(line.data(), 1, line.size(), f);
    }
    std::fclose(f);
}

/* ------------------------------------------------------- binary files */
/* Lossless restart records, an addition to the reference's text format:
 * "PGBDUMP1", an int64 record count, then the records as little-endian
 * doubles {x, y, vx, vy, vz, weight}.  The text format keeps 6 digits;
 * this one keeps the state exactly, so a restart continues the same run. */
static const char kDumpMagic[8] = {'P', 'G', 'B', 'D', 'U', 'M', 'P', '1'};

std::vector<double> read_datadump_bin(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error("cannot open " + path, PGB_ERR_IO);
    char magic[8];
    int64_t n = -1;
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kDumpMagic, 8) != 0 ||
        std::fread(&n, sizeof n, 1, f) != 1 || n < 0 || n > ((int64_t)1 << 40)) {
        std::fclose(f);
        throw Error(path + ": not a binary particle dump", PGB_ERR_IO);
    }
    std::vector<double> out((size_t)n * 6);
    const size_t got = n ? std::fread(out.data(), sizeof(double), out.size(), f) : 0;
    std::fclose(f);
    if (got != out.size()) throw Error(path + ": truncated binary particle dump", PGB_ERR_IO);
    return out;
}

void write_datadump_bin(const std::string& path, const std::vector<double>& a) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error("cannot write " + path, PGB_ERR_IO);
    const int64_t n = (int64_t)(a.size() / 6);
    bool ok = std::fwrite(kDumpMagic, 1, 8, f) == 8 && std::fwrite(&n, sizeof n, 1, f) == 1 &&
              (n == 0 || std::fwrite(a.data(), sizeof(double), (size_t)n * 6, f) == (size_t)n * 6);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) throw Error("cannot write " + path, PGB_ERR_IO);
}

/* --------------------------------------------------------------- Pic */
void Pic::check(int rc, const char* what) {
    if (rc != 0) throw Error(std::string(what) + ": " + pgb_last_error(run_), rc);
}

Pic::Pic(const MacroTable& m, const std::string& dir, bool restart, uint64_t seed, bool binary_dump)
    : dir_(dir), binary_dump_(binary_dump) {
    p_ = params_from_macros(m, seed);
    int rc = pgb_create(&p_, &run_);
    if (rc != 0) throw Error(std::string("pgb_create: ") + pgb_last_error(nullptr), rc);
    time_data_frequency_ = m.has("TIME_DATA_FREQUENCY") ? (int)m.number("TIME_DATA_FREQUENCY") : 100;
    const char* px[3] = {"POINT1X", "POINT2X", "POINT3X"};
    const char* py[3] = {"POINT1Y", "POINT2Y", "POINT3Y"};
    for (int k = 0; k < 3; ++k) {
        point[k][0] = m.has(px[k]) ? (int)m.number(px[k]) : 0;
        point[k][1] = m.has(py[k]) ? (int)m.number(py[k]) : 0;
    }
    /* the graphs of pic::initialize_graph_parameters (pic.cpp:539-577) and
     * the window of pic::pic (pic.h:89): sums over time steps
     * [START_GRAPH_TIME, END_GRAPH_TIME), averaged over NO_GRAPH_STEPS    */
    check(pgb_graphs_params_default(&p_, &graphs_), "pgb_graphs_params_default");
    const struct { const char* name; int32_t* i32; int64_t* i64; } gm[] = {
        {"START_GRAPH_TIME", nullptr, &graphs_.start_step}, {"END_GRAPH_TIME", nullptr, &graphs_.end_step},
        {"NO_GRAPH_STEPS", &graphs_.no_graph_steps, nullptr}, {"NO_BINS", &graphs_.no_bins, nullptr},
        {"DIVIDE_BINS_BY", &graphs_.divide_bins_by, nullptr}, {"SPREAD", &graphs_.spread, nullptr},
        {"DIST_LOCATIONX", &graphs_.dist_location_x, nullptr}, {"DIST_LOCATIONY", &graphs_.dist_location_y, nullptr},
        {"DIST_LOCATION2X", &graphs_.dist_location2_x, nullptr},
        {"DIST_LOCATION2Y", &graphs_.dist_location2_y, nullptr},
    };
    for (auto& g : gm) {
        if (!m.has(g.name)) continue;
        const double v = m.number(g.name);
        if (g.i32) *g.i32 = (int32_t)v;
        else *g.i64 = (int64_t)v;
    }
    if (graphs_.end_step > graphs_.start_step) check(pgb_graphs_enable(run_, &graphs_), "pgb_graphs_enable");
    const char* types[2] = {"e", "i1"};   /* ELECTRON_TYPE, ION_TYPE */
    for (int s = 0; s < 2; ++s) {
        std::vector<double> a;
        if (restart) {
            a = binary_dump_ ? read_datadump_bin(dir_ + "/dataDump_" + types[s] + ".bin")
                             : read_datadump(dir_ + "/dataDump_" + types[s] + ".txt");
        } else {
            /* create_particles + initiate_positions + initiate_velocities
             * (particle.cpp:321-482): a lattice of spacing DXP, repeated
             * while particles remain, weight 1                             */
            long long n = (long long)m.number("INIT_PARTICLE_NO");
            double dxp = m.number(s == 0 ? "DXPE" : "DXPI"), dyp = m.number(s == 0 ? "DYPE" : "DYPI");
            double xl = m.number("XLENGTH"), yl = m.number("YLENGTH");
            double vt = s == 0 ? p_.vte : p_.vti;
            a.assign((size_t)n * 6, 0.0);
            long long i = 0;
            while (i < n) {
                double y = dyp;
                while (y < yl && i < n) {
                    double x = dxp;
                    while (x < xl && i < n) {
                        a[6 * i] = x;
                        a[6 * i + 1] = y;
                        x += dxp;
                        ++i;
                    }
                    y += dyp;
                }
            }
            const double PI = 3.141592654;
            for (long long k = 0; k < n; ++k) {
                pgb_stream st;
                pgb_stream_init(&st, seed, (uint32_t)k, 0xFFFFFFFEu, PGB_STREAM_INJECT, (uint32_t)s);
                for (int c = 0; c < 3; ++c) {
                    double v;
                    do {
                        double R1 = pgb_u01d(pgb_stream_u32(&st)), R2 = pgb_u01d(pgb_stream_u32(&st));
                        v = vt * std::cos(2.0 * PI * R2) * std::sqrt(std::fabs(std::log(R1)));
                    } while (std::fabs(v) > vt * 10000);
                    a[6 * k + 2 + c] = v;
                }
                a[6 * k + 5] = 1.0;
            }
        }
        check(pgb_load_species(run_, s, a.data(), (int64_t)(a.size() / 6)), "pgb_load_species");
    }
}

Pic::~Pic() {
    if (run_) pgb_destroy(run_);
}

pgb_counters Pic::counters() {
    pgb_counters c;
    check(pgb_get_counters(run_, &c), "pgb_get_counters");
    return c;
}

void Pic::pic_run(int run_time, bool verbose) {
    /* pic_run restarts its time_step at 0 and applies both boundaries first
     * (pic.cpp:1049-1069)                                                 */
    check(pgb_set_time_step(run_, 0), "pgb_set_time_step");
    check(pgb_initial_boundary(run_), "pgb_initial_boundary");
    const int nx = p_.x_no_of_cells, ny = p_.y_no_of_cells;
    std::vector<double> phi((size_t)nx * ny), qe((size_t)nx * ny), qi((size_t)nx * ny);
    int t = 0;
    while (t < run_time) {
        int chunk = 1;
        if (!verbose) {
            int next = ((t / time_data_frequency_) + 1) * time_data_frequency_;
            if (t % time_data_frequency_ == 0) next = t + 1;
            /* stop after step END_GRAPH_TIME-1 to write the graph files */
            const int64_t gend = graphs_.end_step;
            if (gend > graphs_.start_step && gend > t && gend < next) next = (int)gend;
            chunk = std::min(run_time, next) - t;
        }
        check(pgb_step(run_, chunk), "pgb_step");
        int last = t + chunk - 1;
        if (last % time_data_frequency_ == 0) {
            pgb_counters c = counters();
            check(pgb_get_grid(run_, PGB_GRID_PHI, phi.data(), (int64_t)phi.size()), "pgb_get_grid");
            check(pgb_get_grid(run_, PGB_GRID_Q_E, qe.data(), (int64_t)qe.size()), "pgb_get_grid");
            check(pgb_get_grid(run_, PGB_GRID_Q_I, qi.data(), (int64_t)qi.size()), "pgb_get_grid");
            Sample s;
            s.t = last; s.ne = c.n_e; s.ni = c.n_i;
            s.phi_l = phi[(size_t)point[0][1] * nx + point[0][0]];
            s.phi_m = phi[(size_t)point[1][1] * nx + point[1][0]];
            s.phi_r = phi[(size_t)point[2][1] * nx + point[2][0]];
            s.eden_r = qe[(size_t)point[2][1] * nx + point[2][0]];
            s.iden_r = qi[(size_t)point[2][1] * nx + point[2][0]];
            samples_.push_back(s);
        }
        /* pic.cpp:1209-1247 */
        if (write_graphs_ && graphs_.end_step > graphs_.start_step && last == graphs_.end_step - 1)
            check(pgb_graphs_write(run_, dir_.c_str()), "pgb_graphs_write");
        if (verbose) {
            pgb_counters c = counters();
            std::printf("time is %d no of electrons= %lld no ions of species1  %lld\n", last, (long long)c.n_e,
                        (long long)c.n_i);
        }
        t += chunk;
    }
}

void Pic::dump_data() {
    const char* types[2] = {"e", "i1"};
    for (int s = 0; s < 2; ++s) {
        int64_t n = 0;
        check(pgb_species_count(run_, s, &n), "pgb_species_count");
        std::vector<double> a((size_t)n * 6);
        int64_t got = 0;
        check(pgb_dump_species(run_, s, a.data(), n, &got), "pgb_dump_species");
        a.resize((size_t)std::min<int64_t>(got, n) * 6);
        write_datadump(dir_ + "/dataDump_" + types[s] + ".txt", a);
        if (binary_dump_) write_datadump_bin(dir_ + "/dataDump_" + types[s] + ".bin", a);
    }
}

void Pic::write_time_data() {
    std::string path = dir_ + "/timeData.txt";
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) throw Error("cannot write " + path, PGB_ERR_IO);
    std::string line;
    for (auto& s : samples_) {
        line = std::to_string(s.t) + " " + std::to_string(s.ne) + " " + std::to_string(s.ni);
        for (double v : {s.phi_l, s.phi_m, s.phi_r, s.eden_r, s.iden_r}) {
            line += ' ';
            put(line, v);
        }
        line += '\n';
        std::fwrite(line.data(), 1, line.size(), f);
    }
    std::fclose(f);
}

}  // namespace picgb

#ifndef PGB_HOST_IN_EXE
/* C ABI: parameters.h -> pgb_params (declared in include/picgb.h) */
extern "C" PGB_API int pgb_params_from_header(const char* path, uint64_t seed, pgb_params* out) {
    if (!path || !out) return PGB_ERR_ARG;
    try {
        picgb::MacroTable m = picgb::read_parameters_h(path);
        *out = picgb::params_from_macros(m, seed);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "pgb_params_from_header: %s\n", e.what());
        return PGB_ERR_IO;
    }
}
#endif
