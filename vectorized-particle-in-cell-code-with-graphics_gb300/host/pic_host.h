/*
 * Host-side driver over libpicgb, mirroring the reference's pic class.
 *
 * The reference configures a run with the macros of parameters.h (compiled
 * in) and drives it with pic::pic (pic.cpp:55-221), pic::pic_run
 * (pic.cpp:1040-1279) and pic::dump_data (pic.cpp:1285-1295).  This driver
 * reads the same parameters.h at run time (read_parameters_h), keeps the same
 * restart and output files (dataDump_e.txt, dataDump_i1.txt, timeData.txt)
 * and calls the C ABI of include/picgb.h in pic_run's order.
 */
#pragma once
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
#include "picgb.h"

namespace picgb {

/* Values of the macros of a parameters.h, evaluated as C expressions
 * (numbers, + - * /, parentheses, casts, sqrt/cos/sin/abs, string and
 * boolean literals, references to other macros).  constants.h is known
 * built in (constants.h:17-37).                                          */
class MacroTable {
public:
    void define(const std::string& name, const std::string& body);
    bool has(const std::string& name) const;
    double number(const std::string& name) const;
    std::string text(const std::string& name) const;   /* string-literal macros */
    bool flag(const std::string& name) const;          /* true/false or YES/NO */
private:
    std::map<std::string, std::string> body_;
    mutable std::map<std::string, double> cache_;
    friend struct ExprParser;
};

/* Parse `#define NAME value` lines of a parameters.h file.  Throws
 * std::runtime_error on an unreadable file.                              */
MacroTable read_parameters_h(const std::string& path);

/* pgb_params from the macros (parameters.h names; pic.cpp:226-529) */
pgb_params params_from_macros(const MacroTable& m, uint64_t seed);

/* particle::load_particles / particle::dump_data text format
 * (particle.cpp:359-401, 1361-1382)                                      */
std::vector<double> read_datadump(const std::string& path);
void write_datadump(const std::string& path, const std::vector<double>& aos6);
/* lossless binary form of the same records (no reference counterpart):
 * "PGBDUMP1", int64 count, little-endian doubles                       */
std::vector<double> read_datadump_bin(const std::string& path);
void write_datadump_bin(const std::string& path, const std::vector<double>& aos6);

class Error : public std::runtime_error {
public:
    Error(const std::string& what, int code) : std::runtime_error(what), code(code) {}
    int code;
};

/* pic::pic / pic_run / dump_data on the GPU */
class Pic {
public:
    /* restart = true loads dataDump_e.txt and dataDump_i1.txt from dir
     * (pic.cpp:110-119); otherwise INIT_PARTICLE_NO particles per species
     * are placed on the lattice of particle::initiate_positions
     * (particle.cpp:410-443) with Maxwellian velocities.  binary_dump
     * restarts from dataDump_*.bin and makes dump_data() write them beside
     * the text files.                                                     */
    Pic(const MacroTable& macros, const std::string& dir, bool restart, uint64_t seed, bool binary_dump = false);
    ~Pic();
    Pic(const Pic&) = delete;
    Pic& operator=(const Pic&) = delete;

    /* run_time steps of pic_run, sampling timeData every
     * TIME_DATA_FREQUENCY steps (pic.cpp:1167-1180); verbose prints the
     * reference's per-step line (pic.cpp:1183-1186)                      */
    void pic_run(int run_time, bool verbose);
    /* pic::setWriteGraphDataToFiles (pic.cpp:980-983): the averaged graph
     * files are written when step END_GRAPH_TIME-1 completes            */
    void set_write_graph_data_to_files(bool on) { write_graphs_ = on; }
    void dump_data();                       /* dataDump_e.txt, dataDump_i1.txt (+ .bin) */
    void write_time_data();                 /* timeData.txt (pic.cpp:1261-1274) */
    pgb_counters counters();
    pgb_run* handle() { return run_; }

private:
    void check(int rc, const char* what);
    pgb_run* run_ = nullptr;
    pgb_params p_;
    std::string dir_;
    int time_data_frequency_ = 100;
    int point[3][2];
    struct Sample { long long t, ne, ni; double phi_l, phi_m, phi_r, eden_r, iden_r; };
    std::vector<Sample> samples_;
    bool first_run_ = true;
    pgb_graphs_params graphs_{};
    bool write_graphs_ = true;
    bool binary_dump_ = false;
};

}  // namespace picgb
