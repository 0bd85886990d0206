/*
 * Driver that runs the reference's own C++ code (built unchanged from its
 * sources by oracle/Makefile) on a prepared state and writes every quantity
 * the parity tests compare.  TEST INFRASTRUCTURE ONLY: its outputs become
 * golden fixtures and pin the C restatement in oracle/picport.c.
 *
 * Modes (argv[1]):
 *   run <dir> <nsteps> [<start_graph> <end_graph>]
 *                        chdir(dir); srand(ORC_SEED); construct the reference
 *                        `pic` with restart=true (it reads dataDump_e.txt and
 *                        dataDump_i1.txt, pic.cpp:110-119) and call pic_run()
 *                        for nsteps (pic.cpp:1040-1279).  Without a window the
 *                        graph window is placed after the run.  With one, the
 *                        graphs sum steps [start, end), average over end-start
 *                        steps (pic::initializeGraphsForInteractive,
 *                        pic.cpp:990-995), and the reference writes its graph
 *                        files into dir at step end-1 (pic.cpp:1209-1247); then write
 *                          e.bin, i1.bin   particles, 6 doubles each (particleVec.h)
 *                          q_e.bin, q_i1.bin  charge after edge doubling (ny*nx)
 *                          rho.bin, phi.bin   (ny*nx, row = y index)
 *                          ex.bin, ey.bin     ((nx+1)*(ny+1), stride nx, fields.cpp:65-76)
 *                        and the reference's own dump (dataDump_*.txt) as
 *                        dump_e.txt / dump_i1.txt.
 *   fields <dir>         read rho.bin (ny*nx doubles) from dir, run
 *                        fields::grid_potential(step 0) and grid_electric_field
 *                        (fields.cpp:169-268, Mglin) and write phi.bin, ex.bin, ey.bin.
 *   sigma <dir>          read energies.bin (doubles, eV) from dir and write
 *                        sigma.bin: per energy the reference's six energy-
 *                        dependent cross-sections (units of 1e-20 m^2), in the
 *                        order e-Ar elastic, e-Ar ionization, e-H elastic, e-H
 *                        ionization, Ar+-Ar charge exchange, H+-H charge
 *                        exchange (e_collisions.cpp:205-308,
 *                        ion_collisions.cpp:170-199).
 *
 * The reference keeps its state in private members; this file alone widens
 * access so that the state can be read without modifying the reference.
 */
#include <chrono>
#include <vector>
#include <algorithm>
#include <new>
#include <string>
#include <complex>
#include <sstream>
#include <iomanip>
#include <limits>
#include <fstream>
#include <iostream>
#include <ctype.h>
#include <fcntl.h>
#include <omp.h>
#include <cstdio>
#include <cstdlib>
#include <climits>
#include <unistd.h>
#include <sys/stat.h>

#define private public
#define protected public
#include "pic.h"
#undef private
#undef protected

static void write_bin(const std::string& path, const void* data, size_t bytes) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(3); }
    if (bytes && std::fwrite(data, 1, bytes, f) != bytes) { std::perror(path.c_str()); std::exit(3); }
    std::fclose(f);
}

static void write_particles(const std::string& path, std::vector<particleVec>& v) {
    std::vector<double> flat(v.size() * 6);
    for (size_t i = 0; i < v.size(); ++i) {
        flat[6 * i + 0] = v[i].x;  flat[6 * i + 1] = v[i].y;
        flat[6 * i + 2] = v[i].vx; flat[6 * i + 3] = v[i].vy;
        flat[6 * i + 4] = v[i].vz; flat[6 * i + 5] = v[i].weight;
    }
    write_bin(path, flat.data(), flat.size() * sizeof(double));
}

static void write_fields(fields& f) {
    const int nx = X_NO_OF_CELLS, ny = Y_NO_OF_CELLS;
    std::vector<double> rho(nx * ny), phi(nx * ny);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            rho[j * nx + i] = f.rho[j][i];
            phi[j * nx + i] = f.phi[j][i];
        }
    write_bin("rho.bin", rho.data(), rho.size() * sizeof(double));
    write_bin("phi.bin", phi.data(), phi.size() * sizeof(double));
    write_bin("ex.bin", f.electric_fieldX, sizeof(double) * (nx + 1) * (ny + 1));
    write_bin("ey.bin", f.electric_fieldY, sizeof(double) * (nx + 1) * (ny + 1));
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s run <dir> <nsteps> | fields <dir> | sigma <dir>\n", argv[0]);
        return 2;
    }
    std::string mode = argv[1];
    if (chdir(argv[2]) != 0) { std::perror(argv[2]); return 2; }
    // The reference opens pic.cl at start-up (pic.cpp:594-606); its text is
    // not used by the in-process runtime, so an empty file satisfies it.
    if (access("pic.cl", F_OK) != 0) { FILE* f = std::fopen("pic.cl", "w"); if (f) std::fclose(f); }

    // The reference prints one line per step; keep it out of the harness output.
    std::streambuf* saved = std::cout.rdbuf();
    std::ofstream devnull("/dev/null");
    std::cout.rdbuf(devnull.rdbuf());

    if (mode == "run") {
        int nsteps = argc > 3 ? std::atoi(argv[3]) : 1;
        const bool window = argc > 5;
        const int start_graph = window ? std::atoi(argv[4]) : INT_MAX - 2;
        const int end_graph = window ? std::atoi(argv[5]) : INT_MAX - 1;
        srand(RAND_SEED);
        pic* p = new pic(true, false, nsteps, start_graph, end_graph);
        if (window) p->initializeGraphsForInteractive(end_graph - start_graph);
        p->pic_run();
        write_particles("e.bin", p->electrons.get_particle());
        write_particles("i1.bin", p->ions[0].get_particle());
        write_bin("q_e.bin", p->electrons.get_q(), sizeof(double) * X_NO_OF_CELLS * Y_NO_OF_CELLS);
        write_bin("q_i1.bin", p->ions[0].get_q(), sizeof(double) * X_NO_OF_CELLS * Y_NO_OF_CELLS);
        write_fields(p->grid_fields);
        // the reference's own text dump (particle.cpp:1361-1382)
        rename("dataDump_e.txt", "input_e.txt");
        rename("dataDump_i1.txt", "input_i1.txt");
        p->dump_data();
        rename("dataDump_e.txt", "dump_e.txt");
        rename("dataDump_i1.txt", "dump_i1.txt");
        rename("input_e.txt", "dataDump_e.txt");
        rename("input_i1.txt", "dataDump_i1.txt");
        delete p;
    } else if (mode == "fields") {
        const int nx = X_NO_OF_CELLS, ny = Y_NO_OF_CELLS;
        std::vector<double> rho(nx * ny);
        FILE* f = std::fopen("rho.bin", "rb");
        if (!f || std::fread(rho.data(), sizeof(double), rho.size(), f) != rho.size()) {
            std::fprintf(stderr, "cannot read rho.bin\n");
            return 3;
        }
        std::fclose(f);
        fields* fl = new fields();
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) fl->rho[j][i] = rho[j * nx + i];
        fl->grid_potential(PHI_LEFT, PHI_RIGHT, PHI_BOTTOM, PHI_TOP, 0, PHI_PERIOD);
        fl->grid_electric_field();
        write_fields(*fl);
        delete fl;
    } else if (mode == "sigma") {
        FILE* f = std::fopen("energies.bin", "rb");
        if (!f) { std::perror("energies.bin"); return 3; }
        std::vector<double> e;
        double v;
        while (std::fread(&v, sizeof v, 1, f) == 1) e.push_back(v);
        std::fclose(f);
        e_collisions ec;
        ion_collisions ic;
        std::vector<double> out(6 * e.size());
        for (size_t k = 0; k < e.size(); ++k) {
            ec.energy = e[k]; out[6 * k + 0] = ec.sigma_Ar_elastic();
            ec.energy = e[k]; out[6 * k + 1] = ec.sigma_Ar_ionize();
            ec.energy = e[k]; out[6 * k + 2] = ec.sigma_H_elastic();
            ec.energy = e[k]; out[6 * k + 3] = ec.sigma_H_ionize();
            ic.energy = e[k]; out[6 * k + 4] = ic.sigma_Ar_cx();
            ic.energy = e[k]; out[6 * k + 5] = ic.sigma_H_cx();   /* rescales its energy member */
        }
        write_bin("sigma.bin", out.data(), out.size() * sizeof(double));
    } else {
        std::cout.rdbuf(saved);
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 2;
    }
    std::cout.rdbuf(saved);
    return 0;
}
