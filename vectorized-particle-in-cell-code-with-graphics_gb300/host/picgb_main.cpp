/*
 * picgb_run: batch-mode driver, the counterpart of the reference's main.cpp
 * batch branch (main.cpp:53-84): build the simulation from a parameters.h,
 * run pic_run, write the particle dump and timeData.txt.
 *
 *   picgb_run <parameters.h> <dir> [--steps N] [--seed S] [--restart|--fresh]
 *             [--verbose] [--no-dump] [--no-graphs] [--binary-dump]
 * dir holds dataDump_e.txt / dataDump_i1.txt for a restart and receives the
 * outputs: dataDump_*.txt, timeData.txt and, when the run reaches
 * END_GRAPH_TIME, the averaged graph files (pic.cpp:1209-1247).  Without
 * --steps the run length is TOTAL_RUN_TIME.  --binary-dump restarts from
 * dataDump_*.bin and writes them beside the text dumps: a lossless copy of
 * the state (the text keeps 6 digits).
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include "pic_host.h"

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr,
                     "usage: %s <parameters.h> <dir> [--steps N] [--seed S] [--restart|--fresh] [--verbose] [--no-dump] "
                     "[--no-graphs] [--binary-dump]\n",
                     argv[0]);
        return 2;
    }
    std::string params = argv[1], dir = argv[2];
    long long steps = -1;
    unsigned long long seed = 1;
    int restart = -1;
    bool verbose = false, dump = true, graphs = true, binary = false;
    for (int k = 3; k < argc; ++k) {
        if (!std::strcmp(argv[k], "--steps") && k + 1 < argc) steps = std::atoll(argv[++k]);
        else if (!std::strcmp(argv[k], "--seed") && k + 1 < argc) seed = std::strtoull(argv[++k], nullptr, 10);
        else if (!std::strcmp(argv[k], "--restart")) restart = 1;
        else if (!std::strcmp(argv[k], "--fresh")) restart = 0;
        else if (!std::strcmp(argv[k], "--verbose")) verbose = true;
        else if (!std::strcmp(argv[k], "--no-dump")) dump = false;
        else if (!std::strcmp(argv[k], "--no-graphs")) graphs = false;
        else if (!std::strcmp(argv[k], "--binary-dump")) binary = true;
        else { std::fprintf(stderr, "unknown argument %s\n", argv[k]); return 2; }
    }
    try {
        picgb::MacroTable m = picgb::read_parameters_h(params);
        if (restart < 0) restart = m.has("RESTART") ? (m.flag("RESTART") ? 1 : 0) : 0;
        if (steps < 0) steps = (long long)m.number("TOTAL_RUN_TIME");
        picgb::Pic pic(m, dir, restart == 1, seed, binary);
        pic.set_write_graph_data_to_files(graphs);
        auto t0 = std::chrono::steady_clock::now();
        pic.pic_run((int)steps, verbose);
        auto t1 = std::chrono::steady_clock::now();
        double s = std::chrono::duration<double>(t1 - t0).count();
        pgb_counters c = pic.counters();
        std::printf("duration of PIC run loop = %.3f s (%lld steps, %lld electrons, %lld ions)\n", s, steps,
                    (long long)c.n_e, (long long)c.n_i);
        pic.write_time_data();
        if (dump) pic.dump_data();
    } catch (const picgb::Error& e) {
        std::fprintf(stderr, "picgb_run: %s\n", e.what());
        return 1;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "picgb_run: %s\n", e.what());
        return 1;
    }
    return 0;
}
