/*
 * picport.h -- CPU restatement of the reference PIC step, in FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA library is checked
 * against (tests/, __graft_entry__.smoke) and the CPU baseline bench.py times.
 * Nothing in the product links it.
 *
 * Every routine restates one reference routine (file:line cited at each
 * function in picport.c) with the same floating-point operation order, so
 * that with ORC_RNG_LIBC + ORC_ORDER_REF it reproduces the reference binary
 * built by oracle/Makefile bit for bit (pinned by tests/test_oracle_pin.py).
 * Two switches select what may differ from the reference:
 *   rng   ORC_RNG_LIBC   draws from rand() in the reference's call order
 *         ORC_RNG_PHILOX draws from the library's Philox streams (pgb_rng.h)
 *   order ORC_ORDER_REF    removes particles by swap-with-last (boundary.cpp:654-666)
 *         ORC_ORDER_STABLE removes particles by stable compaction and appends
 *                          wall secondaries at the end, as the CUDA library does
 * The CUDA library is compared against (PHILOX, STABLE).
 */
#ifndef PICPORT_H
#define PICPORT_H
#include <stdint.h>
#include "picgb.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_RNG_LIBC = 0, ORC_RNG_PHILOX = 1 };
enum { ORC_ORDER_REF = 0, ORC_ORDER_STABLE = 1 };

typedef struct orc_run orc_run;

orc_run* orc_create(const pgb_params* p, int rng_mode, int order_mode);
void     orc_destroy(orc_run* r);
int      orc_load_species(orc_run* r, int sp, const double* aos6, int64_t n);
int64_t  orc_count(orc_run* r, int sp);
int64_t  orc_dump_species(orc_run* r, int sp, double* aos6, uint32_t* ids, int64_t cap);
void     orc_set_time_step(orc_run* r, int64_t t);
void     orc_set_threads(orc_run* r, int threads);

void orc_initial_boundary(orc_run* r);
void orc_step(orc_run* r, int nsteps);

void orc_collide_electrons(orc_run* r);
void orc_inject(orc_run* r);
void orc_gather_push(orc_run* r, int sp);
void orc_collide_ions(orc_run* r);
void orc_boundary(orc_run* r, int which);
void orc_contain_growth(orc_run* r, int sp);
void orc_deposit(orc_run* r, int sp);
void orc_grid_rho(orc_run* r);
void orc_poisson(orc_run* r, int64_t t);
void orc_efield(orc_run* r);

int  orc_get_grid(orc_run* r, int which, double* out, int64_t n);
int  orc_set_rho(orc_run* r, const double* rho, int64_t n);
void orc_get_counters(orc_run* r, pgb_counters* out);
int  orc_get_neutral_table(orc_run* r, int which, double* out, int64_t n);
/* FP64 residual max|f - L u| of the current phi on the interior, and max|f|
 * (f = the Poisson right-hand side assembled by orc_poisson)               */
void orc_poisson_residual(orc_run* r, double* max_res, double* max_rhs);
/* solve the same discrete Poisson problem to convergence (FP64 defect
 * correction around the full multigrid pass) -- the "exact" reference for
 * PGB_POISSON_FP32_DC and PGB_POISSON_DST_DC                                  */
void orc_poisson_converged(orc_run* r, int64_t t, int iters);
/* the graphs class (graphs.cpp): sums over the window's steps, read as
 * the reference's averages; `which` and the layouts are PGB_GRAPH_*       */
int  orc_graphs_enable(orc_run* r, const pgb_graphs_params* g);
int  orc_graphs_get(orc_run* r, int which, int species, double* out, int64_t n);
/* headless viewer plots, the rules of pgb_render (RGB8, row 0 at the top) */
int  orc_render(orc_run* r, int plot, int W, int H, int max_points, uint32_t seed, unsigned char* img, int64_t cap);
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* one of the energy-dependent cross-section fits (PGB_XS_*) at e eV      */
double orc_sigma(int which, double e);

#ifdef __cplusplus
}
#endif
#endif
