/*
 * picgb.h -- C ABI of the GB300 particle-in-cell step library (libpicgb.so).
 *
 * One run handle (`pgb_run`) owns the device state of one 2D electrostatic PIC
 * simulation: electrons and one ion species, the charge/potential/field grids,
 * the multigrid levels and the per-step counters.  The entry points mirror the
 * per-step call sequence of the reference driver pic::pic_run
 * (pic.cpp:1069-1250) and the class methods it calls, so that a host driver
 * written against the reference can call them one for one.  Every function
 * returns 0 on success or a negative PGB_ERR_* code; pgb_last_error() then
 * holds a message.  No exception crosses this boundary, no torch type appears
 * in it, and every pointer argument is a plain host pointer borrowed for the
 * duration of the call.
 *
 * Units and layouts are the reference's: SI units; energies in eV where the
 * reference uses eV; particles as 6 doubles {x, y, vx, vy, vz, weight}
 * (particleVec.h:26-35); charge grids q as ny*nx doubles, row = y index
 * (particle.cpp:663-858); rho and phi as [ny][nx] (fields.cpp:42-62); E grids
 * as (nx+1)*(ny+1) doubles addressed with stride nx (fields.cpp:65-76,
 * 230-268).
 */
#ifndef PICGB_H
#define PICGB_H

#include <stdint.h>

#if defined(__GNUC__)
#define PGB_API __attribute__((visibility("default")))
#else
#define PGB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PGB_OK            0
#define PGB_ERR_ARG      -1   /* invalid argument or parameter set            */
#define PGB_ERR_CUDA     -2   /* a CUDA call failed (message names it)         */
#define PGB_ERR_NOMEM    -3   /* device or host allocation failed              */
#define PGB_ERR_CAPACITY -4   /* a particle or scratch capacity was exceeded   */
#define PGB_ERR_STATE    -5   /* call not valid in the handle's current state  */
#define PGB_ERR_IO       -6   /* file could not be read or written             */

/* Ions move far less per step than electrons, so their slot order stays
 * close to the cell order for longer: they are sorted this many times
 * less often.  The order of slots changes no deterministic result.      */
#define PGB_ION_SORT_FACTOR 4

/* ---- enumerations (string-valued macros of parameters.h) ---- */
enum { PGB_ELECTRONS = 0, PGB_IONS = 1 };
enum { PGB_ARGON = 0, PGB_HYDROGEN = 1 };                 /* SPECIES            */
enum { PGB_SIGMA_CONSTANT = 0, PGB_SIGMA_ENERGY_DEPENDENT = 1 };
enum { PGB_GRID_Q_E = 0, PGB_GRID_Q_I = 1, PGB_GRID_RHO = 2, PGB_GRID_PHI = 3,
       PGB_GRID_EX = 4, PGB_GRID_EY = 5 };
/* Poisson solver.  FMG_REF: the reference's one-pass full multigrid
 * (mglin.cpp:21-196) in FP64 with the same schedule -- bit-identical to the
 * reference for the same rho.  FMG32: the same schedule in FP32.  FP32_DC:
 * FP32 full multigrid inside an FP64 defect-correction loop, which converges
 * to the exact discrete solution (dc_max_iters passes).  DST_DC: the same
 * loop around an FP32 sine-transform solve of the discrete system (exact up
 * to FP32 rounding), so that two passes reach FP64 rounding.             */
enum { PGB_POISSON_FMG_REF = 0, PGB_POISSON_FP32_DC = 1, PGB_POISSON_FMG32 = 2, PGB_POISSON_DST_DC = 3 };
/* energy-dependent cross-section fits, for pgb_cross_sections()          */
enum { PGB_XS_AR_ELASTIC = 0, PGB_XS_AR_IONIZE = 1, PGB_XS_H_ELASTIC = 2, PGB_XS_H_IONIZE = 3,
       PGB_XS_AR_CX = 4, PGB_XS_H_CX = 5 };
/* boundary selector for pgb_boundary(): the two member-function pointers
 * implement_i_boundary / implement_e_boundary (boundary.h:372-383)          */
enum { PGB_BOUNDARY_IONS = 0, PGB_BOUNDARY_ELECTRONS = 1 };

/*
 * Run parameters.  Field names follow the parameters.h macros
 * (parameters.h:41-366, constants.h) and pic.cpp's initialize_* methods
 * (pic.cpp:226-529); pgb_params_default() fills in the reference's defaults.
 */
typedef struct pgb_params {
    int32_t x_no_of_cells;         /* X_NO_OF_CELLS (grid nodes, 2^k+1)          */
    int32_t y_no_of_cells;         /* Y_NO_OF_CELLS (must equal x_no_of_cells)   */
    double  xlength, ylength;      /* XLENGTH, YLENGTH [m]                        */
    double  dt, dti;               /* DT, DTI [s]; DT_DTI = (int)(dti/dt)         */
    double  electron_mass;         /* ELECTRON_MASS [kg]                          */
    double  ion_mass;              /* ION_MASS [kg]                               */
    double  q_over_me, q_over_mi;  /* Q_OVER_ME, Q_OVER_MI [C/kg]                 */
    double  qce, qci;              /* QCE, QCI: macro-particle charge [C]         */
    double  vte, vti, vtn;         /* VTE, VTI, VTN [m/s]                         */
    double  magnetic_field;        /* MAGNETIC_FIELD [T]                          */
    double  angle;                 /* ANGLE [rad]                                 */
    double  phi_left, phi_right, phi_bottom, phi_top;  /* wall potentials [V]    */
    double  phi_period;            /* PHI_PERIOD: right wall = phi_right*cos(phi_period*t) */
    double  neutral_density;       /* NEUTRAL_DENSITY [1/m^3]                     */
    double  threshold;             /* THRESHOLD: ionization threshold [eV]        */
    double  work_function;         /* WORK_FUNCTION [eV]                          */
    int32_t have_collisions;       /* HAVE_COLLISIONS                             */
    int32_t species;               /* SPECIES: PGB_ARGON / PGB_HYDROGEN           */
    int32_t sigma_cx_mode;         /* SIGMA            (CONSTANT/ENERGY_DEPENDENT) */
    int32_t sigma_elastic_mode;    /* SIGMA_ELASTIC                               */
    int32_t sigma_ionization_mode; /* SIGMA_IONIZATION                            */
    double  sigma_value;           /* SIGMA_VALUE [1e-20 m^2]                     */
    double  elastic_sigma_value;   /* ELASTIC_SIGMA_VALUE                         */
    double  ionization_sigma_value;/* IONIZATION_SIGMA_VALUE                      */
    int32_t e_impact_see;          /* E_IMPACT_SEE  (1 = "YES")                   */
    int32_t ion_impact_see;        /* ION_IMPACT_SEE                              */
    int32_t reflection;            /* REFLECTION                                  */
    int32_t backscatter;           /* BACKSCATTER                                 */
    int32_t steadystate;           /* STEADYSTATE                                 */
    int32_t number_to_inject;      /* NUMBER_TO_INJECT per species per step       */
    int32_t init_no_neutrals;      /* INIT_NO_NEUTRALS (neutral velocity table)   */
    double  see_e0, see_max_yield, see_emax0;  /* Vaughan constants (pic.cpp:459-477) */
    /* Kunhardt population control (parameters.h:339-366, pic.cpp:257-327)    */
    int32_t no_groups;             /* NO_GROUPS (<= 3)                            */
    double  v_limit_e[3], v_limit_i[3];
    int32_t group_limit_e[3], group_limit_i[3];
    int32_t new_group_size_e[3], new_group_size_i[3];
    int64_t size_to_check_e, size_to_check_i;  /* SIZE_TO_CHECK_E, SIZE_TO_CHECK */
    /* GB300 run controls (no reference counterpart)                          */
    uint64_t seed;                 /* Philox key for every random draw            */
    int32_t poisson_mode;          /* PGB_POISSON_*                               */
    int32_t dc_max_iters;          /* FP32_DC: max defect-correction passes       */
    double  dc_tolerance;          /* FP32_DC: stop when max|r| <= tol*max|f|     */
    int32_t sort_interval;         /* cell-sort electrons every k steps, ions every
                                      PGB_ION_SORT_FACTOR * k (0 = off)            */
    int64_t capacity_e, capacity_i;/* particle slots to reserve (0 = automatic)   */
} pgb_params;

/* Per-run counters, cumulative since pgb_create (read with pgb_get_counters). */
typedef struct pgb_counters {
    int64_t n_e, n_i;              /* live particles now                          */
    int64_t step;                  /* time steps taken (the reference's time_step) */
    int64_t absorbed_e, absorbed_i;/* removed at walls                            */
    int64_t plopped;               /* steady-state e-ion pairs re-inserted        */
    int64_t reflected, backscattered, see_events, see_emitted;  /* electron walls */
    int64_t ion_see_emitted;       /* electrons emitted by ion impact             */
    int64_t elastic, ionization, charge_exchange;  /* collisions                  */
    int64_t injected_e, injected_i;
    int64_t reductions_e, reductions_i;  /* Kunhardt reductions (count_reduce)    */
} pgb_counters;

/* Opt-in per-phase device time of pgb_step, from CUDA events recorded on
 * the run's stream around each phase (no reference counterpart).        */
typedef struct pgb_profile {
    double ms_push_e;              /* electron collisions+gather+push+deposit+lists */
    double ms_push_i;              /* ion gather+push+deposit+lists (or deposit)   */
    double ms_collide_ions;        /* charge exchange                              */
    double ms_walls;               /* wall passes, ionization products, injection  */
    double ms_fields;              /* charge finalisation, rho, Poisson, E         */
    int64_t steps;                 /* steps profiled                               */
    int64_t slots_e, slots_i;      /* particle slots swept by the push kernels     */
    int64_t launches;              /* kernel launches issued since pgb_create      */
    double ms_push_e_kernel;       /* the electron push kernel alone (in ms_push_e) */
    double ms_collide_e;           /* the electron collision-test kernel alone (in ms_push_e) */
    double ms_scatter_e;           /* the electron scattering kernel alone (in ms_push_e)     */
} pgb_profile;

typedef struct pgb_run pgb_run;

/* Fill *p with the reference's default parameters.h values (Ar, 257x257,
 * steady state, no collisions) and this library's run controls.           */
PGB_API int pgb_params_default(pgb_params* p);

/* Read the run parameters from a parameters.h file at run time: its macro
 * expressions are evaluated as the compiler would (C arithmetic, the
 * constants of constants.h), so derived quantities (DX, DT, VTE, ...) come
 * from the file itself (parameters.h:41-366).  RAND_SEED is replaced by
 * seed.  Returns PGB_ERR_IO when the file cannot be read or parsed.       */
PGB_API int pgb_params_from_header(const char* path, uint64_t seed, pgb_params* out);

/* pic::pic (pic.cpp:55-221) minus particle loading: allocate the device
 * state, build the neutral velocity tables (collisions.cpp:66-89).          */
PGB_API int pgb_create(const pgb_params* p, pgb_run** out);
/* pic::~pic (pic.cpp:1297-1340) */
PGB_API int pgb_destroy(pgb_run* run);
/* Message for the last failing call on this handle (never NULL). */
PGB_API const char* pgb_last_error(const pgb_run* run);

/* particle::load_particles (particle.cpp:359-401): replace the species'
 * particles with n records of 6 doubles (the dataDump_*.txt columns).       */
PGB_API int pgb_load_species(pgb_run* run, int species, const double* aos6, int64_t n);
/* particle::dump_data (particle.cpp:1361-1382) without the text formatting:
 * copy the live particles out as 6 doubles each.  *n_out = live count; at
 * most cap records are written.                                             */
PGB_API int pgb_dump_species(pgb_run* run, int species, double* aos6, int64_t cap, int64_t* n_out);
/* No reference counterpart (the reference's particles carry no identity):
 * the id of every live particle, in pgb_dump_species's order.  Ids key the
 * particle's random streams: loaded particles get 0..n-1, new ones the next
 * ids in creation order.  *n_out = live count; at most cap ids are written. */
PGB_API int pgb_dump_ids(pgb_run* run, int species, uint32_t* ids, int64_t cap, int64_t* n_out);
/* No reference counterpart: the library's FP32 forms of the cross-section
 * fits that the collision kernels use (e_collisions::sigma_Ar_elastic,
 * sigma_Ar_ionize, sigma_H_elastic, sigma_H_ionize at e_collisions.cpp:
 * 205-308; ion_collisions::sigma_Ar_cx, sigma_H_cx at ion_collisions.cpp:
 * 170-199), evaluated on the GPU at n energies (eV, host array; each is
 * converted to FP32 as the kernels hold it) into out (host, 1e-20 m^2).
 * which is a PGB_XS_* index.  For checking the fits against the
 * reference's FP64 functions.                                              */
PGB_API int pgb_cross_sections(int32_t which, const double* energies, int64_t n, double* out);
/* particle::particle_size */
PGB_API int pgb_species_count(pgb_run* run, int species, int64_t* n_out);

/* Set the reference's time_step counter (used by the right-wall potential
 * and the random streams).  pgb_step advances it.                           */
PGB_API int pgb_set_time_step(pgb_run* run, int64_t time_step);

/* The two boundary calls pic_run makes before its loop (pic.cpp:1049-1057). */
PGB_API int pgb_initial_boundary(pgb_run* run);
/* nsteps iterations of the pic_run loop body (pic.cpp:1069-1250) with fused
 * kernels; same physics and call order as the per-phase entry points.      */
PGB_API int pgb_step(pgb_run* run, int32_t nsteps);

/* pgb_step without waiting: the steps are queued on the run's stream and
 * the call returns (no reference counterpart).  pgb_query tells when the
 * run is idle again; pgb_sync waits for it.  Reads of the run's particles,
 * grids or counters wait for the queued steps themselves.               */
PGB_API int pgb_step_async(pgb_run* run, int32_t nsteps);
/* *idle = 1 when no work of the run is queued; device errors of finished
 * work are reported here.                                                */
PGB_API int pgb_query(pgb_run* run, int32_t* idle);
/* Step several independent runs nsteps each.  It has no counterpart in the
 * reference, which steps one run per process (pic.cpp:1069-1250).  Each
 * run's work is queued on its own stream, one step of every run in turn,
 * so that the kernels of runs too small to fill the GPU overlap.  Every run
 * ends in the same state as after pgb_step(run, nsteps) alone.  A handle
 * may appear once only.  On failure the failing run's pgb_last_error (for
 * an argument error, pgb_last_error(NULL)) holds the message.            */
PGB_API int pgb_step_batch(pgb_run* const* runs, int32_t nruns, int32_t nsteps);

/* ---- per-phase entry points, in pic_run order ---- */
PGB_API int pgb_collide_electrons(pgb_run* run);        /* e_collisions::collision (e_collisions.cpp:480-597) */
PGB_API int pgb_inject(pgb_run* run);                   /* particle::inject_more_particles, e then ions (particle.cpp:491-510) */
PGB_API int pgb_gather_push(pgb_run* run, int species); /* get_particle_electric_field + move_particles (particle.cpp:870-1341, pic.cl:56-149) */
PGB_API int pgb_collide_ions(pgb_run* run);             /* ion_collisions::collision (ion_collisions.cpp:255-308) */
PGB_API int pgb_boundary(pgb_run* run, int which);      /* implement_i_boundary / implement_e_boundary (boundary.cpp:581-1103) */
PGB_API int pgb_contain_growth(pgb_run* run, int species); /* particle::contain_particle_growth (particle.cpp:541-653) */
PGB_API int pgb_deposit(pgb_run* run, int species);     /* particle::collect_charge (particle.cpp:663-858, pic.cl:22-52) */
PGB_API int pgb_grid_rho(pgb_run* run);                 /* fields::grid_rho (fields.cpp:100-143) */
PGB_API int pgb_poisson(pgb_run* run, int64_t time_step); /* fields::grid_potential + Mglin (fields.cpp:169-220, mglin.cpp:21-196) */
PGB_API int pgb_efield(pgb_run* run);                   /* fields::grid_electric_field (fields.cpp:230-268) */

/* Copy a grid out in the reference layout (see the header comment).
 * n = number of doubles the caller's buffer holds.                        */
PGB_API int pgb_get_grid(pgb_run* run, int which, double* out, int64_t n);
/* Overwrite rho ([ny][nx]) before pgb_poisson, e.g. to solve a given
 * charge density without particles.                                       */
PGB_API int pgb_set_rho(pgb_run* run, const double* rho, int64_t n);
PGB_API int pgb_get_counters(pgb_run* run, pgb_counters* out);
/* The cudaStream_t every kernel of this run is launched on (so a caller
 * can record CUDA events around pgb_step).                               */
PGB_API int pgb_get_stream(pgb_run* run, void** stream);
/* Launch shapes (no reference counterpart).  They change no result, only
 * speed: the push kernels' grid is the SM count times push_blocks_per_sm
 * (four 256-thread blocks fit on an SM, default 8), and the collision
 * test, which runs beside the previous step's field solve, leaves it
 * field_sms SMs (default 32).                                             */
typedef struct pgb_launch_config {
    int32_t push_blocks_per_sm;
    int32_t field_sms;
} pgb_launch_config;
PGB_API int pgb_get_launch_config(pgb_run* run, pgb_launch_config* out);
/* From the next step on (waits for queued work; captured graphs are rebuilt). */
PGB_API int pgb_set_launch_config(pgb_run* run, const pgb_launch_config* c);
/* Time each candidate (push_blocks_per_sm 4, 8, 12 x field_sms 8, 16, 32,
 * 48, in that order) on this run: 2 untimed steps, then `steps` steps timed
 * with CUDA events on the run's stream; the fastest is kept, returned in
 * *best, its milliseconds per step in *ms_best; ms_all (12 values, may be
 * NULL) gets every candidate's.  The run advances 12 * (steps + 2) steps. */
PGB_API int pgb_autotune(pgb_run* run, int32_t steps, pgb_launch_config* best, double* ms_best, double* ms_all);
/* on = 1 resets and starts the per-phase profile of pgb_step; 0 stops it. */
PGB_API int pgb_set_profiling(pgb_run* run, int on);
PGB_API int pgb_get_profile(pgb_run* run, pgb_profile* out);
/* Wait for all work queued on the handle's stream. */
PGB_API int pgb_sync(pgb_run* run);
/* Device bytes a run of these parameters holds once ne electrons and ni ions
 * are loaded (no reference counterpart; used to admit runs by memory).   */
PGB_API int pgb_footprint(const pgb_params* p, int64_t ne, int64_t ni, int64_t* bytes);

/*
 * Serving: a request loop that keeps many independent runs resident on the
 * GPU and steps them together (no reference counterpart; the reference
 * runs one simulation per process).
 *   - pgb_server_submit copies a request (parameters, initial particles,
 *     step count) into the server's queue.
 *   - pgb_server_round admits queued requests, first fit in submission
 *     order, while their pgb_footprint fits the HBM budget and fewer than
 *     max_active runs are resident.  It gives every idle resident run its
 *     next chunk of min(round_steps, steps left) steps (pgb_step_async, so
 *     the chunks of all runs overlap), returns once at least one chunk has
 *     finished (at once when none is in flight), and retires the runs that
 *     are done.  A run never waits for the others' chunks.
 *   - pgb_server_result hands back a finished request's particles and frees
 *     them.
 * A request's result does not depend on the other requests it ran with.
 * One host thread drives a server.
 */
typedef struct pgb_server pgb_server;
typedef struct pgb_server_stats {
    int64_t submitted, admitted, completed, active, queued;
    int64_t run_steps;             /* steps executed, summed over runs            */
    double  particle_steps;        /* particles x steps, summed over runs         */
    double  busy_seconds;          /* wall time spent inside rounds               */
    double  step_ms_p50, step_ms_p99;  /* time per step of a resident run, from
                                          issuing a chunk to seeing it finished   */
    double  ttc_s_p50, ttc_s_p99;  /* submission to completion                     */
    int64_t hbm_in_use, hbm_budget;
    double  admit_seconds;         /* wall time creating and loading admitted runs */
    double  retire_seconds;        /* wall time reading back and freeing finished runs */
    double  issue_seconds;         /* wall time queueing chunks                    */
} pgb_server_stats;
PGB_API int pgb_server_create(int64_t hbm_budget_bytes, int32_t round_steps, int32_t max_active, pgb_server** out);
PGB_API int pgb_server_destroy(pgb_server* server);
PGB_API int pgb_server_submit(pgb_server* server, const pgb_params* p, const double* e_aos6, int64_t ne,
                              const double* i_aos6, int64_t ni, int32_t nsteps, int64_t* request_id);
/* *completed = requests finished in this round (ids via pgb_server_done) */
PGB_API int pgb_server_round(pgb_server* server, int32_t* completed);
/* ids of finished requests whose results have not been taken, up to cap */
PGB_API int pgb_server_done(pgb_server* server, int64_t* ids, int32_t cap, int32_t* n_out);
/* counts of a finished request's particles (to size the result buffers) */
PGB_API int pgb_server_result_size(pgb_server* server, int64_t id, int64_t* ne, int64_t* ni);
PGB_API int pgb_server_result(pgb_server* server, int64_t id, double* e_aos6, int64_t cap_e, double* i_aos6,
                              int64_t cap_i, pgb_counters* counters);
PGB_API int pgb_server_get_stats(pgb_server* server, pgb_server_stats* out);

/* ------------------------------------------------- averaged diagnostics
 * The graphs class (graphs.cpp, pic.cl:151-251) summed on the device.
 * Once enabled, every step t with start_step <= t < end_step adds, after
 * the field solve (pic.cpp:1189-1207):
 *   - rho, phi, Ex, Ey of every node (graphs::sum_fields);
 *   - each species' charge density / its macro charge (sum_density);
 *   - the mean vx of the particles in each cell of row ny/2, and the mean
 *     vy in each cell of column nx/2 (sum_av_velocities, pic.cl:154-186);
 *   - velocity histograms of NO_BINS bins of width vt/DIVIDE_BINS_BY at
 *     two locations (sum_av_dist, pic.cl:191-251).  The reference hands
 *     the kernel `spread` as an 8-byte double read from its int member and
 *     the next one, dist_locationX (graphs.cpp:865, graphs.h:281-282): the
 *     high word is dist_locationX, which makes the effective spread
 *     a denormal: each histogram takes the location's own cell only.  The
 *     same rule is kept here.
 * The reference's kernels add with plain `+=` from every work item; here
 * the counts are exact and the velocity sums are fixed point (2^-10 m/s).
 * Reading a graph divides by no_graph_steps as graphs::average_* do
 * (graphs.cpp:1000-1155); the velocity profiles of both species are
 * divided by VTE as in the reference (graphs.cpp:1114-1121).             */
typedef struct pgb_graphs_params {
    int64_t start_step, end_step;   /* summed steps: start <= t < end (START/END_GRAPH_TIME) */
    int32_t no_graph_steps;         /* NO_GRAPH_STEPS: divisor of every average */
    int32_t no_bins;                /* NO_BINS, odd */
    int32_t divide_bins_by;         /* DIVIDE_BINS_BY */
    int32_t spread;                 /* SPREAD */
    int32_t dist_location_x, dist_location_y;     /* DIST_LOCATIONX/Y   */
    int32_t dist_location2_x, dist_location2_y;   /* DIST_LOCATION2X/Y  */
} pgb_graphs_params;
enum {
    PGB_GRAPH_RHO = 0, PGB_GRAPH_PHI = 1, PGB_GRAPH_EX = 2, PGB_GRAPH_EY = 3,   /* [ny][nx]             */
    PGB_GRAPH_DENSITY = 4,                                                   /* [ny][nx], per species */
    PGB_GRAPH_VX = 5, PGB_GRAPH_VY = 6,                                      /* [nx] / [ny], per species */
    PGB_GRAPH_DIST_X1 = 7, PGB_GRAPH_DIST_Y1 = 8,                            /* [no_bins], per species */
    PGB_GRAPH_DIST_X2 = 9, PGB_GRAPH_DIST_Y2 = 10,
    PGB_GRAPH_MAXIMA = 11   /* 5 values: max phi, Ex, Ey, density e, density i (phiMax ... qMax) */
};
/* parameters.h's defaults for this grid (parameters.h:288-302), window empty */
PGB_API int pgb_graphs_params_default(const pgb_params* p, pgb_graphs_params* out);
/* allocate and zero the sums; steps queued later add to them */
PGB_API int pgb_graphs_enable(pgb_run* run, const pgb_graphs_params* g);
/* one averaged graph (waits for the run's queued steps) */
PGB_API int pgb_graphs_get(pgb_run* run, int which, int species, double* out, int64_t n);
/* the reference's graph files, names and formats, into dir
 * (graphs::write_*_to_file, graphs.cpp:1167-1370)                       */
PGB_API int pgb_graphs_write(pgb_run* run, const char* dir);

/* ------------------------------------------------ headless viewer plots
 * The interactive viewer's plots (the radio buttons of graphics.cpp:68-77,
 * drawn by graphics.cpp:245-607) rasterised with CUDA into an RGB image;
 * no graphics API is involved.  Row 0 of the image is the top; background
 * black.  Titles, labels and axes are not drawn.
 *   PARTICLE_XY   electrons (lime), then ions (hot pink) on top, as 2x2
 *                 pixel points over the domain (draw_particleXY, :512-607);
 *   *_VX_VY       vx-vy points of one species scaled by the integer part of
 *                 the largest |vx|, |vy| among the plotted particles (at
 *                 least 1), points with |v| below it (drawParticlePhase,
 *                 :396-509);
 *   PHI ... ION_DENSITY   one flat quad per grid cell, inset by a tenth of a
 *                 cell, coloured by |mean of its four corners| / |max| with
 *                 the five-band red-orange-yellow-green-blue-purple ramp
 *                 of drawField (:245-378); the densities skip the outer
 *                 ring (gridStart 1).  The field is the averaged graph when
 *                 graphs are enabled (the viewer's source, pic.cpp:918-960),
 *                 otherwise the current grid; the maximum is taken as
 *                 graphs::average_* take it (NaN values ignored).
 * max_points: particles per species (NUM_PARTICLES_TO_PLOT, 5000 in
 * graphics.h:77); <= 0 plots all.  Where a species has more, a particle is
 * plotted when a hash of its id and sample_seed falls below
 * max_points/n, instead of the viewer's rand() picks, so the sample does
 * not depend on the particle order.  rgb: width*height*3 host bytes.     */
enum { PGB_PLOT_PARTICLE_XY = 0, PGB_PLOT_ELECTRON_VX_VY = 1, PGB_PLOT_ION_VX_VY = 2, PGB_PLOT_PHI = 3,
       PGB_PLOT_EFIELD_X = 4, PGB_PLOT_EFIELD_Y = 5, PGB_PLOT_E_DENSITY = 6, PGB_PLOT_ION_DENSITY = 7 };
PGB_API int pgb_render(pgb_run* run, int plot, int32_t width, int32_t height, int32_t max_points,
                       uint32_t sample_seed, uint8_t* rgb, int64_t cap);

/*
 * Charge grid of one species from particle records already on the device,
 * with no run handle and no allocation.  It has no counterpart in the
 * reference: it is the deposit of pgb_deposit (particle::collect_charge,
 * particle.cpp:663-858) for callers that can't allocate device memory.
 * Two kinds of caller need it:
 *   - a diagnostic or viewer hook that runs between steps on the
 *     simulation's stream.  cudaMalloc and cudaFree would synchronise the
 *     device and drain the queued steps;
 *   - a host that has reserved the device memory for particle capacity.
 *
 * Arguments:
 *   d_aos6  device pointer to n particleVec records {x, y, vx, vy, vz, w}.
 *   d_q     device pointer that receives nx*ny doubles, equal to
 *           pgb_get_grid(PGB_GRID_Q_E or Q_I) after pgb_deposit on the same
 *           records.  Its layout is [ny][nx].
 *   dx, dy  cell sizes; qc is the macro-particle charge.
 *   stream  a cudaStream_t of the current device, or NULL for the default
 *           stream.  The work is queued on it and the call returns without
 *           waiting.
 *
 * Scratch: the per-node accumulator is a fixed device array of
 * PGB_STATIC_DEPOSIT_MAX_NODES entries (513 x 513 nodes, 2.1 MB).
 *   - A grid with more nodes returns PGB_ERR_CAPACITY, and
 *     pgb_last_error(NULL) names the limit.
 *   - Every call shares the array and clears the part it uses first.  Calls
 *     whose work overlaps on the GPU, such as calls on two streams without
 *     an event between them, race.
 *   - The first call on a device looks up the array with
 *     cudaGetSymbolAddress.  Make that first call with the device current,
 *     before any stream capture begins.
 *   - That address is kept for the life of the process.  A cudaDeviceReset
 *     of the device invalidates it: do not call this entry point on a
 *     device after resetting it.
 *
 * Errors: other failures return PGB_ERR_ARG or PGB_ERR_CUDA, with the
 * message in pgb_last_error(NULL).
 */
#define PGB_STATIC_DEPOSIT_MAX_NODES 263169
PGB_API int pgb_deposit_static(const double* d_aos6, int64_t n, int32_t nx, int32_t ny, double dx, double dy,
                               double qc, double* d_q, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PICGB_H */
