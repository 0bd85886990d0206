/*
 * picport.c -- CPU restatement of the reference PIC time step in FP64.
 *
 * TEST INFRASTRUCTURE ONLY (see picport.h).  Each function cites the
 * reference routine it restates.  Floating-point expressions keep the
 * reference's operation order, and the file is compiled with
 * -ffp-contract=off, so that with ORC_RNG_LIBC + ORC_ORDER_REF the results
 * equal the reference binary's bit for bit on the same host.
 *
 * Cell indices: the reference converts x/DX with a C cast (e.g. pic.cl:31,
 * boundary.cpp:595).  On x86-64 (the reference's platform) a NaN or an
 * out-of-range value converts to INT_MIN, which makes NaN particles count as
 * being outside the left wall; on other hosts the cast differs.  cell() fixes
 * the x86-64 result on every host.
 */
#define _GNU_SOURCE
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "picport.h"
#include "pgb_rng.h"

/* constants.h:17-26 */
#define C_PI 3.141592654
#define C_CHARGE 1.602177e-19
#define C_EPSILON 8.854e-12
#define C_EMASS 9.10939e-31
#define C_AMU 1.66054e-27

typedef struct { double x, y, vx, vy, vz, w; } orc_pv;   /* particleVec.h:26-35 */

typedef struct {
    orc_pv* p;
    uint32_t* id;
    int64_t n, cap;
    uint32_t next_id;
    double qc, q_over_m, mass, vt, dt;
} orc_sp;

struct orc_run {
    pgb_params prm;
    int rng_mode, order_mode, threads;
    int nx, ny, dt_dti;
    double dx, dy;
    orc_sp sp[2];
    double *q[2], *rho, *phi, *rhs, *ex, *ey;
    double *efx, *efy;
    int64_t ef_cap;
    double* neut[2][3];  /* [0] e_collisions table, [1] ion_collisions table */
    double* prob_cx;
    int64_t time_step;
    uint32_t rng_step;
    pgb_counters c;
    int ng;              /* multigrid levels */
    double *mg_u[32], *mg_rhs[32], *mg_res[32], *mg_tmp[32], *mg_v[32];
    pgb_stream st;
    /* graphs class sums (orc_graphs_enable) */
    int gr_on;
    pgb_graphs_params gr;
    double* gr_f[4];       /* rho, phi, Ex, Ey [ny][nx]                     */
    double* gr_q[2];       /* density per species [ny][nx]                  */
    double* gr_v[2][2];    /* per-cell mean vx along row ny/2, vy along column nx/2 */
    double* gr_d[2][4];    /* histograms X1, Y1, X2, Y2 [no_bins]           */
};

static inline int cell(double v) {
    return (v > -2147483649.0 && v < 2147483648.0) ? (int)v : INT_MIN;
}

/* ------------------------------------------------------------------ rng */
static void rng_begin(orc_run* r, uint32_t id, uint32_t stream, int sp) {
    if (r->rng_mode == ORC_RNG_PHILOX) pgb_stream_init(&r->st, r->prm.seed, id, r->rng_step, stream, (uint32_t)sp);
}
static double rng_u01(orc_run* r) {
    if (r->rng_mode == ORC_RNG_LIBC) return (double)rand() / ((double)RAND_MAX);
    return pgb_u01d(pgb_stream_u32(&r->st));
}
static uint32_t rng_int(orc_run* r) {
    if (r->rng_mode == ORC_RNG_LIBC) return (uint32_t)rand();
    return pgb_stream_u32(&r->st);
}

/* ------------------------------------------------------------ storage */
static void sp_reserve(orc_sp* s, int64_t need) {
    if (need <= s->cap) return;
    int64_t cap = s->cap ? s->cap : 1024;
    while (cap < need) cap *= 2;
    s->p = (orc_pv*)realloc(s->p, (size_t)cap * sizeof(orc_pv));
    s->id = (uint32_t*)realloc(s->id, (size_t)cap * sizeof(uint32_t));
    if (!s->p || !s->id) { fprintf(stderr, "picport: out of memory\n"); abort(); }
    s->cap = cap;
}
/* push_back(particleVec()) : value-initialised record (all zero) */
static int64_t sp_push(orc_sp* s) {
    sp_reserve(s, s->n + 1);
    memset(&s->p[s->n], 0, sizeof(orc_pv));
    s->id[s->n] = s->next_id++;
    return s->n++;
}
/* swap(v[i], v[n-1]); v.pop_back()  (boundary.cpp:654-666) */
static void sp_swap_pop(orc_sp* s, int64_t i) {
    orc_pv t = s->p[i]; s->p[i] = s->p[s->n - 1]; s->p[s->n - 1] = t;
    uint32_t u = s->id[i]; s->id[i] = s->id[s->n - 1]; s->id[s->n - 1] = u;
    s->n--;
}
/* stable removal of the records flagged in dead[] */
static void sp_compact(orc_sp* s, const unsigned char* dead) {
    int64_t k = 0;
    for (int64_t i = 0; i < s->n; ++i) {
        if (dead[i]) continue;
        s->p[k] = s->p[i]; s->id[k] = s->id[i]; ++k;
    }
    s->n = k;
}

/* --------------------------------------------------------- velocities */
/* particle::get_particle_velocity (particle.cpp:452-464) and
 * boundary::get_particle_velocity (boundary.cpp:833-845)                 */
static double maxwell_component(orc_run* r, double vt) {
    double v;
    do {
        double R1 = rng_u01(r);
        double R2 = rng_u01(r);
        v = vt * cos(2.0 * C_PI * R2) * sqrt(fabs(log(R1)));
    } while (fabs(v) > vt * 10000);
    return v;
}

/* collisions::calc_neutral_velocity (collisions.cpp:66-89) */
static void neutral_table(orc_run* r, double* vx, double* vy, double* vz, int which) {
    const double vtn = r->prm.vtn;
    const int n = r->prm.init_no_neutrals;
    for (int i = 0; i < n; ++i) {
        rng_begin(r, (uint32_t)i, which ? PGB_STREAM_NEUTRAL_I : PGB_STREAM_NEUTRAL_E, 0);
        do {
            double R1 = rng_u01(r);
            double R2 = rng_u01(r);
            vx[i] = vtn * cos(C_PI * R2) * sqrt(fabs(log(R1)));
        } while (fabs(vx[i]) > 10000.0 * vtn);
        do {
            double R1 = rng_u01(r);
            double R2 = rng_u01(r);
            vy[i] = vtn * cos(C_PI * R2) * sqrt(fabs(log(R1)));
            vz[i] = vtn * sin(C_PI * R2) * sqrt(fabs(log(R1)));
        } while (fabs(vy[i]) > 10000.0 * vtn || fabs(vz[i]) > 10000.0 * vtn);
    }
}

/* ------------------------------------------------------------- create */
orc_run* orc_create(const pgb_params* p, int rng_mode, int order_mode) {
    if (!p || p->x_no_of_cells < 3 || p->y_no_of_cells != p->x_no_of_cells) return NULL;
    int n = p->x_no_of_cells;
    if (((n - 1) & (n - 2)) != 0) return NULL;   /* n-1 must be a power of two (mglin.cpp:26) */
    orc_run* r = (orc_run*)calloc(1, sizeof(orc_run));
    r->prm = *p;
    r->rng_mode = rng_mode;
    r->order_mode = order_mode;
    r->threads = 1;
    r->nx = p->x_no_of_cells;
    r->ny = p->y_no_of_cells;
    r->dx = p->xlength / (double)(r->nx - 1);   /* parameters.h:193-194 */
    r->dy = p->ylength / (double)(r->ny - 1);
    r->dt_dti = (int)(p->dti / p->dt);          /* parameters.h:215 */
    if (r->dt_dti < 1) r->dt_dti = 1;
    /* pic::initialize_electron_particles / initialize_ion_particles (pic.cpp:226-332) */
    r->sp[0].qc = p->qce; r->sp[0].q_over_m = p->q_over_me; r->sp[0].mass = p->electron_mass;
    r->sp[0].vt = p->vte; r->sp[0].dt = p->dt;
    r->sp[1].qc = p->qci; r->sp[1].q_over_m = p->q_over_mi; r->sp[1].mass = p->ion_mass;
    r->sp[1].vt = p->vti; r->sp[1].dt = p->dti;
    size_t g = (size_t)r->nx * r->ny, ge = (size_t)(r->nx + 1) * (r->ny + 1);
    r->q[0] = (double*)calloc(g, sizeof(double));
    r->q[1] = (double*)calloc(g, sizeof(double));
    r->rho = (double*)calloc(g, sizeof(double));
    r->phi = (double*)calloc(g, sizeof(double));
    r->rhs = (double*)calloc(g, sizeof(double));
    r->ex = (double*)calloc(ge, sizeof(double));
    r->ey = (double*)calloc(ge, sizeof(double));
    r->prob_cx = (double*)calloc((size_t)r->nx, sizeof(double));
    for (int t = 0; t < 2; ++t)
        for (int k = 0; k < 3; ++k) r->neut[t][k] = (double*)calloc((size_t)p->init_no_neutrals, sizeof(double));
    /* multigrid levels, finest = ng-1 */
    int ng = 0, nn = n;
    while (nn >>= 1) ng++;
    r->ng = ng;
    nn = n;
    for (int j = ng - 1; j >= 0; --j) {
        size_t s = (size_t)nn * nn;
        r->mg_u[j] = (double*)calloc(s, sizeof(double));
        r->mg_rhs[j] = (double*)calloc(s, sizeof(double));
        r->mg_res[j] = (double*)calloc(s, sizeof(double));
        r->mg_tmp[j] = (double*)calloc(s, sizeof(double));
        r->mg_v[j] = (double*)calloc(s, sizeof(double));
        nn = nn / 2 + 1;
    }
    /* pic::pic: srand(RAND_SEED) precedes construction (main.cpp:35); the
     * neutral tables are built ion first, then electron (pic.cpp:135-138) */
    if (rng_mode == ORC_RNG_LIBC) srand((unsigned)p->seed);
    r->rng_step = 0;
    neutral_table(r, r->neut[1][0], r->neut[1][1], r->neut[1][2], 1);
    neutral_table(r, r->neut[0][0], r->neut[0][1], r->neut[0][2], 0);
    return r;
}

void orc_destroy(orc_run* r) {
    if (!r) return;
    for (int s = 0; s < 2; ++s) { free(r->sp[s].p); free(r->sp[s].id); free(r->q[s]); }
    free(r->rho); free(r->phi); free(r->rhs); free(r->ex); free(r->ey);
    free(r->efx); free(r->efy); free(r->prob_cx);
    for (int t = 0; t < 2; ++t) for (int k = 0; k < 3; ++k) free(r->neut[t][k]);
    for (int j = 0; j < r->ng; ++j) { free(r->mg_u[j]); free(r->mg_rhs[j]); free(r->mg_res[j]); free(r->mg_tmp[j]); free(r->mg_v[j]); }
    for (int k = 0; k < 4; ++k) free(r->gr_f[k]);
    for (int s = 0; s < 2; ++s) {
        free(r->gr_q[s]); free(r->gr_v[s][0]); free(r->gr_v[s][1]);
        for (int k = 0; k < 4; ++k) free(r->gr_d[s][k]);
    }
    free(r);
}

void orc_set_threads(orc_run* r, int threads) { r->threads = threads > 0 ? threads : 1; }
/* the phase entry points draw from the streams of step t, as pic_run's
 * loop body for time_step = t does                                     */
void orc_set_time_step(orc_run* r, int64_t t) { r->time_step = t; r->c.step = t; r->rng_step = (uint32_t)t; }

int orc_load_species(orc_run* r, int sp, const double* aos6, int64_t n) {
    if (sp < 0 || sp > 1 || n < 0) return PGB_ERR_ARG;
    orc_sp* s = &r->sp[sp];
    sp_reserve(s, n);
    memcpy(s->p, aos6, (size_t)n * sizeof(orc_pv));
    for (int64_t i = 0; i < n; ++i) s->id[i] = (uint32_t)i;
    s->n = n;
    s->next_id = (uint32_t)n;
    return 0;
}

int64_t orc_count(orc_run* r, int sp) { return r->sp[sp].n; }

int64_t orc_dump_species(orc_run* r, int sp, double* aos6, uint32_t* ids, int64_t cap) {
    orc_sp* s = &r->sp[sp];
    int64_t n = s->n < cap ? s->n : cap;
    if (aos6) memcpy(aos6, s->p, (size_t)n * sizeof(orc_pv));
    if (ids) memcpy(ids, s->id, (size_t)n * sizeof(uint32_t));
    return s->n;
}

int orc_get_neutral_table(orc_run* r, int which, double* out, int64_t n) {
    int m = r->prm.init_no_neutrals;
    if (n < 3 * (int64_t)m) return PGB_ERR_ARG;
    for (int k = 0; k < 3; ++k) memcpy(out + (size_t)k * m, r->neut[which][k], (size_t)m * sizeof(double));
    return 0;
}

/* ------------------------------------------------- deposit / gather / push */
/* particle::collect_charge (particle.cpp:663-858) with the collectCharge
 * kernel (pic.cl:22-52) run in particle order, then the edge doubling
 * (particle.cpp:829-845)                                                   */
void orc_deposit(orc_run* r, int spi) {
    orc_sp* s = &r->sp[spi];
    const int nx = r->nx, ny = r->ny;
    const double dx = r->dx, dy = r->dy;
    const double qc_dxdy = s->qc / (dx * dy);
    double* q = r->q[spi];
    memset(q, 0, sizeof(double) * (size_t)nx * ny);
    int nt = r->threads;
    if (nt <= 1) {
        for (int64_t g = 0; g < s->n; ++g) {
            const orc_pv* P = &s->p[g];
            int jp = cell(P->x / dx), kp = cell(P->y / dy);
            if (jp < nx - 1 && P->x > 0.0 && kp < ny - 1 && P->y > 0.0) {
                double wj = P->x / dx - (double)jp, wk = P->y / dy - (double)kp;
                double a4 = (1.0 - wj) * (1.0 - wk), a3 = wj * (1.0 - wk);
                double a2 = wk * (1.0 - wj), a1 = wj * wk;
                q[kp * nx + jp] += qc_dxdy * a4 * P->w;
                q[kp * nx + jp + 1] += qc_dxdy * a3 * P->w;
                q[(kp + 1) * nx + jp] += qc_dxdy * a2 * P->w;
                q[(kp + 1) * nx + jp + 1] += qc_dxdy * a1 * P->w;
            }
        }
    } else {
        /* timing mode: per-thread private grids (summation order differs) */
        size_t G = (size_t)nx * ny;
        double* priv = (double*)calloc(G * (size_t)nt, sizeof(double));
#pragma omp parallel num_threads(nt)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double* qq = priv + G * (size_t)t;
#pragma omp for schedule(static)
            for (int64_t g = 0; g < s->n; ++g) {
                const orc_pv* P = &s->p[g];
                int jp = cell(P->x / dx), kp = cell(P->y / dy);
                if (jp < nx - 1 && P->x > 0.0 && kp < ny - 1 && P->y > 0.0) {
                    double wj = P->x / dx - (double)jp, wk = P->y / dy - (double)kp;
                    double a4 = (1.0 - wj) * (1.0 - wk), a3 = wj * (1.0 - wk);
                    double a2 = wk * (1.0 - wj), a1 = wj * wk;
                    qq[kp * nx + jp] += qc_dxdy * a4 * P->w;
                    qq[kp * nx + jp + 1] += qc_dxdy * a3 * P->w;
                    qq[(kp + 1) * nx + jp] += qc_dxdy * a2 * P->w;
                    qq[(kp + 1) * nx + jp + 1] += qc_dxdy * a1 * P->w;
                }
            }
        }
        for (int t = 0; t < nt; ++t)
            for (size_t k = 0; k < G; ++k) q[k] += priv[G * (size_t)t + k];
        free(priv);
    }
    for (int j = 0; j < ny; j++) { q[j * nx] *= 2.0; q[j * nx + nx - 1] *= 2.0; }
    for (int i = 0; i < nx; i++) { q[i] *= 2.0; q[(ny - 1) * nx + i] *= 2.0; }
    q[0] *= 2.0;
    q[nx - 1] *= 2.0;
    q[(ny - 1) * nx] *= 2.0;
    q[(ny - 1) * nx + nx - 1] *= 2.0;
}

/* particle::get_particle_electric_field + move_particles
 * (particle.cpp:870-1341; kernels pic.cl:56-92 and pic.cl:95-149)         */
void orc_gather_push(orc_run* r, int spi) {
    orc_sp* s = &r->sp[spi];
    const int nx = r->nx, ny = r->ny;
    const double dx = r->dx, dy = r->dy;
    const double* Ex = r->ex;
    const double* Ey = r->ey;
    const double dt = s->dt;
    const double coef = 0.5 * dt * s->q_over_m;
    const double omega_dt = dt * s->q_over_m * r->prm.magnetic_field;
    const double B = r->prm.magnetic_field;
    const double ca = cos(r->prm.angle), sa = sin(r->prm.angle);
    const double co = cos(omega_dt), so = sin(omega_dt);
    const int64_t n = s->n;
#pragma omp parallel for num_threads(r->threads) schedule(static)
    for (int64_t g = 0; g < n; ++g) {
        orc_pv* P = &s->p[g];
        int jp = cell(P->x / dx), kp = cell(P->y / dy);
        double Exp = 0.0, Eyp = 0.0;
        if (jp < nx && P->x > 0.0 && kp < ny && P->y > 0.0) {
            double wj = P->x / dx - (double)jp, wk = P->y / dy - (double)kp;
            double a4 = (1.0 - wj) * (1.0 - wk), a3 = wj * (1.0 - wk);
            double a2 = wk * (1.0 - wj), a1 = wj * wk;
            Exp = a4 * Ex[kp * nx + jp] + a3 * Ex[kp * nx + jp + 1] +
                  a2 * Ex[(kp + 1) * nx + jp] + a1 * Ex[(kp + 1) * nx + jp + 1];
            Eyp = a4 * Ey[kp * nx + jp] + a3 * Ey[kp * nx + jp + 1] +
                  a2 * Ey[(kp + 1) * nx + jp] + a1 * Ey[(kp + 1) * nx + jp + 1];
        }
        /* move_particles recomputes jp, kp from the same position */
        if (jp < nx && P->x > 0.0 && kp < ny && P->y > 0.0) {
            P->vx += coef * Exp;
            P->vy += coef * Eyp;
            if (B > 0.0) {
                double vpar = ca * P->vx + sa * P->vy;
                double vperp = -sa * P->vx + ca * P->vy;
                double vperp_after = vperp * co + so * P->vz;
                P->vz = -vperp * so + co * P->vz;
                P->vx = ca * vpar - sa * vperp_after;
                P->vy = sa * vpar + ca * vperp_after;
            }
            P->vx += coef * Exp;
            P->vy += coef * Eyp;
            P->x += dt * P->vx;
            P->y += dt * P->vy;
        }
    }
}

/* ---------------------------------------------------------------- fields */
/* fields::grid_rho (fields.cpp:100-143) */
void orc_grid_rho(orc_run* r) {
    size_t G = (size_t)r->nx * r->ny;
    for (size_t k = 0; k < G; ++k) r->rho[k] = r->q[1][k];
    for (size_t k = 0; k < G; ++k) r->rho[k] += r->q[0][k];
}

/* Full multigrid V(1,1) on the square grid, the algorithm of Numerical
 * Recipes 3rd ed. section 20.6 as the reference uses it (mglin.cpp:21-196):
 * red-black Gauss-Seidel smoothing, half-weighting restriction with
 * injected boundary values, bilinear prolongation, an exact 3x3 solve with
 * h = length/2 at the bottom, nested iteration from the 3x3 grid with
 * ncycle V-cycles per level.  h = length/(n-1) on each level.            */
static void mg_relax(double* u, const double* f, int n, double length) {
    double h = length / (n - 1), h2 = h * h;
    for (int color = 0; color < 2; ++color)
        for (int i = 1; i < n - 1; ++i)
            for (int j = 1 + ((i + 1 + color) & 1); j < n - 1; j += 2)
                u[i * n + j] = 0.25 * (u[(i + 1) * n + j] + u[(i - 1) * n + j] + u[i * n + j + 1] +
                                       u[i * n + j - 1] - h2 * f[i * n + j]);
}
static void mg_resid(double* res, const double* u, const double* f, int n, double length) {
    double h = length / (n - 1), h2i = 1.0 / (h * h);
    for (int i = 1; i < n - 1; ++i)
        for (int j = 1; j < n - 1; ++j)
            res[i * n + j] = -h2i * (u[(i + 1) * n + j] + u[(i - 1) * n + j] + u[i * n + j + 1] +
                                     u[i * n + j - 1] - 4.0 * u[i * n + j]) + f[i * n + j];
    for (int i = 0; i < n; ++i) {
        res[i * n] = 0.0; res[i * n + n - 1] = 0.0; res[i] = 0.0; res[(n - 1) * n + i] = 0.0;
    }
}
static void mg_restrict(double* uc, const double* uf, int nc) {
    int nf = 2 * nc - 1;
    for (int ic = 1; ic < nc - 1; ++ic)
        for (int jc = 1; jc < nc - 1; ++jc) {
            int i = 2 * ic, j = 2 * jc;
            uc[ic * nc + jc] = 0.5 * uf[i * nf + j] +
                               0.125 * (uf[(i + 1) * nf + j] + uf[(i - 1) * nf + j] + uf[i * nf + j + 1] + uf[i * nf + j - 1]);
        }
    for (int ic = 0; ic < nc; ++ic) {
        uc[ic * nc] = uf[(2 * ic) * nf];
        uc[ic * nc + nc - 1] = uf[(2 * ic) * nf + nf - 1];
    }
    for (int jc = 0; jc < nc; ++jc) {
        uc[jc] = uf[2 * jc];
        uc[(nc - 1) * nc + jc] = uf[(nf - 1) * nf + 2 * jc];
    }
}
static void mg_prolong(double* uf, const double* uc, int nf) {
    int nc = nf / 2 + 1;
    for (int ic = 0; ic < nc; ++ic)
        for (int jc = 0; jc < nc; ++jc) uf[(2 * ic) * nf + 2 * jc] = uc[ic * nc + jc];
    for (int j = 0; j < nf; j += 2)
        for (int i = 1; i < nf - 1; i += 2) uf[i * nf + j] = 0.5 * (uf[(i + 1) * nf + j] + uf[(i - 1) * nf + j]);
    for (int j = 1; j < nf - 1; j += 2)
        for (int i = 0; i < nf; ++i) uf[i * nf + j] = 0.5 * (uf[i * nf + j + 1] + uf[i * nf + j - 1]);
}
static void mg_coarsest(double* u, const double* f, double length) {
    double h = 0.5 * length;
    for (int k = 0; k < 9; ++k) u[k] = 0.0;
    u[4] = -h * h * f[4] / 4.0;
}
static void mg_vcycle(orc_run* r, int j, double* u, const double* f, int n, double length) {
    if (j == 0) { mg_coarsest(u, f, length); return; }
    int nc = (n + 1) / 2;
    double* tmp = r->mg_tmp[j];
    double* res = r->mg_res[j - 1];
    double* v = r->mg_v[j - 1];
    mg_relax(u, f, n, length);
    mg_resid(tmp, u, f, n, length);
    mg_restrict(res, tmp, nc);
    memset(v, 0, sizeof(double) * (size_t)nc * nc);
    mg_vcycle(r, j - 1, v, res, nc, length);
    mg_prolong(tmp, v, n);
    for (int k = 0; k < n * n; ++k) u[k] += tmp[k];
    mg_relax(u, f, n, length);
}
static void mg_fmg(orc_run* r, double* u_io, int n, double length, int ncycle) {
    int ng = r->ng;
    memcpy(r->mg_rhs[ng - 1], u_io, sizeof(double) * (size_t)n * n);
    int nn = n;
    for (int j = ng - 2; j >= 0; --j) {
        nn = nn / 2 + 1;
        mg_restrict(r->mg_rhs[j], r->mg_rhs[j + 1], nn);
    }
    mg_coarsest(r->mg_u[0], r->mg_rhs[0], length);
    nn = 3;
    for (int j = 1; j < ng; ++j) {
        nn = 2 * nn - 1;
        mg_prolong(r->mg_u[j], r->mg_u[j - 1], nn);
        for (int c = 0; c < ncycle; ++c) mg_vcycle(r, j, r->mg_u[j], r->mg_rhs[j], nn, length);
    }
    memcpy(u_io, r->mg_u[ng - 1], sizeof(double) * (size_t)n * n);
}

/* fields::grid_potential (fields.cpp:169-220): right-hand side -rho/eps0
 * with the wall potentials folded into the first interior rows/columns,
 * one FMG pass, then the wall values written on the edges.               */
static void assemble_rhs(orc_run* r, double* f, double phi_right) {
    const int nx = r->nx, ny = r->ny;
    const double coef = 1.0 / C_EPSILON;
    const double divdxdy = 1.0 / (r->dx * r->dy);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) f[j * nx + i] = -coef * r->rho[j * nx + i];
    for (int j = 0; j < ny; j++) {
        f[j * nx + 1] = f[j * nx + 1] - r->prm.phi_left * divdxdy;
        f[j * nx + nx - 2] = f[j * nx + nx - 2] - phi_right * divdxdy;
    }
    for (int i = 0; i < nx; i++) {
        f[nx + i] = f[nx + i] - r->prm.phi_bottom * divdxdy;
        f[(ny - 2) * nx + i] = f[(ny - 2) * nx + i] - r->prm.phi_top * divdxdy;
    }
}
/* FP64 full-multigrid passes of the converged solve: each divides the
 * error by more than 1e3, so 12 reach FP64 rounding at 513^2           */
#define ORC_CONVERGED_PASSES 12
static void apply_walls(orc_run* r, double* phi, double phi_right) {
    const int nx = r->nx, ny = r->ny;
    for (int j = 0; j < ny; j++) { phi[j * nx] = r->prm.phi_left; phi[j * nx + nx - 1] = phi_right; }
    for (int i = 0; i < nx; i++) { phi[i] = r->prm.phi_bottom; phi[(ny - 1) * nx + i] = r->prm.phi_top; }
}
void orc_poisson(orc_run* r, int64_t t) {
    /* PGB_POISSON_FP32_DC and PGB_POISSON_DST_DC approximate the exact
     * discrete solution: their FP64 oracle is that solution (defect
     * correction to convergence)                                        */
    if (r->prm.poisson_mode == PGB_POISSON_FP32_DC || r->prm.poisson_mode == PGB_POISSON_DST_DC) {
        orc_poisson_converged(r, t, ORC_CONVERGED_PASSES);
        return;
    }
    double phi_right = r->prm.phi_right * cos(r->prm.phi_period * (double)t);
    assemble_rhs(r, r->phi, phi_right);
    memcpy(r->rhs, r->phi, sizeof(double) * (size_t)r->nx * r->ny);
    mg_fmg(r, r->phi, r->nx, r->prm.xlength, 2);
    apply_walls(r, r->phi, phi_right);
}

/* max |f - L u| over interior nodes for the interior solution u (zero walls) */
static double residual_max(const double* u, const double* f, int n, double length) {
    double h = length / (n - 1), h2i = 1.0 / (h * h), m = 0.0;
    for (int i = 1; i < n - 1; ++i)
        for (int j = 1; j < n - 1; ++j) {
            double lu = h2i * (u[(i + 1) * n + j] + u[(i - 1) * n + j] + u[i * n + j + 1] + u[i * n + j - 1] - 4.0 * u[i * n + j]);
            double d = fabs(f[i * n + j] - lu);
            if (d > m) m = d;
        }
    return m;
}
void orc_poisson_residual(orc_run* r, double* max_res, double* max_rhs) {
    int n = r->nx;
    size_t G = (size_t)n * n;
    double* u = (double*)malloc(G * sizeof(double));
    memcpy(u, r->phi, G * sizeof(double));
    for (int i = 0; i < n; ++i) { u[i] = 0; u[(n - 1) * n + i] = 0; u[i * n] = 0; u[i * n + n - 1] = 0; }
    double mf = 0.0;
    for (int i = 1; i < n - 1; ++i)
        for (int j = 1; j < n - 1; ++j) if (fabs(r->rhs[i * n + j]) > mf) mf = fabs(r->rhs[i * n + j]);
    *max_res = residual_max(u, r->rhs, n, r->prm.xlength);
    *max_rhs = mf;
    free(u);
}
/* the converged FP64 solution of the same discrete problem */
void orc_poisson_converged(orc_run* r, int64_t t, int iters) {
    int n = r->nx;
    size_t G = (size_t)n * n;
    double phi_right = r->prm.phi_right * cos(r->prm.phi_period * (double)t);
    assemble_rhs(r, r->rhs, phi_right);
    double* u = (double*)calloc(G, sizeof(double));
    double* d = (double*)malloc(G * sizeof(double));
    double h = r->prm.xlength / (n - 1), h2i = 1.0 / (h * h);
    for (int it = 0; it < iters; ++it) {
        for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) {
            if (i == 0 || j == 0 || i == n - 1 || j == n - 1) { d[i * n + j] = 0.0; continue; }
            double lu = h2i * (u[(i + 1) * n + j] + u[(i - 1) * n + j] + u[i * n + j + 1] + u[i * n + j - 1] - 4.0 * u[i * n + j]);
            d[i * n + j] = r->rhs[i * n + j] - lu;
        }
        mg_fmg(r, d, n, r->prm.xlength, 2);
        for (size_t k = 0; k < G; ++k) u[k] += d[k];
    }
    memcpy(r->phi, u, G * sizeof(double));
    apply_walls(r, r->phi, phi_right);
    free(u); free(d);
}

/* fields::grid_electric_field (fields.cpp:230-268), stride-nx layout */
void orc_efield(orc_run* r) {
    const int nx = r->nx, ny = r->ny;
    const double twoDX = 2.0 * r->dx;
    double *Ex = r->ex, *Ey = r->ey;
    const double* phi = r->phi;
    for (int j = 1; j < ny - 1; j++)
        for (int i = 1; i < nx - 1; i++) {
            Ex[j * nx + i] = (phi[j * nx + i - 1] - phi[j * nx + i + 1]) / twoDX;
            Ey[j * nx + i] = (phi[(j - 1) * nx + i] - phi[(j + 1) * nx + i]) / twoDX;
        }
    for (int j = 0; j < ny; j++) {
        Ex[j * nx] = 2.0 * Ex[j * nx + 1] - Ex[j * nx + 2];
        Ex[j * nx + nx - 1] = 2.0 * Ex[j * nx + nx - 2] - Ex[j * nx + nx - 3];
        Ex[j * nx + nx] = 0.0;
    }
    for (int i = 0; i < nx; i++) {
        Ey[i] = 2.0 * Ey[nx + i] - Ey[2 * nx + i];
        Ey[(ny - 1) * nx + i] = 2.0 * Ey[(ny - 2) * nx + i] - Ey[(ny - 3) * nx + i];
        Ey[ny * nx + i] = 0.0;
    }
}

/* ------------------------------------------------------- cross sections */
/* e_collisions.cpp:205-308; a value the reference leaves uninitialised
 * (energy exactly on a branch edge) is taken as 0                          */
static double sigma_ar_elastic(double e) {
    if (e < 0.35)
        return 28019.0 * pow(e, 6.0) - 32798.0 * pow(e, 5.0) + 15048.0 * pow(e, 4.0) - 34312.0 * pow(e, 3.0) +
               4084.0 * pow(e, 2.0) - 249.0 * e + 7.576;
    if (e < 15.0 && e > 0.35) return -0.013 * pow(e, 3.0) + 0.232 * pow(e, 2.0) + 1.066 * e + 0.085;
    if (e > 15.0) return 126.2 * pow(e, -0.69);
    return 0.0;
}
static double sigma_ar_ionize(double e) {
    if (e < 15.755) return 0.0;
    if (e < 100.0 && e > 15.755)
        return (-3.0e-7) * pow(e, 4.0) + (8.0e-5) * pow(e, 3.0) - 0.008 * pow(e, 2.0) + 0.416 * e - 4.758;
    if (e > 100.0) return 130.0 * pow(e, -0.74);
    return 0.0;
}
static double sigma_h_elastic(double e) {
    if (e < 1.0e-2) return 3.834 * pow(e, 2.0) - 20.82 * e + 40.98;
    if (e >= 1.0e-2 && e < 20.0) return -6.15 * log(e) + 20.91;
    if (e >= 20.0) return 102.2 * pow(e, -1.19);
    return 0.0;   /* NaN energy */
}
static double sigma_h_ionize(double e) {
    double I = 13.6, I_E = e / I, C = (1.0 - (1.0 / I_E));
    double A = 0.18450, B1 = -0.032226, B2 = -0.034539, B3 = 1.4003, B4 = -2.8115, B5 = 2.2986;
    if (e < I) return 0.0;
    if (e >= I)
        return (1.0 / (I * e)) * (A * log(I_E) + B1 * C + B2 * pow(C, 2.0) + B3 * pow(C, 3.0) + B4 * pow(C, 4.0) +
                                  B5 * pow(C, 5.0));
    return 0.0;
}
/* ion_collisions.cpp:159-199 (sigma_H_cx rescales its energy argument) */
static double sigma_ar_cx(double e) {
    if (e > 4.0) return (2.0 + 5.5 / sqrt(e)) * 10.0;
    return (-2.95 * sqrt(e) + 10.65) * 10.0;
}
static double sigma_h_cx(double e) {
    double A1 = 3.2345, A2 = 235.88, A3 = 0.038371, A4 = 3.8068e-6, A5 = 1.1832e-10, A6 = 2.3713;
    e = e / 1000.0;
    e = e / C_AMU;
    if (e < 1.0e-4) return 0.0;
    return (A1 * log((A2 / e) + A6)) / (1.0 + A3 * e + A4 * pow(e, 3.5) + A5 * pow(e, 5.4));
}
/* the six energy-dependent fits by PGB_XS_* index (tabulated by the tests) */
double orc_sigma(int which, double e) {
    switch (which) {
        case PGB_XS_AR_ELASTIC: return sigma_ar_elastic(e);
        case PGB_XS_AR_IONIZE: return sigma_ar_ionize(e);
        case PGB_XS_H_ELASTIC: return sigma_h_elastic(e);
        case PGB_XS_H_IONIZE: return sigma_h_ionize(e);
        case PGB_XS_AR_CX: return sigma_ar_cx(e);
        case PGB_XS_H_CX: return sigma_h_cx(e);
        default: return 0.0;
    }
}
static double sigma_el(orc_run* r, double e) {
    if (r->prm.sigma_elastic_mode == PGB_SIGMA_CONSTANT) return r->prm.elastic_sigma_value;
    return r->prm.species == PGB_ARGON ? sigma_ar_elastic(e) : sigma_h_elastic(e);
}
static double sigma_ion(orc_run* r, double e) {
    if (r->prm.sigma_ionization_mode == PGB_SIGMA_CONSTANT) return r->prm.ionization_sigma_value;
    return r->prm.species == PGB_ARGON ? sigma_ar_ionize(e) : sigma_h_ionize(e);
}
static double sigma_cx(orc_run* r, double e) {
    if (r->prm.sigma_cx_mode == PGB_SIGMA_CONSTANT) return r->prm.sigma_value;
    return r->prm.species == PGB_ARGON ? sigma_ar_cx(e) : sigma_h_cx(e);
}

/* ------------------------------------------------------------- collisions */
/* collisions::scattered_velocity (collisions.cpp:107-171), yes_or_no = YES */
static void scattered_velocity(orc_run* r, orc_pv* P, double energy, double coll_factor) {
    const double two_pi = 2.0 * C_PI;
    double R = rng_u01(r), cosChi;
    if (energy < 1.0e-2) cosChi = sqrt(1.0 - R);
    else cosChi = 2.0 * (1.0 - pow((1.0 + energy), R)) / energy + 1.0;
    double sinChi = sqrt(1.0 - cosChi * cosChi);
    double cosPhi = cos(two_pi * R), sinPhi = sin(two_pi * R);
    int index = (int)(rng_int(r) % (uint32_t)(r->prm.init_no_neutrals - 1));
    double nvx = r->neut[0][0][index] * ((double)1), nvy = r->neut[0][1][index] * ((double)1),
           nvz = r->neut[0][2][index] * ((double)1);
    double ux = P->vx - nvx, uy = P->vy - nvy, uz = P->vz - nvz;
    double uperp = sqrt(uy * uy + uz * uz);
    double u = sqrt(ux * ux + uperp * uperp);
    double uyp, uzp;
    if (uperp < 1.0) { uyp = 1.0; uzp = 1.0; }
    else { uyp = uy / uperp; uzp = uz / uperp; }
    P->vz -= coll_factor * (uz * (1.0 - cosChi) - (ux * uzp * cosPhi - u * uyp * sinPhi) * sinChi);
    P->vy -= coll_factor * (uy * (1.0 - cosChi) - (ux * uyp * cosPhi + u * uzp * sinPhi) * sinChi);
    P->vx -= coll_factor * (ux * (1.0 - cosChi) + uperp * cosPhi * sinChi);
}

/* e_collisions::ionization (e_collisions.cpp:319-443).  The excess energy
 * subtracts the threshold in eV from an energy in J (line 377), so it is
 * negative and the three velocities come out NaN, as in the reference.   */
static void ionization(orc_run* r, int64_t i, double reduced_mass) {
    orc_sp* E = &r->sp[0];
    orc_sp* I = &r->sp[1];
    const double me = r->prm.electron_mass, mi = r->prm.ion_mass;
    double weight = E->p[i].w;
    double xe = E->p[i].x, ye = E->p[i].y;
    reduced_mass *= me;
    double R = rng_u01(r);
    double Rxe = 1.0 - 2.0 * (rng_u01(r));
    double Rye = 1.0 - 2.0 * (rng_u01(r));
    double Rze = 1.0 - 2.0 * (rng_u01(r));
    double R2xe = 1.0 - 2.0 * (rng_u01(r));
    double R2ye = 1.0 - 2.0 * (rng_u01(r));
    double R2ze = 1.0 - 2.0 * (rng_u01(r));
    int index = (int)(rng_int(r) % (uint32_t)(r->prm.init_no_neutrals - 1));
    double nvx = r->neut[0][0][index], nvy = r->neut[0][1][index], nvz = r->neut[0][2][index];
    double vxe = E->p[i].vx, vye = E->p[i].vy, vze = E->p[i].vz;
    double Wx = (mi * nvx + me * vxe) / (mi + me);
    double Wy = (mi * nvy + me * vye) / (mi + me);
    double Wz = (mi * nvz + me * vze) / (mi + me);
    double ve = sqrt(vxe * vxe + vye * vye + vze * vze);
    double vn = sqrt(nvx * nvx + nvy * nvy + nvz * nvz);
    double excess = (reduced_mass / 2.0) * (ve - vn) * (ve - vn) - r->prm.threshold;
    double ve_after = sqrt(2.0 * R * excess / me);
    double v2e_after = sqrt(2.0 * (1.0 - R) * excess / me);
    double vxe_after = ve_after * Rxe, vye_after = ve_after * Rye, vze_after = ve_after * Rze;
    double v2xe_after = v2e_after * R2xe, v2ye_after = v2e_after * R2ye, v2ze_after = v2e_after * R2ze;
    double vxi = Wx - (me / mi) * (vxe_after + v2xe_after);
    double vyi = Wy - (me / mi) * (vye_after + v2ye_after);
    double vzi = Wz - (me / mi) * (vze_after + v2ze_after);
    double xi = xe + vxi * r->prm.dti, yi = ye + vyi * r->prm.dti;
    int64_t k = sp_push(I);
    I->p[k].x = xi; I->p[k].y = yi; I->p[k].vx = vxi; I->p[k].vy = vyi; I->p[k].vz = vzi; I->p[k].w = weight;
    vxe_after += Wx; vye_after += Wy; vze_after += Wz;
    v2xe_after += Wx; v2ye_after += Wy; v2ze_after += Wz;
    E->p[i].vx = vxe_after; E->p[i].vy = vye_after; E->p[i].vz = vze_after;
    double x2e = xe + v2xe_after * r->prm.dt, y2e = ye + v2ye_after * r->prm.dt;
    k = sp_push(E);
    E->p[k].x = x2e; E->p[k].y = y2e; E->p[k].vx = v2xe_after; E->p[k].vy = v2ye_after; E->p[k].vz = v2ze_after;
    E->p[k].w = weight;
}

/* e_collisions::collision (e_collisions.cpp:480-597) */
void orc_collide_electrons(orc_run* r) {
    orc_sp* E = &r->sp[0];
    const int nx = r->nx, ny = r->ny;
    const double me = r->prm.electron_mass, mi = r->prm.ion_mass;
    const double dt = r->prm.dt, nd = r->prm.neutral_density;
    const double reduced_mass = mi / (me + mi);
    const int64_t particle_no = E->n;
    for (int64_t i = 0; i < particle_no; ++i) {
        int jp = cell(E->p[i].x / r->dx), kp = cell(E->p[i].y / r->dy);
        if (!(jp >= 0 && jp < nx && kp >= 0 && kp < ny)) continue;
        rng_begin(r, E->id[i], PGB_STREAM_EMCC, 0);
        double vx = E->p[i].vx, vy = E->p[i].vy, vz = E->p[i].vz;
        double u2 = vx * vx + vy * vy + vz * vz;
        double energy = (0.5 / C_CHARGE) * me * u2;
        double u = sqrt((2.0 * C_CHARGE * energy) / me);
        double s_el = sigma_el(r, energy);
        double s_io = sigma_ion(r, energy);
        double R = rng_u01(r);
        double prob = 1.0 - exp(-(u * dt * 1.0e-20 * nd * s_el));
        if (prob > 2.0 * R) {
            scattered_velocity(r, &E->p[i], energy, reduced_mass);
            r->c.elastic++;
        }
        prob = 1.0 - exp(-(u * dt * 1.0e-20 * nd * s_io));
        if (prob > 0.0) {
            rng_begin(r, E->id[i], PGB_STREAM_IONIZE, 0);
            ionization(r, i, reduced_mass);
            r->c.ionization++;
        }
    }
}

/* ion_collisions::collision (ion_collisions.cpp:255-308) with
 * charge_exchange_velocity (ion_collisions.cpp:209-221)                  */
void orc_collide_ions(orc_run* r) {
    orc_sp* I = &r->sp[1];
    const int nx = r->nx, ny = r->ny;
    const double mi = r->prm.ion_mass, dt = r->prm.dti, nd = r->prm.neutral_density;
    const int64_t particle_no = I->n;
    for (int64_t i = 0; i < particle_no; ++i) {
        int jp = cell(I->p[i].x / r->dx), kp = cell(I->p[i].y / r->dy);
        if (!(jp >= 0 && jp < nx && kp >= 0 && kp < ny)) continue;
        double vx = I->p[i].vx, vy = I->p[i].vy, vz = I->p[i].vz;
        double u2 = vx * vx + vy * vy + vz * vz;
        double energy = (0.5 / C_CHARGE) * mi * u2;
        double u = sqrt((2.0 * C_CHARGE * energy) / mi);
        double s = sigma_cx(r, energy);
        r->prob_cx[jp] += (1.0 - exp(-(u * dt * 1.0e-20 * nd * s)));
        if (r->prob_cx[jp] > 1.0) {
            rng_begin(r, I->id[i], PGB_STREAM_CX, 1);
            (void)rng_u01(r);
            int index = (int)(rng_int(r) % (uint32_t)(r->prm.init_no_neutrals - 1));
            I->p[i].vx = r->neut[1][0][index];
            I->p[i].vy = r->neut[1][1][index];
            I->p[i].vz = r->neut[1][2][index];
            r->c.charge_exchange++;
            r->prob_cx[jp] = 0.0;
        }
    }
}

/* particle::inject_more_particles (particle.cpp:491-510), electrons then
 * ions (pic.cpp:1080-1083); the weight is never set and stays 0.0        */
void orc_inject(orc_run* r) {
    for (int s = 0; s < 2; ++s) {
        orc_sp* S = &r->sp[s];
        for (int k = 0; k < r->prm.number_to_inject; ++k) {
            int64_t i = sp_push(S);
            rng_begin(r, S->id[i], PGB_STREAM_INJECT, s);
            double rx = rng_u01(r);
            double ry = rng_u01(r);
            S->p[i].x = (r->dx + rx * (r->prm.xlength - 2.0 * r->dx));
            S->p[i].y = (r->dy + ry * (r->prm.ylength - 2.0 * r->dy));
            S->p[i].vx = maxwell_component(r, S->vt);
            S->p[i].vy = maxwell_component(r, S->vt);
            S->p[i].vz = maxwell_component(r, S->vt);
            if (s == 0) r->c.injected_e++; else r->c.injected_i++;
        }
    }
}

/* --------------------------------------------------------------- walls */
typedef struct {
    double energy, angleX, angleY, yield, refl, back;
    int onX;
} wall_state;

/* boundary::calc_energy / calc_angleX / calc_angleY (boundary.cpp:186-220) */
static void wall_energy(wall_state* w, double m, double vx, double vy, double vz) {
    double u2 = vx * vx + vy * vy + vz * vz;
    w->energy = (0.5 / C_CHARGE) * m * u2;
    double uu = 2.0 * w->energy / m;
    w->angleX = acos(vx / (sqrt(uu) + 1.0e-6));
    w->angleY = acos(vy / (sqrt(uu) + 1.0e-6));
}
/* boundary::e_impact_see_yield_v (boundary.cpp:281-300) */
static void see_yield(orc_run* r, wall_state* w) {
    if (!r->prm.e_impact_see) { w->yield = 0.0; return; }
    double twoPi = 2.0 * C_PI, E0 = r->prm.see_e0, Emax0 = r->prm.see_emax0, my = r->prm.see_max_yield;
    double v = (w->energy - E0) / (Emax0 - E0);
    double k = (v > 1) ? 0.25 : 0.62;
    double a = w->onX ? w->angleX : w->angleY;
    double ww = (w->energy - E0) / (Emax0 * (1.0 + k * (a * a / twoPi)) - E0);
    w->yield = my * (1.0 + k * (a * a / twoPi)) * pow((ww * exp((1.0 - ww))), k);
}
/* boundary::calc_reflection_yield_v / calc_backscatter_yield_v (boundary.cpp:323-337) */
static void refl_back_yields(orc_run* r, wall_state* w) {
    w->refl = 0.0;
    if (r->prm.reflection && w->energy > 50.0) w->refl = 0.1 * w->yield;
    w->back = 0.0;
    if (r->prm.backscatter && w->energy > 50.0) w->back = 0.1 * w->yield;
}

/* boundary::reflect_electron (boundary.cpp:374-417) */
static void reflect_electron(orc_run* r, orc_pv* P) {
    const int nx = r->nx, ny = r->ny;
    const double dt = r->prm.dt;
    const double lengthX = r->dx * nx, lengthY = r->dy * ny;
    double R = rng_u01(r);
    int jp = cell(P->x / r->dx), kp = cell(P->y / r->dy);
    if (jp >= nx) { P->vx = -P->vx; P->x = lengthX - R * dt * fabs(P->vx); }
    else if (jp < 0) { P->vx = -P->vx; P->x = R * dt * fabs(P->vx); }
    if (kp >= ny) { P->vy = -P->vy; P->y = lengthY - R * dt * fabs(P->vy); }
    else if (kp < 0) { P->vy = -P->vy; P->y = R * dt * fabs(P->vy); }
}
/* boundary::secondary_vel (boundary.cpp:427-486) */
static void secondary_vel(orc_run* r, orc_pv* P, double velocity) {
    const int nx = r->nx, ny = r->ny;
    const double dt = r->prm.dt;
    const double lengthX = r->dx * nx, lengthY = r->dy * ny;
    int jp = cell(P->x / r->dx), kp = cell(P->y / r->dy);
    if (jp < 0 || jp >= nx) {
        double R = rng_u01(r), Rphi = rng_u01(r), Rchi = rng_u01(r);
        double chi = asin(sqrt(Rchi)), phi = 2.0 * C_PI * Rphi;
        P->vx = fabs(velocity * cos(chi));
        P->vy = velocity * sin(chi) * cos(phi);
        P->vz = velocity * sin(chi) * sin(phi);
        P->x = R * dt * fabs(P->vx);
        if (jp >= nx) { P->x = lengthX - P->x; P->vx = -fabs(velocity * cos(chi)); }
    }
    if (kp < 0 || kp >= ny) {
        double R = rng_u01(r), Rphi = rng_u01(r), Rchi = rng_u01(r);
        double chi = asin(sqrt(Rchi)), phi = 2.0 * C_PI * Rphi;
        P->vy = fabs(velocity * cos(chi));
        P->vx = velocity * sin(chi) * cos(phi);
        P->vz = velocity * sin(chi) * sin(phi);
        P->y = R * dt * fabs(P->vy);
        if (kp >= ny) { P->y = lengthY - P->y; P->vy = -fabs(velocity * cos(chi)); }
    }
}
/* boundary::secondary_electrons (boundary.cpp:494-529): the new electron
 * takes the incident x on a left/right wall, else the incident y; the other
 * coordinate stays 0.0                                                     */
static int64_t secondary_electron(orc_run* r, int64_t inc) {
    orc_sp* E = &r->sp[0];
    int jp = cell(E->p[inc].x / r->dx);
    int64_t k = sp_push(E);
    E->p[k].w = 1.0;
    E->p[k].w = E->p[inc].w;
    if (jp < 0 || jp >= r->nx) E->p[k].x = E->p[inc].x;
    else E->p[k].y = E->p[inc].y;
    if (r->rng_mode == ORC_RNG_PHILOX) rng_begin(r, E->id[k], PGB_STREAM_SEE, 0);
    double R = rng_u01(r);
    double velocity = sqrt((2.0 * R * C_CHARGE * (r->prm.threshold - 2.0 * r->prm.work_function) / r->prm.electron_mass));
    secondary_vel(r, &E->p[k], velocity);
    r->c.see_emitted++;
    return k;
}

static int outside(orc_run* r, const orc_pv* P) {
    int jp = cell(P->x / r->dx), kp = cell(P->y / r->dy);
    return jp < 0 || jp >= r->nx || kp < 0 || kp >= r->ny;
}

/* One wall interaction of electron i (boundary.cpp:599-668).  Returns 0 if
 * the electron stays (reflected or backscattered), 1 if absorbed, 2 if it
 * was replaced by secondaries, -1 if no branch fired (the reference then
 * examines the same electron again).  *first/*count give the secondaries. */
static int e_wall_event(orc_run* r, int64_t i, int64_t* nsec) {
    orc_sp* E = &r->sp[0];
    wall_state w;
    int jp = cell(E->p[i].x / r->dx);
    w.onX = (jp < 0 || jp >= r->nx);
    wall_energy(&w, r->prm.electron_mass, E->p[i].vx, E->p[i].vy, E->p[i].vz);
    see_yield(r, &w);
    double R = rng_u01(r);
    if (R < w.yield) {
        refl_back_yields(r, &w);
        int no_inject = (int)floor(fabs((w.yield - w.refl - w.back))) + 1;
        const double offset = 1.0e-6;
        R = rng_u01(r);
        if (R < w.refl / (w.yield + offset)) {
            reflect_electron(r, &E->p[i]);
            r->c.reflected++;
            return 0;
        } else if (R > w.refl / w.yield && R < (w.refl + w.back) / (w.yield + offset)) {
            double R3 = (double)(rng_int(r) % 10000) / 10000.0;
            double velocity = R3 * sqrt((2.0 * C_CHARGE * w.energy) / r->prm.electron_mass);
            secondary_vel(r, &E->p[i], velocity);
            r->c.backscattered++;
            return 0;
        } else if (R > (w.refl + w.back) / (w.yield + offset)) {
            *nsec = no_inject;
            r->c.see_events++;
            return 2;
        }
        return -1;
    }
    r->c.absorbed_e++;
    return 1;
}

/* boundary::e_boundary (boundary.cpp:581-677) */
static void e_boundary(orc_run* r) {
    orc_sp* E = &r->sp[0];
    if (r->order_mode == ORC_ORDER_REF) {
        int64_t i = 0, n = E->n;
        while (i < n) {
            if (outside(r, &E->p[i])) {
                int64_t nsec = 0;
                int res = e_wall_event(r, i, &nsec);
                if (res == 0) i++;
                else if (res == 1) sp_swap_pop(E, i);
                else if (res == 2) {
                    for (int64_t j = 0; j < nsec; ++j) secondary_electron(r, i);
                    sp_swap_pop(E, i);
                }
            } else {
                i++;
            }
            n = E->n;
        }
        return;
    }
    /* stable order: walk the electrons present at entry; secondaries are
     * appended and the incident electron is removed                       */
    int64_t n0 = E->n, nd = 0;
    int64_t* dl = NULL;
    for (int64_t i = 0; i < n0; ++i) {
        if (!outside(r, &E->p[i])) continue;
        rng_begin(r, E->id[i], PGB_STREAM_EWALL, 0);
        int res = -1;
        int64_t nsec = 0;
        for (int attempt = 0; attempt < 64 && res == -1; ++attempt) res = e_wall_event(r, i, &nsec);
        if (res == -1) { r->c.absorbed_e++; res = 1; }
        if (res == 2)
            for (int64_t j = 0; j < nsec; ++j) secondary_electron(r, i);
        if (res == 1 || res == 2) {
            dl = (int64_t*)realloc(dl, sizeof(int64_t) * (size_t)(nd + 1));
            dl[nd++] = i;
        }
    }
    if (nd) {
        unsigned char* dead = (unsigned char*)calloc((size_t)E->n + 1, 1);
        for (int64_t k = 0; k < nd; ++k) dead[dl[k]] = 1;
        sp_compact(E, dead);
        free(dead);
    }
    free(dl);
}

/* boundary::i_impact_see_yield_Ar (boundary.cpp:310-317) */
static double ion_see_yield(orc_run* r, double energy) {
    if (!(r->prm.species == PGB_ARGON && r->prm.ion_impact_see)) return 0.0;
    double y = 0.0;
    if (energy >= 80.0)
        y = 0.006 * energy / (1.0 + (energy / 10.0)) + 1.05e-4 * (sqrt((energy - 80.0)) / (1.0 + pow((energy / 8000.0), 1.5)));
    return y;
}
/* boundary::i_secondary_vel (boundary.cpp:687-756) */
static void i_secondary_vel(orc_run* r, int64_t k, double x, double y, double weight) {
    orc_sp* E = &r->sp[0];
    const int nx = r->nx, ny = r->ny;
    const double dt = r->prm.dt;
    const double lengthX = r->dx * nx, lengthY = r->dy * ny;
    int jp = cell(x / r->dx), kp = cell(y / r->dy);
    orc_pv* P = &E->p[k];
    if (jp < 0 || jp >= nx) {
        double R = rng_u01(r);
        double velocity = sqrt((2.0 * R * C_CHARGE * (r->prm.threshold - 2.0 * r->prm.work_function) / r->prm.electron_mass));
        double Rphi = rng_u01(r), Rchi = rng_u01(r);
        double chi = asin(sqrt(Rchi)), phi = 2.0 * C_PI * Rphi;
        P->vx = fabs(velocity * cos(chi));
        P->vy = velocity * sin(chi) * cos(phi);
        P->vz = velocity * sin(chi) * sin(phi);
        P->w = weight;
        P->x = R * dt * fabs(P->vx);
        if (jp >= nx) { P->x = lengthX - P->x; P->vx = -fabs(velocity * cos(chi)); }
    }
    if (kp < 0 || kp >= ny) {
        double R = rng_u01(r);
        double velocity = sqrt((2.0 * R * C_CHARGE * (r->prm.threshold - 2.0 * r->prm.work_function) / r->prm.electron_mass));
        double Rphi = rng_u01(r), Rchi = rng_u01(r);
        double chi = asin(sqrt(Rchi)), phi = 2.0 * C_PI * Rphi;
        P->vy = fabs(velocity * cos(chi));
        P->vx = velocity * sin(chi) * cos(phi);
        P->vz = velocity * sin(chi) * sin(phi);
        P->w = weight;
        P->y = R * dt * fabs(P->vy);
        if (kp >= ny) { P->y = lengthY - P->y; P->vy = -fabs(velocity * cos(chi)); }
    }
}

/* boundary::ion_boundary (boundary.cpp:765-824) */
static void ion_boundary(orc_run* r) {
    orc_sp* I = &r->sp[1];
    orc_sp* E = &r->sp[0];
    int64_t n0 = I->n;
    unsigned char* dead = r->order_mode == ORC_ORDER_STABLE ? (unsigned char*)calloc((size_t)n0 + 1, 1) : NULL;
    int64_t i = 0, n = I->n;
    while (i < (r->order_mode == ORC_ORDER_REF ? n : n0)) {
        if (!outside(r, &I->p[i])) { i++; continue; }
        rng_begin(r, I->id[i], PGB_STREAM_IWALL, 1);
        double vx = I->p[i].vx, vy = I->p[i].vy, vz = I->p[i].vz;
        double energy = (0.5 / C_CHARGE) * r->prm.ion_mass * (vx * vx + vy * vy + vz * vz);
        double yield = ion_see_yield(r, energy);
        double R = rng_u01(r);
        if (R < yield) {
            int no_inject = (int)floor(yield) + 1;
            for (int j = 0; j < no_inject; ++j) {
                int64_t k = sp_push(E);
                E->p[k].w = 1.0;
                if (r->rng_mode == ORC_RNG_PHILOX) rng_begin(r, E->id[k], PGB_STREAM_SEE, 0);
                i_secondary_vel(r, k, I->p[i].x, I->p[i].y, I->p[i].w);
                r->c.ion_see_emitted++;
            }
        }
        r->c.absorbed_i++;
        if (r->order_mode == ORC_ORDER_REF) {
            sp_swap_pop(I, i);
            n = I->n;
        } else {
            dead[i] = 1;
            i++;
        }
    }
    if (dead) { sp_compact(I, dead); free(dead); }
}

/* boundary::plop_particles (boundary.cpp:854-878) */
static void plop(orc_run* r, orc_pv* e, orc_pv* ion) {
    double rx = rng_u01(r), ry = rng_u01(r);
    e->x = (r->dx + rx * (r->prm.xlength - 2.0 * r->dx));
    ion->x = (r->dx + rx * (r->prm.xlength - 2.0 * r->dx));
    e->y = (r->dy + ry * (r->prm.ylength - 2.0 * r->dy));
    ion->y = (r->dy + ry * (r->prm.ylength - 2.0 * r->dy));
    e->vx = maxwell_component(r, r->prm.vte);
    ion->vx = maxwell_component(r, r->prm.vti);
    e->vy = maxwell_component(r, r->prm.vte);
    ion->vy = maxwell_component(r, r->prm.vti);
    e->vz = maxwell_component(r, r->prm.vte);
    ion->vz = maxwell_component(r, r->prm.vti);
}
/* boundary::steadyBoundaryX / steadyBoundaryY (boundary.cpp:890-1082):
 * the j-th outside electron at a wall is paired with the j-th outside ion
 * at the same wall, in array order, while both last.  axis 0 = x, 1 = y.  */
static void steady_axis(orc_run* r, int axis) {
    orc_sp* E = &r->sp[0];
    orc_sp* I = &r->sp[1];
    const int nc = axis == 0 ? r->nx : r->ny;
    const double d = axis == 0 ? r->dx : r->dy;
    int64_t n = E->n, n_ion = I->n;
    int64_t cnt_lo = 0, cnt_hi = 0;
    for (int64_t i = 0; i < n; ++i) {
        double c = axis == 0 ? E->p[i].x : E->p[i].y;
        int jp = cell(c / d);
        if (c < 0.0) cnt_lo++;
        else if (jp >= nc) cnt_hi++;
    }
    int64_t left_lo = (int64_t)(1.0 * (double)cnt_lo), left_hi = (int64_t)(1.0 * (double)cnt_hi);
    int64_t klast_lo = 0, klast_hi = 0, i = 0;
    while (i < n) {
        double c = axis == 0 ? E->p[i].x : E->p[i].y;
        int jp = cell(c / d);
        if (c < 0.0 || jp >= nc) {
            int lo = c < 0.0;
            int64_t k = lo ? klast_lo : klast_hi, i_before = i;
            int64_t* left = lo ? &left_lo : &left_hi;
            while (*left > 0 && k < n_ion) {
                double ci = axis == 0 ? I->p[k].x : I->p[k].y;
                int hit = lo ? (ci < 0.0) : (cell(ci / d) >= nc);
                if (hit) {
                    rng_begin(r, E->id[i], PGB_STREAM_PLOP, 0);
                    plop(r, &E->p[i], &I->p[k]);
                    (*left)--;
                    i++;
                    r->c.plopped++;
                    break;
                }
                k++;
            }
            if (lo) klast_lo = k + 1; else klast_hi = k + 1;
            if (i == i_before) i++;
        } else {
            i++;
        }
    }
}

void orc_boundary(orc_run* r, int which) {
    if (which == PGB_BOUNDARY_IONS) {
        if (!r->prm.steadystate) ion_boundary(r);   /* steady_i_boundary is empty (boundary.cpp:1099-1103) */
    } else {
        if (r->prm.steadystate) { steady_axis(r, 0); steady_axis(r, 1); }   /* boundary.cpp:1094-1097 */
        else e_boundary(r);
    }
}

/* -------------------------------------------------- population control */
static int vgroup(const double* vlim, int ng, double vxy) {
    int g = 0;
    while (g < ng - 1 && vxy > vlim[g]) g++;
    return g;
}
typedef struct { uint32_t key, id; int64_t idx; } orc_prio;
static int prio_cmp(const void* a, const void* b) {
    const orc_prio* x = (const orc_prio*)a;
    const orc_prio* y = (const orc_prio*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    if (x->id != y->id) return x->id < y->id ? -1 : 1;
    return 0;
}
/* particle::contain_particle_growth + reduce_population (particle.cpp:520-653).
 * REF order: the reference's sequential random removal with rand().
 * STABLE order: in each over-full group the Nremove particles with the
 * smallest Philox priority (ties by id) are removed, then the survivors of
 * the group are re-weighted by Ngroup/(Ngroup-Nremove).                   */
void orc_contain_growth(orc_run* r, int spi) {
    orc_sp* S = &r->sp[spi];
    int64_t size_to_check = spi == 0 ? r->prm.size_to_check_e : r->prm.size_to_check_i;
    if (!(S->n > size_to_check)) return;
    const int ng = r->prm.no_groups;
    const double* vlim = spi == 0 ? r->prm.v_limit_e : r->prm.v_limit_i;
    const int32_t* glim = spi == 0 ? r->prm.group_limit_e : r->prm.group_limit_i;
    const int32_t* gnew = spi == 0 ? r->prm.new_group_size_e : r->prm.new_group_size_i;
    int64_t Ngroup[3] = {0, 0, 0}, Nremove[3] = {0, 0, 0}, jgroup[3] = {0, 0, 0};
    double gw[3] = {1.0, 1.0, 1.0};
    for (int64_t i = 0; i < S->n; ++i) {
        double vxy = sqrt((S->p[i].vx) * (S->p[i].vx) + (S->p[i].vy) * (S->p[i].vy));
        Ngroup[vgroup(vlim, ng, vxy)] += 1;
    }
    int64_t to_remove = 0;
    for (int g = 0; g < ng; ++g) {
        if (Ngroup[g] > glim[g]) Nremove[g] = Ngroup[g] - gnew[g];
        to_remove += Nremove[g];
    }
    if (r->order_mode == ORC_ORDER_REF) {
        int64_t i = 0;
        while (i < to_remove) {
            int64_t R = (int64_t)((uint32_t)rand() % (uint64_t)(S->n - 1));
            double vxy = sqrt((S->p[R].vx) * (S->p[R].vx) + (S->p[R].vy) * (S->p[R].vy));
            int g = vgroup(vlim, ng, vxy);
            if (jgroup[g] < Nremove[g]) { jgroup[g]++; sp_swap_pop(S, R); i++; }
        }
    } else if (to_remove > 0) {
        unsigned char* dead = (unsigned char*)calloc((size_t)S->n + 1, 1);
        for (int g = 0; g < ng; ++g) {
            if (Nremove[g] <= 0) continue;
            orc_prio* pr = (orc_prio*)malloc(sizeof(orc_prio) * (size_t)Ngroup[g]);
            int64_t m = 0;
            for (int64_t i = 0; i < S->n; ++i) {
                double vxy = sqrt((S->p[i].vx) * (S->p[i].vx) + (S->p[i].vy) * (S->p[i].vy));
                if (vgroup(vlim, ng, vxy) != g) continue;
                pgb_stream st;
                pgb_stream_init(&st, r->prm.seed, S->id[i], r->rng_step, PGB_STREAM_REDUCE, (uint32_t)spi);
                pr[m].key = pgb_stream_u32(&st); pr[m].id = S->id[i]; pr[m].idx = i; ++m;
            }
            qsort(pr, (size_t)m, sizeof(orc_prio), prio_cmp);
            for (int64_t k = 0; k < Nremove[g] && k < m; ++k) dead[pr[k].idx] = 1;
            jgroup[g] = Nremove[g] < m ? Nremove[g] : m;
            free(pr);
        }
        sp_compact(S, dead);
        free(dead);
    }
    if (to_remove > 0) {
        for (int g = 0; g < ng; ++g)
            if (jgroup[g] > 0) gw[g] = (double)Ngroup[g] / ((double)(Ngroup[g] - jgroup[g]));
        for (int64_t i = 0; i < S->n; ++i) {
            double vxy = sqrt((S->p[i].vx) * (S->p[i].vx) + (S->p[i].vy) * (S->p[i].vy));
            S->p[i].w = (S->p[i].w) * gw[vgroup(vlim, ng, vxy)];
        }
    }
    if (spi == 0) r->c.reductions_e++; else r->c.reductions_i++;
}

/* The library keeps a position as a signed 32-bit fixed-point number of
 * cells with ps fraction bits (pgb_pos_shift of the grid), saturated at
 * +-2^30 units; NaN is its own code.  These restate that rounding where the
 * oracle must decide as the library decides (bin order, plot pixels).    */
#define LIB_POS_NAN INT64_MIN
static int64_t lib_fixed(double x, double d, int ps) {
    double c = x / d;
    if (c != c) return LIB_POS_NAN;
    double v = ldexp(c, ps);
    v = v < -1073741824.0 ? -1073741824.0 : (v > 1073741824.0 ? 1073741824.0 : v);
    return (int64_t)nearbyint(v);
}
/* (int)(x/DX) of a fixed-point position: toward zero, INT_MIN for NaN */
static int lib_cell(int64_t v, int ps) {
    if (v == LIB_POS_NAN) return INT_MIN;
    return v >= 0 ? (int)(v >> ps) : -(int)((-v) >> ps);
}
/* A position in FP32 cells as the library plots it: x/DX rounded to its
 * fixed-point grid of 2^-ps of a cell (saturated at +-2^30 units), then to
 * FP32 (the library keeps positions in that fixed point).              */
static float plot_cells(double x, double d, int ps) {
    int64_t v = lib_fixed(x, d, ps);
    return v == LIB_POS_NAN ? (float)(x / d) : (float)ldexp((double)v, -ps);
}
static int lib_shift(const orc_run* r) {   /* the library's fraction bits for this grid (pgb_pos_shift) */
    int cells = (r->nx > r->ny ? r->nx : r->ny) - 1, b = 0;
    while ((1 << b) < cells) ++b;
    int ps = 29 - b;
    return ps > 23 ? 23 : (ps < 8 ? 8 : ps);
}

/* Stable sort of a species by spatial bin, as the CUDA library orders its
 * particle slots (electrons every sort_interval steps, ions every
 * PGB_ION_SORT_FACTOR * sort_interval; bins of 32x32 cells inside the
 * deposit region of pic.cl:35, then everything else).  Only the order
 * changes; it matters for the order-dependent rules (charge-exchange
 * accumulation, wall lists).                                              */
static int64_t* g_sort_keys;
static int key_cmp(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    int64_t kx = g_sort_keys[x], ky = g_sort_keys[y];
    if (kx != ky) return kx < ky ? -1 : 1;
    return x < y ? -1 : (x > y);
}
static void orc_sort_bins(orc_run* r, int spi) {
    orc_sp* S = &r->sp[spi];
    const int nx = r->nx, ny = r->ny, BIN = 32;
    const int nbx = (nx - 1 + BIN - 1) / BIN, nby = (ny - 1 + BIN - 1) / BIN, nbins = nbx * nby;
    const int ps = lib_shift(r);
    int64_t n = S->n;
    if (n == 0) return;
    int64_t* keys = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        /* the library classifies its fixed-point positions (2^-ps of a cell) */
        int64_t xf = lib_fixed(S->p[i].x, r->dx, ps), yf = lib_fixed(S->p[i].y, r->dy, ps);
        int jp = lib_cell(xf, ps), kp = lib_cell(yf, ps);
        keys[i] = (jp < nx - 1 && xf > 0 && kp < ny - 1 && yf > 0) ? (kp / BIN) * nbx + jp / BIN : nbins;
        idx[i] = i;
    }
    g_sort_keys = keys;
    qsort(idx, (size_t)n, sizeof(int64_t), key_cmp);
    orc_pv* p2 = (orc_pv*)malloc(sizeof(orc_pv) * (size_t)n);
    uint32_t* id2 = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
    for (int64_t k = 0; k < n; ++k) { p2[k] = S->p[idx[k]]; id2[k] = S->id[idx[k]]; }
    memcpy(S->p, p2, sizeof(orc_pv) * (size_t)n);
    memcpy(S->id, id2, sizeof(uint32_t) * (size_t)n);
    free(keys); free(idx); free(p2); free(id2);
    (void)nby;
}

/* ------------------------------------------------------------- driver */
/* pic::pic_run, the two boundary calls ahead of the loop (pic.cpp:1049-1057) */
void orc_initial_boundary(orc_run* r) {
    r->rng_step = 0xFFFFFFFFu;
    orc_boundary(r, PGB_BOUNDARY_IONS);
    orc_boundary(r, PGB_BOUNDARY_ELECTRONS);
}

/* ------------------------------------------------------------- graphs */
/* The value sum_av_dist sees as `spread`: graphs.cpp:865 passes &spread
 * (an int) with sizeof(cl_double), so the kernel reads spread in the low
 * word and the next member, dist_locationX (graphs.h:281-282), in the high
 * word of a little-endian double.                                         */
static double gr_kernel_spread(const pgb_graphs_params* g) {
    uint64_t bits = ((uint64_t)(uint32_t)g->dist_location_x << 32) | (uint32_t)g->spread;
    double d;
    memcpy(&d, &bits, sizeof d);
    return d;
}

/* vbin = (int)((v / vt) * divide_bins_by); counted when |vbin| <= half
 * (pic.cl:218-221).  A value outside the int range is not counted.       */
static void gr_bin(double* d, double v, double vt, double dbb, int half) {
    double b = (v / vt) * dbb;
    if (!(b > -2147483649.0 && b < 2147483648.0)) return;
    int vbin = (int)b;
    if (abs(vbin) <= half) d[vbin + half] += 1.0;
}

int orc_graphs_enable(orc_run* r, const pgb_graphs_params* g) {
    if (!g || g->no_bins < 1 || (g->no_bins & 1) == 0 || g->no_graph_steps < 1) return PGB_ERR_ARG;
    const size_t G = (size_t)r->nx * r->ny;
    r->gr = *g;
    for (int k = 0; k < 4; ++k) { free(r->gr_f[k]); r->gr_f[k] = (double*)calloc(G, sizeof(double)); }
    for (int s = 0; s < 2; ++s) {
        free(r->gr_q[s]); r->gr_q[s] = (double*)calloc(G, sizeof(double));
        free(r->gr_v[s][0]); r->gr_v[s][0] = (double*)calloc((size_t)r->nx, sizeof(double));
        free(r->gr_v[s][1]); r->gr_v[s][1] = (double*)calloc((size_t)r->ny, sizeof(double));
        for (int k = 0; k < 4; ++k) { free(r->gr_d[s][k]); r->gr_d[s][k] = (double*)calloc((size_t)g->no_bins, sizeof(double)); }
    }
    r->gr_on = 1;
    return 0;
}

/* one graph step: graphs::sum_fields, then per species sum_density,
 * sum_av_velocities and sum_av_dist (pic.cpp:1189-1207, graphs.cpp:412-985,
 * pic.cl:154-251), particles in storage order                           */
static void orc_graphs_accumulate(orc_run* r) {
    const int nx = r->nx, ny = r->ny;
    const int64_t G = (int64_t)nx * ny;
    for (int64_t k = 0; k < G; ++k) {
        r->gr_f[0][k] += r->rho[k];
        r->gr_f[1][k] += r->phi[k];
        r->gr_f[2][k] += r->ex[k];   /* EgridX[j*nx+i]: stride nx */
        r->gr_f[3][k] += r->ey[k];
    }
    const pgb_graphs_params* g = &r->gr;
    const double sp = gr_kernel_spread(g);
    const double l1 = g->dist_location_x, l2 = g->dist_location2_x;
    const double l3 = g->dist_location_y, l4 = g->dist_location2_y;
    const double dbb = (double)g->divide_bins_by;
    const int half = (g->no_bins - 1) / 2;
    double* vx_t = (double*)calloc((size_t)nx, sizeof(double));
    double* cx_t = (double*)calloc((size_t)nx, sizeof(double));
    double* vy_t = (double*)calloc((size_t)ny, sizeof(double));
    double* cy_t = (double*)calloc((size_t)ny, sizeof(double));
    for (int s = 0; s < 2; ++s) {
        const double qc = s == 0 ? -C_CHARGE : C_CHARGE;   /* ELECTRON_CHARGE, CHARGE */
        for (int64_t k = 0; k < G; ++k) r->gr_q[s][k] += r->q[s][k] / qc;
        const orc_sp* S = &r->sp[s];
        memset(vx_t, 0, (size_t)nx * sizeof(double)); memset(cx_t, 0, (size_t)nx * sizeof(double));
        memset(vy_t, 0, (size_t)ny * sizeof(double)); memset(cy_t, 0, (size_t)ny * sizeof(double));
        const int xv = nx / 2, yv = ny / 2;   /* sum_av_velocities (pic.cl:161-162) */
        const int xd = ny / 2, yd = ny / 2;   /* sum_av_dist (pic.cl:202-203)      */
        for (int64_t i = 0; i < S->n; ++i) {
            const orc_pv* p = &S->p[i];
            const int jp = cell(p->x / r->dx), kp = cell(p->y / r->dy);
            /* jp, kp >= 0: a position beyond the int range gives INT_MIN */
            if (jp >= 0 && jp < nx && p->x > 0.0 && kp == yv) { vx_t[jp] += p->vx; cx_t[jp] += 1.0; }
            if (jp == xv && kp >= 0 && kp < ny && p->y > 0.0) { vy_t[kp] += p->vy; cy_t[kp] += 1.0; }
            if (jp >= (l1 - sp) && p->x > 0.0 && jp <= (l1 + sp) && jp < nx && kp == yd)
                gr_bin(r->gr_d[s][0], p->vx, S->vt, dbb, half);
            if (jp >= (l2 - sp) && p->x > 0.0 && jp <= (l2 + sp) && jp < nx && kp == yd)
                gr_bin(r->gr_d[s][2], p->vx, S->vt, dbb, half);
            if (kp >= (l3 - sp) && p->y > 0.0 && kp <= (l3 + sp) && kp < ny && jp == xd)
                gr_bin(r->gr_d[s][1], p->vy, S->vt, dbb, half);
            if (kp >= (l4 - sp) && p->y > 0.0 && kp <= (l4 + sp) && kp < ny && jp == xd)
                gr_bin(r->gr_d[s][3], p->vy, S->vt, dbb, half);
        }
        for (int j = 0; j < nx; ++j)
            if (cx_t[j] > 0.5) r->gr_v[s][0][j] += vx_t[j] / cx_t[j];
        for (int j = 0; j < ny; ++j)
            if (cy_t[j] > 0.5) r->gr_v[s][1][j] += vy_t[j] / cy_t[j];
    }
    free(vx_t); free(cx_t); free(vy_t); free(cy_t);
}

/* running maximum that starts from element `first` (graphs.cpp:1002-1028,
 * 1093-1104)                                                             */
static double gr_max(const double* sum, int64_t n, int64_t first, double steps) {
    double m = sum[first] / steps;
    for (int64_t k = 0; k < n; ++k) {
        double v = sum[k] / steps;
        if (m < v) m = v;
    }
    return m;
}

/* averages of graphs::average_fields / _density / _velocities / _dist1/2
 * (graphs.cpp:1000-1155)                                                 */
int orc_graphs_get(orc_run* r, int which, int species, double* out, int64_t n) {
    if (!r->gr_on || species < 0 || species > 1) return PGB_ERR_ARG;
    const int64_t G = (int64_t)r->nx * r->ny;
    const double steps = (double)r->gr.no_graph_steps;
    const double* src = NULL;
    int64_t cnt = G;
    double div = steps;
    switch (which) {
        case PGB_GRAPH_RHO: case PGB_GRAPH_PHI: case PGB_GRAPH_EX: case PGB_GRAPH_EY:
            src = r->gr_f[which]; break;
        case PGB_GRAPH_DENSITY: src = r->gr_q[species]; break;
        case PGB_GRAPH_VX: src = r->gr_v[species][0]; cnt = r->nx; div = r->prm.vte * steps; break;
        case PGB_GRAPH_VY: src = r->gr_v[species][1]; cnt = r->ny; div = r->prm.vte * steps; break;
        case PGB_GRAPH_DIST_X1: case PGB_GRAPH_DIST_Y1: case PGB_GRAPH_DIST_X2: case PGB_GRAPH_DIST_Y2:
            src = r->gr_d[species][which - PGB_GRAPH_DIST_X1]; cnt = r->gr.no_bins; break;
        case PGB_GRAPH_MAXIMA:
            if (n < 5) return PGB_ERR_ARG;
            out[0] = gr_max(r->gr_f[1], G, 0, steps);
            out[1] = gr_max(r->gr_f[2], G, 0, steps);
            out[2] = gr_max(r->gr_f[3], G, 0, steps);
            out[3] = gr_max(r->gr_q[0], G, r->nx + 1, steps);
            out[4] = gr_max(r->gr_q[1], G, r->nx + 1, steps);
            return 0;
        default: return PGB_ERR_ARG;
    }
    if (n < cnt) return PGB_ERR_ARG;
    for (int64_t k = 0; k < cnt; ++k) out[k] = src[k] / div;
    return 0;
}

/* ------------------------------------------------------------- plots */
/* CPU restatement of the headless viewer plots of pgb_render, written
 * separately from the CUDA code: the same selection, mapping and colour
 * rules (graphics.cpp:245-607), in the same FP32/FP64 operations, with
 * -ffp-contract=off.  Particles are converted to FP32 cell units as the
 * library's load does.                                                    */
static unsigned char plot_byte(float c) {
    float v = c * 255.0f + 0.5f;
    if (v < 0.0f) v = 0.0f;
    if (v > 255.0f) v = 255.0f;
    return (unsigned char)(int)v;
}
static uint32_t plot_hash(uint32_t id, uint32_t seed) {   /* lowbias32 */
    uint32_t x = id ^ (seed * 0x9E3779B9u);
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
static int plot_keep(uint32_t id, uint32_t seed, int64_t nlive, int max_points) {
    if (max_points <= 0 || nlive <= max_points) return 1;
    uint64_t thresh = (uint64_t)((double)max_points / (double)nlive * 4294967296.0);
    return (uint64_t)plot_hash(id, seed) < thresh;
}
static void plot_point(unsigned char* img, int W, int H, int px, int py, const unsigned char* c) {
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            int x = px + dx, y = py - dy;
            if (x < 0 || x >= W || y < 0 || y >= H) continue;
            memcpy(img + 3 * ((size_t)y * W + x), c, 3);
        }
}
static void plot_species(orc_run* r, int s, int phase, int W, int H, int max_points, uint32_t seed,
                         const unsigned char* colour, unsigned char* img) {
    const int ps = lib_shift(r);
    const orc_sp* S = &r->sp[s];
    const float lx = (float)(r->nx - 1), ly = (float)(r->ny - 1);
    int mvx = 1, mvy = 1;
    if (phase) {
        float mx = 0.0f, my = 0.0f;
        for (int64_t i = 0; i < S->n; ++i) {
            float xs = plot_cells(S->p[i].x, r->dx, ps), ys = plot_cells(S->p[i].y, r->dy, ps);
            if (!(xs > 0.0f && xs < lx && ys > 0.0f && ys < ly) || !plot_keep(S->id[i], seed, S->n, max_points)) continue;
            float ax = fabsf((float)S->p[i].vx), ay = fabsf((float)S->p[i].vy);
            if (ax == ax && ax > mx) mx = ax;
            if (ay == ay && ay > my) my = ay;
        }
        mvx = mx < 2147483520.0f ? (int)mx : 2147483647;
        mvy = my < 2147483520.0f ? (int)my : 2147483647;
        if (mvx < 1) mvx = 1;
        if (mvy < 1) mvy = 1;
    }
    for (int64_t i = 0; i < S->n; ++i) {
        float xs = plot_cells(S->p[i].x, r->dx, ps), ys = plot_cells(S->p[i].y, r->dy, ps);
        if (!(xs > 0.0f && xs < lx && ys > 0.0f && ys < ly) || !plot_keep(S->id[i], seed, S->n, max_points)) continue;
        float fx, fy;
        if (phase) {
            float vx = (float)S->p[i].vx, vy = (float)S->p[i].vy;
            if (!(fabsf(vx) < (float)mvx && fabsf(vy) < (float)mvy)) continue;
            fx = (vx / (float)mvx + 1.0f) * 0.5f;
            fy = (vy / (float)mvy + 1.0f) * 0.5f;
        } else {
            fx = xs / lx;
            fy = ys / ly;
        }
        int px = (int)(fx * (float)W), py = H - 1 - (int)(fy * (float)H);
        px = px < 0 ? 0 : (px > W - 1 ? W - 1 : px);
        py = py < 0 ? 0 : (py > H - 1 ? H - 1 : py);
        plot_point(img, W, H, px, py, colour);
    }
}
/* drawField's ramp (graphics.cpp:303-356) */
static void plot_ramp(float zAv, float c[3]) {
    static const float red[3] = {1.0f, 0.0f, 0.0f}, orange[3] = {1.0f, 0.396f, 0.0f},
                       yellow[3] = {1.0f, 1.0f, 0.0f}, green[3] = {0.0f, 1.0f, 0.0f},
                       blue[3] = {0.0f, 0.0f, 1.0f}, purple[3] = {0.396f, 0.0f, 1.0f};
    const float rd = 0.2f;
    float alpha = zAv < 1.0f ? zAv : 1.0f;
    const float *c1, *c2;
    if (zAv < rd) { alpha /= rd; c1 = red; c2 = orange; }
    else if ((double)zAv < 2.0 * (double)rd) { alpha = (alpha - rd) / rd; c1 = orange; c2 = yellow; }
    else if ((double)zAv < 3.0 * (double)rd) { alpha = (float)(((double)alpha - 2.0 * (double)rd) / (double)rd); c1 = yellow; c2 = green; }
    else if ((double)zAv < 4.0 * (double)rd) { alpha = (float)(((double)alpha - 3.0 * (double)rd) / (double)rd); c1 = green; c2 = blue; }
    else { alpha = (float)(((double)alpha - 4.0 * (double)rd) / (double)rd); c1 = blue; c2 = purple; }
    for (int k = 0; k < 3; ++k) c[k] = c1[k] * (1.0f - alpha) + c2[k] * alpha;
}

int orc_render(orc_run* r, int plot, int W, int H, int max_points, uint32_t seed, unsigned char* img, int64_t cap) {
    if (W < 1 || H < 1 || cap < 3LL * W * H || plot < 0 || plot > PGB_PLOT_ION_DENSITY) return PGB_ERR_ARG;
    static const unsigned char lime[3] = {142, 255, 29}, pink[3] = {255, 29, 142};
    memset(img, 0, (size_t)3 * W * H);
    if (plot == PGB_PLOT_PARTICLE_XY) {
        plot_species(r, 0, 0, W, H, max_points, seed, lime, img);
        plot_species(r, 1, 0, W, H, max_points, seed, pink, img);
        return 0;
    }
    if (plot == PGB_PLOT_ELECTRON_VX_VY || plot == PGB_PLOT_ION_VX_VY) {
        int s = plot == PGB_PLOT_ELECTRON_VX_VY ? 0 : 1;
        plot_species(r, s, 1, W, H, max_points, seed, s == 0 ? lime : pink, img);
        return 0;
    }
    const int n = r->nx, G = r->nx * r->ny;
    const double* src;
    double div = 1.0;
    int gs = 0;
    switch (plot) {
        case PGB_PLOT_PHI: src = r->gr_on ? r->gr_f[1] : r->phi; break;
        case PGB_PLOT_EFIELD_X: src = r->gr_on ? r->gr_f[2] : r->ex; break;
        case PGB_PLOT_EFIELD_Y: src = r->gr_on ? r->gr_f[3] : r->ey; break;
        default: {
            int s = plot == PGB_PLOT_E_DENSITY ? 0 : 1;
            gs = 1;
            src = r->gr_on ? r->gr_q[s] : r->q[s];
            if (!r->gr_on) div = s == 0 ? -C_CHARGE : C_CHARGE;
        }
    }
    if (r->gr_on) div = (double)r->gr.no_graph_steps;
    int have = 0;
    double mx = 0.0;
    for (int k = 0; k < G; ++k) {
        double v = src[k] / div;
        if (v == v && (!have || v > mx)) { mx = v; have = 1; }
    }
    double fmax = fabs(mx);
    if (!have || !(fmax >= 1.0)) fmax = 1.0;
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            unsigned char* q = img + 3 * ((size_t)py * W + px);
            float u = ((float)px + 0.5f) * (float)(n - 1) / (float)W;
            float v = ((float)(H - 1 - py) + 0.5f) * (float)(n - 1) / (float)H;
            int i = (int)u, j = (int)v;
            float fu = u - (float)i, fv = v - (float)j;
            if (i < gs || i >= n - gs - 1 || j < gs || j >= n - gs - 1 || fu < 0.1f || fu > 0.9f || fv < 0.1f ||
                fv > 0.9f)
                continue;
            float z0 = (float)(src[(size_t)(j + 1) * n + i] / div / fmax);
            float z1 = (float)(src[(size_t)(j + 1) * n + i + 1] / div / fmax);
            float z2 = (float)(src[(size_t)j * n + i + 1] / div / fmax);
            float z3 = (float)(src[(size_t)j * n + i] / div / fmax);
            float zAv = (float)fabs((double)(z0 + z1 + z2 + z3) / 4.0);
            float c[3];
            plot_ramp(zAv, c);
            q[0] = plot_byte(c[0]); q[1] = plot_byte(c[1]); q[2] = plot_byte(c[2]);
        }
    return 0;
}

/* pic::pic_run loop body (pic.cpp:1069-1250) and the graphs sums of the
 * window (pic.cpp:1189-1207); printing left out                          */
void orc_step(orc_run* r, int nsteps) {
    for (int k = 0; k < nsteps; ++k) {
        int64_t t = r->time_step;
        r->rng_step = (uint32_t)t;
        if (r->order_mode == ORC_ORDER_STABLE && r->prm.sort_interval > 0) {
            if (t % r->prm.sort_interval == 0) orc_sort_bins(r, PGB_ELECTRONS);
            if (t % ((int64_t)r->prm.sort_interval * PGB_ION_SORT_FACTOR) == 0) orc_sort_bins(r, PGB_IONS);
        }
        if (r->prm.have_collisions) orc_collide_electrons(r);
        orc_inject(r);
        orc_gather_push(r, PGB_ELECTRONS);
        if (t % r->dt_dti == 0) {
            if (r->prm.have_collisions) orc_collide_ions(r);
            orc_gather_push(r, PGB_IONS);
            orc_boundary(r, PGB_BOUNDARY_IONS);
            orc_boundary(r, PGB_BOUNDARY_ELECTRONS);
        } else {
            orc_boundary(r, PGB_BOUNDARY_ELECTRONS);
        }
        if (!r->prm.steadystate) orc_contain_growth(r, PGB_ELECTRONS);
        if (!r->prm.steadystate) orc_contain_growth(r, PGB_IONS);
        orc_deposit(r, PGB_IONS);
        orc_deposit(r, PGB_ELECTRONS);
        orc_grid_rho(r);
        orc_poisson(r, t);
        orc_efield(r);
        if (r->gr_on && t >= r->gr.start_step && t < r->gr.end_step) orc_graphs_accumulate(r);
        r->time_step = t + 1;
        r->c.step = r->time_step;
    }
}

/* ---------------------------------------------------------------- io */
int orc_get_grid(orc_run* r, int which, double* out, int64_t n) {
    int64_t G = (int64_t)r->nx * r->ny, GE = (int64_t)(r->nx + 1) * (r->ny + 1);
    const double* src = NULL;
    int64_t cnt = G;
    switch (which) {
        case PGB_GRID_Q_E: src = r->q[0]; break;
        case PGB_GRID_Q_I: src = r->q[1]; break;
        case PGB_GRID_RHO: src = r->rho; break;
        case PGB_GRID_PHI: src = r->phi; break;
        case PGB_GRID_EX: src = r->ex; cnt = GE; break;
        case PGB_GRID_EY: src = r->ey; cnt = GE; break;
        default: return PGB_ERR_ARG;
    }
    if (n < cnt) return PGB_ERR_ARG;
    memcpy(out, src, (size_t)cnt * sizeof(double));
    return 0;
}

int orc_set_rho(orc_run* r, const double* rho, int64_t n) {
    int64_t G = (int64_t)r->nx * r->ny;
    if (n < G) return PGB_ERR_ARG;
    memcpy(r->rho, rho, (size_t)G * sizeof(double));
    return 0;
}

void orc_get_counters(orc_run* r, pgb_counters* out) {
    *out = r->c;
    out->n_e = r->sp[0].n;
    out->n_i = r->sp[1].n;
    out->step = r->time_step;
}

/* Philox4x32-10 block, exposed for the known-answer test of the shared generator */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    pgb_u32x4 r = pgb_philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
    for (int k = 0; k < 4; ++k) out[k] = r.v[k];
}
