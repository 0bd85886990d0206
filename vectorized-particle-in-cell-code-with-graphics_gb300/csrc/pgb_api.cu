/*
 * C ABI of libpicgb (include/picgb.h): run handles, particle I/O and the
 * host-side sequencing of the per-step kernels.
 *
 * pgb_step follows pic::pic_run's loop body (pic.cpp:1069-1250) on one CUDA
 * stream without host synchronisation inside a step:
 *   electron collisions + gather + push + deposit + wall list   (one kernel)
 *   ionization products, injection (+ push of the injected electrons)
 *   [ion step] charge exchange, ion gather + push + deposit + wall list,
 *              ion walls, electron walls
 *   [other steps] ion deposit, electron walls
 *   charge -> rho -> Poisson right-hand side, full multigrid, E
 * The per-phase entry points run the same kernels one reference call at a
 * time.
 */
#include <cuda_runtime.h>
#include <cstdlib>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <new>
#include <string>
#include <vector>
#include <nvtx3/nvToolsExt.h>
#include "pgb_internal.h"

/* NVTX ranges around the entry points and each issued step: host-side
 * enqueue spans for a timeline tool (no cost without one attached)     */
namespace {
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};
}
#include "pgb_physics.cuh"
#include "pgb_rng.h"

static std::string g_create_error = "no error";

bool pgb_cuda_ok(pgb_run* r, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    if (r) r->err = msg;
    else g_create_error = msg;
    return false;
}

static int fail(pgb_run* r, int code, const std::string& msg) {
    if (r) r->err = msg;
    else g_create_error = msg;
    return code;
}

void pgb_set_unbound_error(const std::string& msg) { g_create_error = msg; }

extern "C" const char* pgb_last_error(const pgb_run* r) {
    return r ? r->err.c_str() : g_create_error.c_str();
}

/* pgb_params from parameters.h defaults (parameters.h:41-366 and the
 * boundary constants of pic.cpp:459-484)                               */
extern "C" int pgb_params_default(pgb_params* p) {
    if (!p) return PGB_ERR_ARG;
    memset(p, 0, sizeof(*p));
    const double CHARGE = 1.602177e-19, EPS = 8.854e-12, ME = 9.10939e-31, AMU = 1.66054e-27, PI = 3.141592654;
    const double T = 1.5, ne = 1.0e15;
    double ion_mass = 39.948 * AMU;
    double xl = (double)64 * sqrt((EPS * T) / (ne * CHARGE));
    double pf = sqrt((ne * 2.566971e-38) / (EPS * ME));
    p->x_no_of_cells = p->y_no_of_cells = 257;
    p->xlength = p->ylength = xl;
    p->dt = 0.1 / pf;
    p->dti = 1.0 * p->dt;
    p->electron_mass = ME;
    p->ion_mass = ion_mass;
    p->q_over_me = -CHARGE / ME;
    p->q_over_mi = CHARGE / ion_mass;
    p->qce = 1.0e6 * -CHARGE;
    p->qci = 1.0e6 * CHARGE;
    p->vte = sqrt(T * CHARGE / ME);
    p->vti = sqrt(T * CHARGE / ion_mass);
    p->vtn = sqrt(0.025 * CHARGE / ion_mass);
    p->angle = 30.0 * PI / 180.0;
    p->neutral_density = (0.2 * 133.32) / (0.025 * CHARGE);
    p->threshold = 15.75;
    p->work_function = 4.6;
    p->species = PGB_ARGON;
    p->steadystate = 1;
    p->init_no_neutrals = 10000;
    p->see_e0 = 4.32; p->see_max_yield = 1.4; p->see_emax0 = 650.0;
    p->no_groups = 3;
    for (int k = 0; k < 3; ++k) {
        p->v_limit_e[k] = (k == 0 ? 2.0 : k == 1 ? 3.0 : 1000.0) * p->vte;
        p->v_limit_i[k] = (k == 0 ? 2.0 : k == 1 ? 3.0 : 1000.0) * p->vti;
        p->group_limit_e[k] = 400000; p->new_group_size_e[k] = 200000;
        p->group_limit_i[k] = k == 0 ? 400000 : 100000;
        p->new_group_size_i[k] = k == 0 ? 200000 : 50000;
    }
    p->size_to_check_e = p->size_to_check_i = 1000001;
    p->seed = 1;
    p->poisson_mode = PGB_POISSON_FMG_REF;
    p->dc_max_iters = 8;
    p->dc_tolerance = 1e-10;
    return 0;
}

/* collisions::calc_neutral_velocity (collisions.cpp:66-89) on the Philox
 * stream of entry i; the same host code builds the CPU oracle's table.   */
static void neutral_table(const pgb_params& p, int which, double* out) {
    const int n = p.init_no_neutrals;
    const double PI = 3.141592654, vtn = p.vtn;
    for (int i = 0; i < n; ++i) {
        pgb_stream st;
        pgb_stream_init(&st, p.seed, (uint32_t)i, 0u, which ? PGB_STREAM_NEUTRAL_I : PGB_STREAM_NEUTRAL_E, 0u);
        double vx, vy, vz;
        do {
            double R1 = pgb_u01d(pgb_stream_u32(&st));
            double R2 = pgb_u01d(pgb_stream_u32(&st));
            vx = vtn * cos(PI * R2) * sqrt(fabs(log(R1)));
        } while (fabs(vx) > 10000.0 * vtn);
        do {
            double R1 = pgb_u01d(pgb_stream_u32(&st));
            double R2 = pgb_u01d(pgb_stream_u32(&st));
            vy = vtn * cos(PI * R2) * sqrt(fabs(log(R1)));
            vz = vtn * sin(PI * R2) * sqrt(fabs(log(R1)));
        } while (fabs(vy) > 10000.0 * vtn || fabs(vz) > 10000.0 * vtn);
        out[i] = vx; out[n + i] = vy; out[2 * n + i] = vz;
    }
}

static int validate(const pgb_params* p, std::string& why) {
    int n = p->x_no_of_cells;
    if (n < 5 || p->y_no_of_cells != n) { why = "grid must be square with at least 5 nodes"; return 0; }
    if (((n - 1) & (n - 2)) != 0) { why = "X_NO_OF_CELLS-1 must be a power of 2 (mglin.cpp:26)"; return 0; }
    if ((n - 1) > 32768) { why = "grid too large"; return 0; }
    if (!(p->xlength > 0) || !(p->ylength > 0) || !(p->dt > 0) || !(p->dti > 0)) { why = "lengths and time steps must be positive"; return 0; }
    if (p->init_no_neutrals < 2) { why = "INIT_NO_NEUTRALS must be >= 2"; return 0; }
    if (p->no_groups < 1 || p->no_groups > 3) { why = "NO_GROUPS must be 1..3"; return 0; }
    if (p->poisson_mode < PGB_POISSON_FMG_REF || p->poisson_mode > PGB_POISSON_DST_DC) {
        why = "poisson_mode must be one of PGB_POISSON_FMG_REF, _FP32_DC, _FMG32, _DST_DC";
        return 0;
    }
    if (p->dc_max_iters < 0 || p->dc_max_iters > 64) { why = "dc_max_iters must be 0..64"; return 0; }
    return 1;
}

static void free_species(Species& S) {
    cudaFree(S.xv); cudaFree(S.vz); cudaFree(S.w); cudaFree(S.id);
    cudaFree(S.xv2); cudaFree(S.vz2); cudaFree(S.w2); cudaFree(S.id2);
    S.xv = nullptr; S.vz = nullptr; S.w = nullptr; S.id = nullptr;
    S.xv2 = nullptr; S.vz2 = nullptr; S.w2 = nullptr; S.id2 = nullptr;
    S.cap = 0;
}

static void free_lists(pgb_run* r) {
    for (int l = 0; l < 4; ++l) {
        cudaFree(r->tile_list[l]); cudaFree(r->tile_cnt[l]); cudaFree(r->list[l]);
        r->tile_list[l] = r->tile_cnt[l] = r->list[l] = nullptr;
    }
    cudaFree(r->aux_i); cudaFree(r->aux_j); cudaFree(r->cx_tile_sum);
    cudaFree(r->cx_mask); cudaFree(r->cx_total);
    r->cx_mask = nullptr;
    r->cx_total = nullptr;
    for (int q = 0; q < 2; ++q) {
        cudaFree(r->tile_bin[q]); cudaFree(r->pieces[q]);
        r->tile_bin[q] = nullptr; r->pieces[q] = nullptr;
    }
    cudaFree(r->sort_counts); cudaFree(r->sort_offs); cudaFree(r->sort_key_total); cudaFree(r->sort_key_start);
    r->sort_counts = r->sort_offs = r->sort_key_total = nullptr;
    r->sort_key_start = nullptr;
    r->aux_i = r->aux_j = nullptr;
    r->cx_tile_sum = nullptr;
    r->list_cap = 0;
    r->ntiles_cap = 0;
}

/* grow particle storage (keeps contents) and the capacity-sized scratch */
static void drop_graphs(pgb_run* r);

static int ensure_capacity(pgb_run* r, int s, long long need) {
    Species& S = r->sp[s];
    if (need > S.cap || std::max(r->sp[0].cap, r->sp[1].cap) > r->list_cap) {
        /* the buffers about to be replaced may still be in use by queued
         * work (pgb_step_async): drain the run's streams first          */
        PGB_CK(r, cudaStreamSynchronize(r->stream));
        PGB_CK(r, cudaStreamSynchronize(r->copy_stream));
        if (r->side) PGB_CK(r, cudaStreamSynchronize(r->side));
        drop_graphs(r);
    }
    if (need > S.cap) {
        /* a species that already has storage grows by at least a quarter:
         * a load or a step that needs a few more slots than last time (ions
         * gain NUMBER_TO_INJECT a step) would otherwise reallocate every
         * buffer and re-capture the step graphs each time.  The first
         * allocation is exact, as pgb_footprint counts it.                  */
        long long cap = std::max<long long>(need, 1024);
        if (S.cap > 0) cap = std::min<long long>(std::max<long long>(cap, S.cap + S.cap / 4), 0x7fffffffLL);
        Species T;   /* the new storage; S keeps the old until it is copied */
        T.qc = S.qc; T.q_over_m = S.q_over_m; T.mass = S.mass; T.vt = S.vt; T.dt = S.dt;
        T.cap = cap;
        /* host-side fault injection (tests): the handle's fault_alloc-th
         * growth fails as if the device were out of memory              */
        const bool injected = r->fault_alloc > 0 && ++r->alloc_events == r->fault_alloc;
        if (injected || cudaMalloc(&T.xv, sizeof(float4) * cap) != cudaSuccess ||
            cudaMalloc(&T.vz, sizeof(float) * cap) != cudaSuccess || cudaMalloc(&T.w, sizeof(float) * cap) != cudaSuccess ||
            cudaMalloc(&T.id, sizeof(unsigned) * cap) != cudaSuccess || cudaMalloc(&T.xv2, sizeof(float4) * cap) != cudaSuccess ||
            cudaMalloc(&T.vz2, sizeof(float) * cap) != cudaSuccess || cudaMalloc(&T.w2, sizeof(float) * cap) != cudaSuccess ||
            cudaMalloc(&T.id2, sizeof(unsigned) * cap) != cudaSuccess) {
            cudaGetLastError();
            free_species(T);   /* what was allocated before the failure */
            return fail(r, PGB_ERR_NOMEM, "device allocation of particle storage failed");
        }
        if (S.cap > 0) {
            long long n = r->hs->n[s];
            PGB_CK(r, cudaMemcpyAsync(T.xv, S.xv, sizeof(float4) * n, cudaMemcpyDeviceToDevice, r->stream));
            PGB_CK(r, cudaMemcpyAsync(T.vz, S.vz, sizeof(float) * n, cudaMemcpyDeviceToDevice, r->stream));
            PGB_CK(r, cudaMemcpyAsync(T.w, S.w, sizeof(float) * n, cudaMemcpyDeviceToDevice, r->stream));
            PGB_CK(r, cudaMemcpyAsync(T.id, S.id, sizeof(unsigned) * n, cudaMemcpyDeviceToDevice, r->stream));
            PGB_CK(r, cudaStreamSynchronize(r->stream));
        }
        free_species(S);
        S = T;
        r->orient[s] = 0;
    }
    long long lc = std::max(r->sp[0].cap, r->sp[1].cap);
    if (lc > r->list_cap) {
        free_lists(r);
        long long nt = (lc + PGB_TILE - 1) / PGB_TILE + 1;
        for (int l = 0; l < 4; ++l) {
            /* a tile's list is its 32 ballot words (tile_masks) */
            if (cudaMalloc(&r->tile_list[l], sizeof(int) * nt * 32) != cudaSuccess ||
                cudaMalloc(&r->tile_cnt[l], sizeof(int) * nt) != cudaSuccess ||
                cudaMalloc(&r->list[l], sizeof(int) * lc) != cudaSuccess) {
                cudaGetLastError();
                return fail(r, PGB_ERR_NOMEM, "device allocation of event lists failed");
            }
            /* on the run's stream: a plain cudaMemset goes to the legacy
             * stream, which does not order against the run's non-blocking
             * stream                                                    */
            PGB_CK(r, cudaMemsetAsync(r->tile_cnt[l], 0, sizeof(int) * nt, r->stream));
        }
        if (cudaMalloc(&r->aux_i, sizeof(int) * std::max(lc, nt)) != cudaSuccess ||
            cudaMalloc(&r->aux_j, sizeof(int) * std::max(lc, nt)) != cudaSuccess) {
            cudaGetLastError();
            return fail(r, PGB_ERR_NOMEM, "device allocation of scratch failed");
        }
        int nbx, nby;
        pgb_bins(r, &nbx, &nby);
        long long nkeys = (long long)nbx * nby + 1;
        r->sort_chunks_cap = (lc + PGB_SORT_CHUNK - 1) / PGB_SORT_CHUNK + 1;
        for (int q = 0; q < 2; ++q) {
            if (cudaMalloc(&r->tile_bin[q], sizeof(int) * nt) != cudaSuccess ||
                cudaMalloc(&r->pieces[q], sizeof(int4) * (nt + nkeys + 1)) != cudaSuccess) {
                cudaGetLastError();
                return fail(r, PGB_ERR_NOMEM, "device allocation of sort tables failed");
            }
        }
        if (cudaMalloc(&r->sort_counts, sizeof(int) * nkeys * r->sort_chunks_cap) != cudaSuccess ||
            cudaMalloc(&r->sort_offs, sizeof(int) * nkeys * r->sort_chunks_cap) != cudaSuccess ||
            cudaMalloc(&r->sort_key_total, sizeof(int) * nkeys) != cudaSuccess ||
            cudaMalloc(&r->sort_key_start, sizeof(long long) * (nkeys + 1)) != cudaSuccess) {
            cudaGetLastError();
            return fail(r, PGB_ERR_NOMEM, "device allocation of sort scratch failed");
        }
        long long cxt = (lc + PGB_CX_TILE - 1) / PGB_CX_TILE + 1;
        r->cx_tiles_cap = cxt;
        r->cx_mask_words = (int)((cxt + 63) / 64);
        if (cudaMalloc(&r->cx_tile_sum, sizeof(long long) * cxt * r->nx) != cudaSuccess ||
            cudaMalloc(&r->cx_mask, sizeof(unsigned long long) * r->cx_mask_words * r->nx) != cudaSuccess ||
            cudaMalloc(&r->cx_total, sizeof(long long) * r->nx) != cudaSuccess) {
            cudaGetLastError();
            return fail(r, PGB_ERR_NOMEM, "device allocation of CX scratch failed");
        }
        PGB_CK(r, cudaMemsetAsync(r->cx_mask, 0, sizeof(unsigned long long) * r->cx_mask_words * r->nx, r->stream));
        PGB_CK(r, cudaMemsetAsync(r->cx_total, 0, sizeof(long long) * r->nx, r->stream));
        r->list_cap = lc;
        r->ntiles_cap = nt;
        /* the bin-piece tables of both species went with the old block
         * (a growth of the ions at a sort step drops the pieces that the
         * electron sort has just written): both species are unsorted
         * until their next sort, and the push walks them tile by tile   */
        for (int q = 0; q < 2; ++q) {
            PGB_CK(r, cudaMemsetAsync(&r->ds->n_pieces[q], 0, sizeof(int), r->stream));
            PGB_CK(r, cudaMemsetAsync(&r->ds->sorted_tiles[q], 0, sizeof(long long), r->stream));
        }
    }
    return 0;
}

static int sync_state(pgb_run* r) {
    PGB_CK(r, cudaMemcpyAsync(r->hs, r->ds, sizeof(DevState), cudaMemcpyDeviceToHost, r->stream));
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    if (r->hs->err) {
        int e = r->hs->err;
        std::string m = "device reported:";
        if (e & ERR_CAP_E) m += " electron capacity exceeded;";
        if (e & ERR_CAP_I) m += " ion capacity exceeded;";
        if (e & ERR_LIST) m += " event list overflow;";
        r->hs->err = 0;
        PGB_CK(r, cudaMemsetAsync(&r->ds->err, 0, sizeof(int), r->stream));
        return fail(r, PGB_ERR_CAPACITY, m);
    }
    return 0;
}

extern "C" int pgb_create(const pgb_params* p, pgb_run** out) {
    if (!p || !out) return fail(nullptr, PGB_ERR_ARG, "null argument");
    *out = nullptr;
    std::string why;
    if (!validate(p, why)) return fail(nullptr, PGB_ERR_ARG, why);
    pgb_run* r = new (std::nothrow) pgb_run();
    if (!r) return fail(nullptr, PGB_ERR_NOMEM, "host allocation failed");
    r->p = *p;
    r->nx = p->x_no_of_cells;
    r->ny = p->y_no_of_cells;
    r->ps = pgb_pos_shift(r->nx, r->ny);
    r->dx = p->xlength / (double)(r->nx - 1);
    r->dy = p->ylength / (double)(r->ny - 1);
    r->dt_dti = std::max(1, (int)(p->dti / p->dt));
    r->sp[0].qc = p->qce; r->sp[0].q_over_m = p->q_over_me; r->sp[0].mass = p->electron_mass;
    r->sp[0].vt = p->vte; r->sp[0].dt = p->dt;
    r->sp[1].qc = p->qci; r->sp[1].q_over_m = p->q_over_mi; r->sp[1].mass = p->ion_mass;
    r->sp[1].vt = p->vti; r->sp[1].dt = p->dti;
    auto bail = [&](int code) { pgb_destroy(r); return code; };
    if (!pgb_cuda_ok(nullptr, cudaGetDevice(&r->dev), "cudaGetDevice")) return bail(PGB_ERR_CUDA);
    if (!pgb_cuda_ok(nullptr, cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, r->dev), "sm count"))
        return bail(PGB_ERR_CUDA);
    if (!pgb_cuda_ok(nullptr, cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !pgb_cuda_ok(nullptr, cudaStreamCreateWithFlags(&r->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate"))
        return bail(PGB_ERR_CUDA);
    for (int k = 0; k < PGB_COPY_EVENTS; ++k)
        if (!pgb_cuda_ok(nullptr, cudaEventCreateWithFlags(&r->copy_ev[k], cudaEventDisableTiming), "cudaEventCreate")) {
            for (int j = 0; j < k; ++j) cudaEventDestroy(r->copy_ev[j]);
            return bail(PGB_ERR_CUDA);
        }
    r->copy_ev_ok = true;
    if (const char* fa = std::getenv("PGB_FAULT_ALLOC")) r->fault_alloc = std::atoi(fa);
    /* the side stream only speeds steps up: without it steps run in turn.
     * It takes the highest priority, so that the field solve's short
     * kernels get SMs ahead of queued blocks of the run's own stream.     */
    int prio_lo = 0, prio_hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) == cudaSuccess &&
        cudaStreamCreateWithPriority(&r->side, cudaStreamNonBlocking, prio_hi) == cudaSuccess) {
        r->prio_hi = prio_hi;
        if (cudaEventCreateWithFlags(&r->ev_fork, cudaEventDisableTiming) == cudaSuccess) {
            if (cudaEventCreateWithFlags(&r->ev_join, cudaEventDisableTiming) == cudaSuccess) r->side_ok = true;
            else cudaEventDestroy(r->ev_fork);
        }
        if (!r->side_ok) { cudaStreamDestroy(r->side); r->side = nullptr; }
    }
    cudaGetLastError();
    const size_t G = (size_t)r->nx * r->ny, GE = (size_t)(r->nx + 1) * (r->ny + 1);
    bool ok = true;
    ok = ok && cudaMalloc(&r->ds, sizeof(DevState)) == cudaSuccess;
    ok = ok && cudaMallocHost(&r->hs, sizeof(DevState)) == cudaSuccess;
    for (int s = 0; s < 2; ++s) {
        ok = ok && cudaMalloc(&r->qacc[s], sizeof(unsigned long long) * G) == cudaSuccess;
        ok = ok && cudaMalloc(&r->q[s], sizeof(double) * G) == cudaSuccess;
    }
    ok = ok && cudaMalloc(&r->rho, sizeof(double) * G) == cudaSuccess;
    ok = ok && cudaMalloc(&r->phi, sizeof(double) * G) == cudaSuccess;
    ok = ok && cudaMalloc(&r->ex, sizeof(double) * GE) == cudaSuccess;
    ok = ok && cudaMalloc(&r->ey, sizeof(double) * GE) == cudaSuccess;
    ok = ok && cudaMalloc(&r->exy, sizeof(float2) * GE) == cudaSuccess;
    ok = ok && cudaMalloc(&r->prob_cx, sizeof(long long) * r->nx) == cudaSuccess;
    r->phi_tab_cap = 4096;
    ok = ok && cudaMalloc(&r->inject_flag, sizeof(int) * (p->number_to_inject + 1)) == cudaSuccess;
    ok = ok && cudaMalloc(&r->phi_tab, sizeof(double) * r->phi_tab_cap) == cudaSuccess;
    ok = ok && cudaMallocHost(&r->phi_host, sizeof(double) * r->phi_tab_cap) == cudaSuccess;
    ok = ok && cudaMallocHost(&r->t_host, sizeof(long long) * 2) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&r->phi_ev, cudaEventDisableTiming) == cudaSuccess;
    if (ok) r->phi_ev_ok = true;
    int ng = 0, nn = r->nx;
    while (nn >>= 1) ng++;
    r->ng = ng;
    nn = r->nx;
    for (int j = ng - 1; j >= 0; --j) {
        r->mg_n[j] = nn;
        size_t s = (size_t)nn * nn * sizeof(double);
        ok = ok && cudaMalloc(&r->mg_u[j], s) == cudaSuccess && cudaMalloc(&r->mg_f[j], s) == cudaSuccess &&
             cudaMalloc(&r->mg_v[j], s) == cudaSuccess && cudaMalloc(&r->mg_r[j], s) == cudaSuccess;
        nn = nn / 2 + 1;
    }
    for (int w = 0; w < 2; ++w)
        ok = ok && cudaMalloc(&r->neut[w], sizeof(float) * 3 * p->init_no_neutrals) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        fail(nullptr, PGB_ERR_NOMEM, "device allocation failed");
        return bail(PGB_ERR_NOMEM);
    }
    memset(r->hs, 0, sizeof(DevState));
    if (!pgb_cuda_ok(nullptr, cudaMemset(r->ds, 0, sizeof(DevState)), "memset")) return bail(PGB_ERR_CUDA);
    cudaMemset(r->q[0], 0, sizeof(double) * G);
    cudaMemset(r->q[1], 0, sizeof(double) * G);
    cudaMemset(r->rho, 0, sizeof(double) * G);
    cudaMemset(r->phi, 0, sizeof(double) * G);
    cudaMemset(r->ex, 0, sizeof(double) * GE);
    cudaMemset(r->ey, 0, sizeof(double) * GE);
    cudaMemset(r->exy, 0, sizeof(float2) * GE);
    cudaMemset(r->prob_cx, 0, sizeof(long long) * r->nx);
    cudaMemset(r->inject_flag, 0, sizeof(int) * (p->number_to_inject + 1));
    /* ion table first, then electron table (pic.cpp:135-138) */
    {
        const int nn = 3 * p->init_no_neutrals;
        std::vector<double> tab((size_t)nn);
        std::vector<float> tab32((size_t)nn);
        for (int w = 1; w >= 0; --w) {
            neutral_table(*p, w, tab.data());
            for (int k = 0; k < nn; ++k) tab32[k] = (float)tab[k];
            double vmax = 0.0;
            for (int k = 0; k < p->init_no_neutrals; ++k) {
                double a = tab32[k], b = tab32[p->init_no_neutrals + k], c = tab32[2 * p->init_no_neutrals + k];
                vmax = std::max(vmax, std::sqrt(a * a + b * b + c * c));
            }
            r->vn_max[w] = (float)vmax;
            cudaMemcpy(r->neut[w], tab32.data(), sizeof(float) * nn, cudaMemcpyHostToDevice);
        }
    }
    if (pgb_mg_setup(r) || pgb_sort_setup(r)) { g_create_error = r->err; return bail(PGB_ERR_CUDA); }
    if (!pgb_cuda_ok(nullptr, cudaDeviceSynchronize(), "create")) return bail(PGB_ERR_CUDA);
    *out = r;
    return 0;
}

extern "C" int pgb_destroy(pgb_run* r) {
    if (!r) return 0;
    if (r->stream) cudaStreamSynchronize(r->stream);
    if (r->side) cudaStreamSynchronize(r->side);
    drop_graphs(r);
    cudaFree(r->phi_tab);
    if (r->phi_host) cudaFreeHost(r->phi_host);
    if (r->t_host) cudaFreeHost(r->t_host);
    if (r->phi_ev_ok) cudaEventDestroy(r->phi_ev);
    cudaFree(r->inject_flag);
    free_species(r->sp[0]);
    free_species(r->sp[1]);
    free_lists(r);
    cudaFree(r->ds);
    if (r->hs) cudaFreeHost(r->hs);
    for (int s = 0; s < 2; ++s) { cudaFree(r->qacc[s]); cudaFree(r->q[s]); }
    cudaFree(r->rho); cudaFree(r->phi); cudaFree(r->ex); cudaFree(r->ey); cudaFree(r->exy);
    cudaFree(r->prob_cx);
    for (int j = 0; j < r->ng; ++j) { cudaFree(r->mg_u[j]); cudaFree(r->mg_f[j]); cudaFree(r->mg_v[j]); cudaFree(r->mg_r[j]); }
    cudaFree(r->mg_tab);
    pgb_mg_free(r);
    for (int w = 0; w < 2; ++w) cudaFree(r->neut[w]);
    if (r->h_stage) cudaFreeHost(r->h_stage);
    cudaFree(r->d_stage);
    cudaFree(r->kh);
    cudaFree(r->gr.buf);
    cudaFree(r->rd_img);
    cudaFree(r->rd_scratch);
    if (r->prof_ev_ok)
        for (int k = 0; k < 13; ++k) cudaEventDestroy(r->prof_ev[k]);
    if (r->copy_ev_ok)
        for (int k = 0; k < PGB_COPY_EVENTS; ++k) cudaEventDestroy(r->copy_ev[k]);
    if (r->side_ok) { cudaEventDestroy(r->ev_fork); cudaEventDestroy(r->ev_join); }
    if (r->side) cudaStreamDestroy(r->side);
    if (r->copy_stream) cudaStreamDestroy(r->copy_stream);
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
    return 0;
}

/* device staging buffer for AoS transfers, kept between calls */
static int dstage(pgb_run* r, size_t bytes) {
    if (bytes <= r->d_stage_bytes) return 0;
    cudaFree(r->d_stage);
    r->d_stage = nullptr;
    r->d_stage_bytes = 0;
    PGB_CK(r, cudaMalloc(&r->d_stage, bytes));
    r->d_stage_bytes = bytes;
    return 0;
}

/* slots the spatial sort may add: every bin (and the key of particles
 * outside the deposit region) starts on a tile boundary                  */
static long long sort_pad_slots(const pgb_params* p) {
    if (p->sort_interval <= 0) return 0;
    const long long nbx = (p->x_no_of_cells - 1 + PGB_BIN - 1) / PGB_BIN, nby = (p->y_no_of_cells - 1 + PGB_BIN - 1) / PGB_BIN;
    return (nbx * nby + 2) * PGB_TILE;
}

extern "C" int pgb_load_species(pgb_run* r, int s, const double* aos6, int64_t n) {
    Range range("pgb_load_species");
    if (!r || s < 0 || s > 1 || n < 0 || (n > 0 && !aos6)) return fail(r, PGB_ERR_ARG, "pgb_load_species: bad argument");
    if (n > 0x7fffffffLL) return fail(r, PGB_ERR_ARG, "pgb_load_species: too many particles");
    int rc = sync_state(r);
    if (rc) return rc;
    long long want = s == 0 ? r->p.capacity_e : r->p.capacity_i;
    long long cap = std::max<long long>(want, 2 * n + 65536 + sort_pad_slots(&r->p));
    if (cap > 0x7fffffffLL) cap = 0x7fffffffLL;
    r->hs->n[s] = 0;
    if ((rc = ensure_capacity(r, s, cap))) return rc;
    if ((rc = ensure_capacity(r, 1 - s, std::max<long long>(r->sp[1 - s].cap, 1024)))) return rc;
    if (n > 0) {
        if ((rc = dstage(r, sizeof(double) * 6 * n))) return rc;
        /* chunks: the copy of chunk c+1 (copy stream) overlaps the
         * conversion of chunk c (run stream)                              */
        bool ok = cudaEventRecord(r->copy_ev[0], r->stream) == cudaSuccess &&
                  cudaStreamWaitEvent(r->copy_stream, r->copy_ev[0], 0) == cudaSuccess;
        for (long long c = 0, k = 1; ok && c < n; c += PGB_COPY_CHUNK, ++k) {
            const long long e = std::min<long long>(n, c + PGB_COPY_CHUNK);
            cudaEvent_t ev = r->copy_ev[k % PGB_COPY_EVENTS];
            ok = cudaMemcpyAsync(r->d_stage + 6 * c, aos6 + 6 * c, sizeof(double) * 6 * (e - c), cudaMemcpyHostToDevice,
                                 r->copy_stream) == cudaSuccess &&
                 cudaEventRecord(ev, r->copy_stream) == cudaSuccess &&
                 cudaStreamWaitEvent(r->stream, ev, 0) == cudaSuccess && pgb_launch_load(r, s, r->d_stage, c, e) == 0;
        }
        if (!ok || cudaStreamSynchronize(r->stream) != cudaSuccess)
            return fail(r, PGB_ERR_CUDA, "pgb_load_species: upload failed");
    }
    r->hs->n[s] = n;
    r->hs->dead[s] = 0;
    r->hs->next_id[s] = (unsigned)n;
    PGB_CK(r, cudaMemcpyAsync(&r->ds->n[s], &r->hs->n[s], sizeof(long long), cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaMemcpyAsync(&r->ds->dead[s], &r->hs->dead[s], sizeof(long long), cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaMemcpyAsync(&r->ds->next_id[s], &r->hs->next_id[s], sizeof(unsigned), cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaMemsetAsync(&r->ds->n_pieces[s], 0, sizeof(int), r->stream));
    PGB_CK(r, cudaMemsetAsync(&r->ds->sorted_tiles[s], 0, sizeof(long long), r->stream));
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    return 0;
}

/* device bytes a run holds once ne electrons and ni ions are loaded, from
 * the allocations of pgb_create, ensure_capacity and the load staging    */
extern "C" int pgb_footprint(const pgb_params* p, int64_t ne, int64_t ni, int64_t* bytes) {
    if (!p || !bytes || ne < 0 || ni < 0 || p->x_no_of_cells < 3) return fail(nullptr, PGB_ERR_ARG, "pgb_footprint: bad argument");
    const long long nx = p->x_no_of_cells, ny = p->y_no_of_cells, G = nx * ny, GE = (nx + 1) * (ny + 1);
    const long long pad = sort_pad_slots(p);
    auto cap_of = [pad](long long want, long long n) {
        return std::min<long long>(std::max<long long>(want, 2 * n + 65536 + pad), 0x7fffffffLL);
    };
    const long long ce = cap_of(p->capacity_e, ne), ci = cap_of(p->capacity_i, ni), lc = std::max(ce, ci);
    const long long nt = (lc + PGB_TILE - 1) / PGB_TILE + 1;
    const long long nbx = (nx - 1 + PGB_BIN - 1) / PGB_BIN, nby = (ny - 1 + PGB_BIN - 1) / PGB_BIN, nkeys = nbx * nby + 1;
    long long b = 0;
    b += 2 * (16 + 4 + 4 + 4) * (ce + ci);                               /* particles, two copies */
    b += 4 * (4 * nt * 32 + 4 * nt + 4 * lc);                            /* event lists (32 mask words a tile) */
    b += 2 * 4 * std::max(lc, nt);                                        /* aux_i, aux_j */
    b += 2 * (4 * nt + 16 * (nt + nkeys + 1));                            /* tile bins, pieces */
    const long long chunks = (lc + PGB_SORT_CHUNK - 1) / PGB_SORT_CHUNK + 1;
    b += 2 * 4 * nkeys * chunks + 4 * nkeys + 8 * (nkeys + 1);            /* sort scratch */
    b += 8 * nx * ((lc + PGB_CX_TILE - 1) / PGB_CX_TILE + 1) + 8 * nx * ((lc + PGB_CX_TILE - 1) / PGB_CX_TILE / 64 + 2); /* CX tile sums, masks */
    b += 48 * std::max(ne, ni);                                           /* load/dump staging */
    long long levels = 0;
    for (long long n = nx; n >= 3; n = n / 2 + 1) { levels += n * n; if (n == 3) break; }
    b += 5 * 8 * levels + 5 * 4 * levels;                                 /* multigrid, FP64 and FP32 */
    b += 8 * (2 + 2 + 2 + 1) * G + 8 * 3 * GE + 8 * nx + 8 * 4096;        /* grids, phi table */
    b += 6 * p->init_no_neutrals * 4 + (16 << 20);                        /* neutral tables, streams, graphs */
    *bytes = b;
    return 0;
}

extern "C" int pgb_species_count(pgb_run* r, int s, int64_t* n_out) {
    if (!r || s < 0 || s > 1 || !n_out) return fail(r, PGB_ERR_ARG, "pgb_species_count: bad argument");
    int rc = sync_state(r);
    if (rc) return rc;
    *n_out = r->hs->n[s] - r->hs->dead[s];
    return 0;
}

extern "C" int pgb_dump_species(pgb_run* r, int s, double* aos6, int64_t cap, int64_t* n_out) {
    Range range("pgb_dump_species");
    if (!r || s < 0 || s > 1 || cap < 0 || (cap > 0 && !aos6)) return fail(r, PGB_ERR_ARG, "pgb_dump_species: bad argument");
    int rc = sync_state(r);
    if (rc) return rc;
    long long live = r->hs->n[s] - r->hs->dead[s];
    if (n_out) *n_out = live;
    long long m = std::min<long long>(live, cap);
    if (m <= 0 || r->sp[s].cap == 0) return 0;
    if ((rc = dstage(r, sizeof(double) * 6 * live))) return rc;
    /* live-slot offsets of every tile, then chunks of tiles: the copy of
     * chunk c (copy stream) overlaps the packing of chunk c+1 (run stream) */
    const long long n = r->hs->n[s];
    const int ntiles = (int)((n + PGB_TILE - 1) / PGB_TILE);
    std::vector<int> toff((size_t)ntiles);
    if (pgb_launch_dump_offsets(r, s) ||
        cudaMemcpyAsync(toff.data(), r->aux_j, sizeof(int) * (size_t)ntiles, cudaMemcpyDeviceToHost, r->stream) != cudaSuccess ||
        cudaStreamSynchronize(r->stream) != cudaSuccess)
        return fail(r, PGB_ERR_CUDA, "pgb_dump_species: offsets failed");
    const int per = PGB_COPY_CHUNK / PGB_TILE;
    bool ok = true;
    for (int t0 = 0, k = 0; ok && t0 < ntiles; t0 += per, ++k) {
        const int t1 = std::min(ntiles, t0 + per);
        const long long a = std::min<long long>(toff[t0], m), b = std::min<long long>(t1 < ntiles ? toff[t1] : live, m);
        cudaEvent_t ev = r->copy_ev[k % PGB_COPY_EVENTS];
        ok = pgb_launch_dump(r, s, r->d_stage, nullptr, live, t0, t1) == 0 && cudaEventRecord(ev, r->stream) == cudaSuccess &&
             cudaStreamWaitEvent(r->copy_stream, ev, 0) == cudaSuccess &&
             (b <= a || cudaMemcpyAsync(aos6 + 6 * a, r->d_stage + 6 * a, sizeof(double) * 6 * (b - a),
                                        cudaMemcpyDeviceToHost, r->copy_stream) == cudaSuccess);
    }
    if (!ok || cudaStreamSynchronize(r->copy_stream) != cudaSuccess || cudaStreamSynchronize(r->stream) != cudaSuccess)
        return fail(r, PGB_ERR_CUDA, "pgb_dump_species: download failed");
    return 0;
}

extern "C" int pgb_dump_ids(pgb_run* r, int s, uint32_t* ids, int64_t cap, int64_t* n_out) {
    Range range("pgb_dump_ids");
    if (!r || s < 0 || s > 1 || cap < 0 || (cap > 0 && !ids)) return fail(r, PGB_ERR_ARG, "pgb_dump_ids: bad argument");
    int rc = sync_state(r);
    if (rc) return rc;
    long long live = r->hs->n[s] - r->hs->dead[s];
    if (n_out) *n_out = live;
    long long m = std::min<long long>(live, cap);
    if (m <= 0 || r->sp[s].cap == 0) return 0;
    if ((rc = dstage(r, sizeof(double) * 6 * live))) return rc;
    const int ntiles = (int)((r->hs->n[s] + PGB_TILE - 1) / PGB_TILE);
    unsigned int* d_ids = reinterpret_cast<unsigned int*>(r->d_stage);
    if (pgb_launch_dump_offsets(r, s) || pgb_launch_dump(r, s, nullptr, d_ids, m, 0, ntiles) ||
        cudaMemcpyAsync(ids, d_ids, sizeof(uint32_t) * (size_t)m, cudaMemcpyDeviceToHost, r->stream) != cudaSuccess ||
        cudaStreamSynchronize(r->stream) != cudaSuccess)
        return fail(r, PGB_ERR_CUDA, "pgb_dump_ids: download failed");
    return 0;
}

extern "C" int pgb_cross_sections(int32_t which, const double* energies, int64_t n, double* out) {
    if (which < PGB_XS_AR_ELASTIC || which > PGB_XS_H_CX || n < 0 || (n > 0 && (!energies || !out)))
        return fail(nullptr, PGB_ERR_ARG, "pgb_cross_sections: bad argument");
    if (n == 0) return 0;
    double* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * 2 * (size_t)n);
    if (e != cudaSuccess) return fail(nullptr, PGB_ERR_CUDA, std::string("pgb_cross_sections: ") + cudaGetErrorString(e));
    int rc = 0;
    if (cudaMemcpy(d, energies, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess ||
        pgb_launch_cross_sections(which, d, n, d + n, nullptr) != 0 ||
        cudaMemcpy(out, d + n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = fail(nullptr, PGB_ERR_CUDA, "pgb_cross_sections: evaluation failed");
    cudaFree(d);
    return rc;
}

extern "C" int pgb_set_time_step(pgb_run* r, int64_t t) {
    if (!r) return PGB_ERR_ARG;
    r->time_step = t;
    return 0;
}

static int need_particles(pgb_run* r) {
    if (r->sp[0].cap == 0 || r->sp[1].cap == 0) return fail(r, PGB_ERR_STATE, "load both species first");
    return 0;
}

/* ds->t = t0 and the right-wall potentials phi_right*cos(phi_period*t) of
 * steps t0 .. t0+n-1 (fields.cpp:177), computed on the host as the
 * reference does                                                         */
static int set_device_step(pgb_run* r, int64_t t0, int n) {
    if (n > r->phi_tab_cap) return fail(r, PGB_ERR_ARG, "step table too small");
    /* the pinned staging is reused once its previous upload has left */
    PGB_CK(r, cudaEventSynchronize(r->phi_ev));
    for (int k = 0; k < n; ++k) r->phi_host[k] = r->p.phi_right * cos(r->p.phi_period * (double)(t0 + k));
    r->t_host[0] = (long long)t0;
    PGB_CK(r, cudaMemcpyAsync(r->phi_tab, r->phi_host, sizeof(double) * n, cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaMemcpyAsync(&r->ds->t, r->t_host, sizeof(long long), cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaMemcpyAsync(&r->ds->t_base, r->t_host, sizeof(long long), cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaMemcpyAsync(&r->ds->tf, r->t_host, sizeof(long long), cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaEventRecord(r->phi_ev, r->stream));
    return 0;
}

/* ---------------------------------------------------- phase entry points */
static int boundary_phase(pgb_run* r, int which) {
    if (r->p.steadystate) {
        if (which != PGB_BOUNDARY_ELECTRONS) return 0;   /* steady_i_boundary is empty */
        if (pgb_launch_flag_outside(r, 0) || pgb_build_list(r, LIST_OUT_E, 0)) return PGB_ERR_CUDA;
        if (pgb_launch_flag_outside(r, 1) || pgb_build_list(r, LIST_OUT_I, 1)) return PGB_ERR_CUDA;
        return pgb_launch_walls(r, which);
    }
    int s = which == PGB_BOUNDARY_IONS ? 1 : 0;
    int l = s ? LIST_OUT_I : LIST_OUT_E;
    if (pgb_launch_flag_outside(r, s) || pgb_build_list(r, l, s)) return PGB_ERR_CUDA;
    return pgb_launch_walls(r, which);
}

extern "C" int pgb_boundary(pgb_run* r, int which) {
    if (!r || (which != 0 && which != 1)) return fail(r, PGB_ERR_ARG, "pgb_boundary: bad argument");
    int rc = need_particles(r);
    if (rc) return rc;
    /* deposits made by wall events go to the accumulators of the step; in
     * the phase-by-phase form the charge is recomputed by pgb_deposit     */
    if ((rc = set_device_step(r, r->time_step, 1))) return rc;
    if ((rc = boundary_phase(r, which))) return rc;
    return sync_state(r);
}

extern "C" int pgb_initial_boundary(pgb_run* r) {
    if (!r) return PGB_ERR_ARG;
    int rc = need_particles(r);
    if (rc) return rc;
    /* random streams of the pre-loop boundary pass use step -1 */
    if ((rc = set_device_step(r, -1, 1))) return rc;
    rc = boundary_phase(r, PGB_BOUNDARY_IONS);
    if (!rc) rc = boundary_phase(r, PGB_BOUNDARY_ELECTRONS);
    if (rc) return rc;
    return sync_state(r);
}

extern "C" int pgb_collide_electrons(pgb_run* r) {
    if (!r) return PGB_ERR_ARG;
    int rc = need_particles(r);
    if (rc) return rc;
    if ((rc = set_device_step(r, r->time_step, 1))) return rc;
    if (pgb_launch_mcc(r, 0) || pgb_launch_scatter(r, 0) || pgb_build_list(r, LIST_ION_EV, 0) ||
        pgb_launch_ionize_appends(r, 1, 1))
        return PGB_ERR_CUDA;
    return sync_state(r);
}

extern "C" int pgb_inject(pgb_run* r) {
    if (!r) return PGB_ERR_ARG;
    int rc = need_particles(r);
    if (rc) return rc;
    if ((rc = set_device_step(r, r->time_step, 1))) return rc;
    if (pgb_launch_inject(r, 3, false)) return PGB_ERR_CUDA;
    return sync_state(r);
}

extern "C" int pgb_gather_push(pgb_run* r, int s) {
    if (!r || s < 0 || s > 1) return fail(r, PGB_ERR_ARG, "pgb_gather_push: bad argument");
    int rc = need_particles(r);
    if (rc) return rc;
    if (pgb_launch_push(r, s, false)) return PGB_ERR_CUDA;
    return sync_state(r);
}

extern "C" int pgb_collide_ions(pgb_run* r) {
    if (!r) return PGB_ERR_ARG;
    int rc = need_particles(r);
    if (rc) return rc;
    if ((rc = set_device_step(r, r->time_step, 1))) return rc;
    if (pgb_launch_cx(r, 0, 0)) return PGB_ERR_CUDA;
    return sync_state(r);
}

extern "C" int pgb_contain_growth(pgb_run* r, int s) {
    if (!r || s < 0 || s > 1) return fail(r, PGB_ERR_ARG, "pgb_contain_growth: bad argument");
    int rc = sync_state(r);
    if (rc) return rc;
    long long live = r->hs->n[s] - r->hs->dead[s];
    long long lim = s == 0 ? r->p.size_to_check_e : r->p.size_to_check_i;
    if (!(live > lim)) return 0;
    if ((rc = set_device_step(r, r->time_step, 1))) return rc;
    if ((rc = pgb_launch_reduce(r, s))) return rc;
    return sync_state(r);
}

extern "C" int pgb_deposit(pgb_run* r, int s) {
    if (!r || s < 0 || s > 1) return fail(r, PGB_ERR_ARG, "pgb_deposit: bad argument");
    int rc = need_particles(r);
    if (rc) return rc;
    PGB_CK(r, cudaMemsetAsync(r->qacc[s], 0, sizeof(unsigned long long) * r->nx * r->ny, r->stream));
    if (pgb_launch_deposit(r, s) || pgb_launch_finalize(r, 1 << s, false)) return PGB_ERR_CUDA;
    return sync_state(r);
}

extern "C" int pgb_grid_rho(pgb_run* r) {
    if (!r) return PGB_ERR_ARG;
    int rc;
    if ((rc = set_device_step(r, r->time_step, 1))) return rc;
    if (pgb_launch_finalize(r, 0, false)) return PGB_ERR_CUDA;
    return sync_state(r);
}

extern "C" int pgb_poisson(pgb_run* r, int64_t t) {
    if (!r) return PGB_ERR_ARG;
    int rc = set_device_step(r, t, 1);
    if (rc) return rc;
    if (pgb_launch_rhs(r) || pgb_poisson_solve(r)) return PGB_ERR_CUDA;
    return sync_state(r);
}

extern "C" int pgb_efield(pgb_run* r) {
    if (!r) return PGB_ERR_ARG;
    if (pgb_launch_efield(r, 0)) return PGB_ERR_CUDA;
    return sync_state(r);
}

/* -------------------------------------------------------------- pgb_step */
/* event k marks the start of section k; event 5 the end of the step */
#define PROF_MARK(r, k) \
    do { if ((r)->prof_on) PGB_CK((r), cudaEventRecord((r)->prof_ev[k], (r)->stream)); } while (0)

/* One pic_run iteration in three parts.  The device counters ds->t
 * (particle phases) and ds->tf (field solve) select the random streams
 * and the right-wall potential, so the same launches can be replayed as
 * CUDA graphs for every step.
 *   step_mcc:       e_collisions::collision (pic.cpp:1071-1075): collision
 *                   tests, scattering and the list of ionization events;
 *                   on an ion step, charge exchange of the ions present
 *                   (ion_collisions::collision, pic.cpp:1102-1104, which
 *                   reads only ions and comes before their push); reads
 *                   no field
 *   step_particles: charge reset, electron push and deposit, ionization
 *                   products, injection, charge exchange of the ions they
 *                   appended, ion push, walls, population control
 *                   (pic.cpp:1080-1141), then ds->t += 1
 *   step_fields:    charge finalisation, grid_rho, grid_potential,
 *                   grid_electric_field (pic.cpp:1143-1161), then ds->tf += 1
 * Run in this order they are the reference's step.  The collisions of step
 * t+1 need the particles after step t's walls, not step t's fields, so the
 * pipelined path (issue_one_step) runs them while step t's field solve is
 * still in flight on the run's side stream.                              */
static int mcc_part(pgb_run* r, int leave_sms, bool ion_step) {
    if (!r->p.have_collisions) return 0;
    if (pgb_launch_mcc(r, leave_sms)) return PGB_ERR_CUDA;
    PROF_MARK(r, 9);
    /* the field solve beside the collisions ends before the collision test
     * does (0.11 against 0.15 ms at 513^2): the kernels after the test take
     * every SM (their blocks queue behind the solve's, which have the
     * higher priority, when it has not ended)                             */
    if (pgb_launch_scatter(r, 0)) return PGB_ERR_CUDA;
    PROF_MARK(r, 10);
    /* the ionization products are stored (so the event list is read) only
     * with steady-state walls or off ion steps; else only their number is */
    const bool products = r->p.steadystate || !ion_step;
    if (pgb_build_list(r, LIST_ION_EV, 0, !products)) return PGB_ERR_CUDA;
    PROF_MARK(r, 11);
    if (ion_step && pgb_launch_cx(r, 0, 0)) return PGB_ERR_CUDA;
    PROF_MARK(r, 12);
    return 0;
}
static int step_mcc(pgb_run* r, bool ion_step) { return mcc_part(r, 0, ion_step); }
/* beside a field solve, which needs SMs of its own (r->tune_field_sms) */
static int step_mcc_beside(pgb_run* r, bool ion_step) { return mcc_part(r, r->tune_field_sms, ion_step); }

static int step_particles(pgb_run* r, bool ion_step) {
    const bool coll = r->p.have_collisions != 0;
    const size_t G = (size_t)r->nx * r->ny;
    PGB_CK(r, cudaMemsetAsync(r->qacc[0], 0, sizeof(unsigned long long) * G, r->stream));
    PGB_CK(r, cudaMemsetAsync(r->qacc[1], 0, sizeof(unsigned long long) * G, r->stream));
    /* get_particle_electric_field + move_particles, charge deposit */
    PROF_MARK(r, 8);
    if (pgb_launch_push(r, 0, true)) return PGB_ERR_CUDA;
    PROF_MARK(r, 7);
    if (pgb_build_list(r, LIST_OUT_E, 0)) return PGB_ERR_CUDA;
    PROF_MARK(r, 1);
    if (coll) {
        /* the ionization products join after the push: an ion takes its
         * parent electron's new position                                */
        int store_e = r->p.steadystate ? 1 : 0;
        int store_i = (r->p.steadystate || !ion_step) ? 1 : 0;
        if (pgb_launch_ionize_appends(r, store_e, store_i)) return PGB_ERR_CUDA;
    }
    /* inject_more_particles: electrons are pushed as they are created */
    if (r->p.number_to_inject > 0 && pgb_launch_inject(r, 3, true)) return PGB_ERR_CUDA;
    PROF_MARK(r, 2);
    if (ion_step) {
        /* charge exchange of the ions appended since the collision pass:
         * without steady-state re-insertion only the injected ones (the
         * ionization products of an ion step are not stored), one block  */
        const bool appended = r->p.number_to_inject > 0 || r->p.steadystate;
        const bool few = !r->p.steadystate && r->p.number_to_inject <= 4096;
        if (coll && appended && pgb_launch_cx(r, few ? 2 : 1, 0)) return PGB_ERR_CUDA;
        PROF_MARK(r, 3);
        if (pgb_launch_push(r, 1, true)) return PGB_ERR_CUDA;
        if (pgb_build_list(r, LIST_OUT_I, 1)) return PGB_ERR_CUDA;
        PROF_MARK(r, 4);
        if (pgb_launch_walls(r, PGB_BOUNDARY_IONS)) return PGB_ERR_CUDA;
        if (pgb_launch_walls(r, PGB_BOUNDARY_ELECTRONS)) return PGB_ERR_CUDA;
    } else {
        PROF_MARK(r, 3);
        if (pgb_launch_deposit(r, 1)) return PGB_ERR_CUDA;
        if (r->p.steadystate && (pgb_launch_flag_outside(r, 1) || pgb_build_list(r, LIST_OUT_I, 1))) return PGB_ERR_CUDA;
        PROF_MARK(r, 4);
        if (pgb_launch_walls(r, PGB_BOUNDARY_ELECTRONS)) return PGB_ERR_CUDA;
    }
    /* contain_particle_growth: only when a species can exceed its limit */
    if (!r->p.steadystate) {
        for (int s = 0; s < 2; ++s) {
            long long lim = s == 0 ? r->p.size_to_check_e : r->p.size_to_check_i;
            if (r->sp[s].cap > lim) {
                int rc = sync_state(r);
                if (rc) return rc;
                if (r->hs->n[s] - r->hs->dead[s] > lim) {
                    if ((rc = pgb_launch_reduce(r, s))) return rc;
                    /* the reduction changes weights: rebuild both charges */
                    PGB_CK(r, cudaMemsetAsync(r->qacc[0], 0, sizeof(unsigned long long) * G, r->stream));
                    PGB_CK(r, cudaMemsetAsync(r->qacc[1], 0, sizeof(unsigned long long) * G, r->stream));
                    if (pgb_launch_deposit(r, 0) || pgb_launch_deposit(r, 1)) return PGB_ERR_CUDA;
                }
            }
        }
    }
    return pgb_launch_step_advance(r);
}

static int step_fields(pgb_run* r, bool) {
    /* collect_charge edge doubling, grid_rho, grid_potential, grid_electric_field */
    PROF_MARK(r, 5);
    if (pgb_launch_finalize(r, 3, true)) return PGB_ERR_CUDA;
    if (pgb_poisson_solve(r)) return PGB_ERR_CUDA;
    if (pgb_launch_efield(r, 1)) return PGB_ERR_CUDA;
    PROF_MARK(r, 6);
    return 0;
}

static int step_once(pgb_run* r, bool ion_step) {
    PROF_MARK(r, 0);
    int rc;
    if ((rc = step_mcc(r, ion_step)) || (rc = step_particles(r, ion_step)) || (rc = step_fields(r, ion_step)))
        return rc;
    return 0;
}

/* add the section times of the step just queued (waits for it) */
static int profile_collect(pgb_run* r) {
    PGB_CK(r, cudaEventSynchronize(r->prof_ev[6]));
    float ms[6];
    for (int k = 0; k < 6; ++k) PGB_CK(r, cudaEventElapsedTime(&ms[k], r->prof_ev[k], r->prof_ev[k + 1]));
    r->prof.ms_push_e += ms[0];
    float mk;
    PGB_CK(r, cudaEventElapsedTime(&mk, r->prof_ev[8], r->prof_ev[7]));
    r->prof.ms_push_e_kernel += mk;
    if (r->p.have_collisions) {
        PGB_CK(r, cudaEventElapsedTime(&mk, r->prof_ev[0], r->prof_ev[9]));
        r->prof.ms_collide_e += mk;
        PGB_CK(r, cudaEventElapsedTime(&mk, r->prof_ev[9], r->prof_ev[10]));
        r->prof.ms_scatter_e += mk;
        PGB_CK(r, cudaEventElapsedTime(&mk, r->prof_ev[11], r->prof_ev[12]));
        r->prof.ms_collide_ions += mk;
    }
    r->prof.ms_walls += ms[1] + ms[4];
    r->prof.ms_collide_ions += ms[2];
    r->prof.ms_push_i += ms[3];
    r->prof.ms_fields += ms[5];
    r->prof.steps += 1;
    return 0;
}

static void drop_graphs(pgb_run* r) {
    for (int k = 0; k < 8; ++k) {
        if (r->graph[k]) { cudaGraphExecDestroy(r->graph[k]); r->graph[k] = nullptr; }
        if (r->graph_a[k]) { cudaGraphExecDestroy(r->graph_a[k]); r->graph_a[k] = nullptr; }
        if (r->graph_b[k]) { cudaGraphExecDestroy(r->graph_b[k]); r->graph_b[k] = nullptr; }
        if (r->graph_m[k]) { cudaGraphExecDestroy(r->graph_m[k]); r->graph_m[k] = nullptr; }
        if (r->tmpl_a[k]) { cudaGraphDestroy(r->tmpl_a[k]); r->tmpl_a[k] = nullptr; }
        if (r->tmpl_b[k]) { cudaGraphDestroy(r->tmpl_b[k]); r->tmpl_b[k] = nullptr; }
    }
    if (r->graph_f) { cudaGraphExecDestroy(r->graph_f); r->graph_f = nullptr; }
    if (r->tmpl_f) { cudaGraphDestroy(r->tmpl_f); r->tmpl_f = nullptr; }
}

/* graphs are usable when no step needs a host decision: no profiling and
 * no species that could reach its reduction limit                       */
static bool graphs_ok(pgb_run* r) {
    if (!r->use_graphs || r->prof_on) return false;
    if (!r->p.steadystate && (r->sp[0].cap > r->p.size_to_check_e || r->sp[1].cap > r->p.size_to_check_i)) return false;
    return true;
}

/* capture fn(r, ion_step) as a graph; -1 if the launches cannot be captured.
 * keep: where to keep the captured template (else it is destroyed)     */
static int capture(pgb_run* r, int (*fn)(pgb_run*, bool), bool ion_step, cudaGraphExec_t* out, long long* nl,
                   cudaGraph_t* keep = nullptr) {
    cudaGraph_t g = nullptr;
    PGB_CK(r, cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
    long long l0 = r->launches;
    int rc = fn(r, ion_step);
    cudaError_t e = cudaStreamEndCapture(r->stream, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        r->launches = l0;
        return -1;
    }
    *nl = r->launches - l0;
    r->launches = l0;
    e = cudaGraphInstantiate(out, g, 0);
    if (keep && e == cudaSuccess) {
        if (*keep) cudaGraphDestroy(*keep);
        *keep = g;
    } else {
        cudaGraphDestroy(g);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return -1;
    }
    return 0;
}

/* run fn as graph *slot (captured on first use), or launch it directly
 * when graphs are off or cannot be captured                            */
static int replay(pgb_run* r, int (*fn)(pgb_run*, bool), bool ion_step, cudaGraphExec_t* slot, long long* nl,
                  cudaGraph_t* keep = nullptr) {
    if (graphs_ok(r) && !*slot && capture(r, fn, ion_step, slot, nl, keep)) r->use_graphs = 0;
    if (!*slot || !graphs_ok(r)) return fn(r, ion_step);
    PGB_CK(r, cudaGraphLaunch(*slot, r->stream));
    r->launches += *nl;
    return 0;
}

static int graph_key(pgb_run* r, bool ion_step) { return (ion_step ? 4 : 0) | (r->orient[0] << 1) | r->orient[1]; }

static int launch_step(pgb_run* r, bool ion_step) {
    const int key = graph_key(r, ion_step);
    return replay(r, step_once, ion_step, &r->graph[key], &r->graph_launches[key]);
}

/* the field solve of the last step issued, if it is still to be issued */
static int flush_fields(pgb_run* r) {
    if (!r->fields_pending) return 0;
    r->fields_pending = false;
    return replay(r, step_fields, false, &r->graph_f, &r->graph_f_launches, &r->tmpl_f);
}

/* pipelining needs collisions to overlap and graphs to replay the parts */
static bool pipelined(pgb_run* r) { return r->side_ok && r->p.have_collisions && r->use_graphs && graphs_ok(r); }

/* queue step r->time_step of r: host decisions (spatial sort or compaction),
 * then the step's launches or graphs; the host does not wait (except for
 * profiling and for a population check that may trigger a reduction).
 * Pipelined, the previous step's field solve (graph F) runs on the side
 * stream while this step's collisions (graph A) run on the run's stream;
 * the rest of the step (graph B) waits for both, and this step's field
 * solve is left pending.                                                */
/* a step that needs a host decision before its collisions: a spatial sort
 * or a compaction (both launch kernels between F and A)                  */
static bool host_work_due(pgb_run* r) {
    if (r->p.sort_interval > 0) return r->time_step % r->p.sort_interval == 0;
    for (int s = 0; s < 2; ++s)
        if (r->hs->dead[s] * 8 > r->hs->n[s] && r->hs->dead[s] > 0) return true;
    return false;
}

/* The pipelined step as one graph launch: the previous step's field solve
 * (F, its kernels at the side stream's top priority) beside this step's
 * collisions (A), then the other particle phases (B), built once per key
 * from the captured templates.  0: launched; 1: not available (graphs off
 * or a capture failed), use the separate graphs.                         */
static int launch_merged(pgb_run* r, bool ion_step) {
    const int key = graph_key(r, ion_step);
    if (!r->graph_m[key]) {
        if (!r->graph_f && capture(r, step_fields, false, &r->graph_f, &r->graph_f_launches, &r->tmpl_f)) return 1;
        if (!r->graph_a[key] &&
            capture(r, step_mcc_beside, ion_step, &r->graph_a[key], &r->graph_a_launches[key], &r->tmpl_a[key]))
            return 1;
        if (!r->graph_b[key] &&
            capture(r, step_particles, ion_step, &r->graph_b[key], &r->graph_b_launches[key], &r->tmpl_b[key]))
            return 1;
        if (!r->tmpl_f || !r->tmpl_a[key] || !r->tmpl_b[key]) return 1;
        /* F's kernels at the top priority, as on the side stream */
        size_t nn = 0;
        if (cudaGraphGetNodes(r->tmpl_f, nullptr, &nn) != cudaSuccess) return 1;
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn && cudaGraphGetNodes(r->tmpl_f, nodes.data(), &nn) != cudaSuccess) return 1;
        for (cudaGraphNode_t nd : nodes) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) {
                cudaLaunchAttributeValue v = {};
                v.priority = r->prio_hi;
                cudaGraphKernelNodeSetAttribute(nd, cudaLaunchAttributePriority, &v);
            }
        }
        cudaGetLastError();
        cudaGraph_t g = nullptr;
        cudaGraphNode_t nf, na, nb;
        bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
                  cudaGraphAddChildGraphNode(&nf, g, nullptr, 0, r->tmpl_f) == cudaSuccess &&
                  cudaGraphAddChildGraphNode(&na, g, nullptr, 0, r->tmpl_a[key]) == cudaSuccess;
        if (ok) {
            cudaGraphNode_t deps[2] = {nf, na};
            ok = cudaGraphAddChildGraphNode(&nb, g, deps, 2, r->tmpl_b[key]) == cudaSuccess &&
                 cudaGraphInstantiate(&r->graph_m[key], g, 0) == cudaSuccess;
        }
        if (g) cudaGraphDestroy(g);
        if (!ok) {
            cudaGetLastError();
            r->graph_m[key] = nullptr;
            return 1;
        }
    }
    PGB_CK(r, cudaGraphLaunch(r->graph_m[key], r->stream));
    r->launches += r->graph_f_launches + r->graph_a_launches[key] + r->graph_b_launches[key];
    return 0;
}

static int issue_one_step(pgb_run* r) {
    Range range("step");
    int rc;
    const bool pipe = pipelined(r);
    bool forked = false, merged = false;
    if (pipe && r->fields_pending && !host_work_due(r)) {
        rc = launch_merged(r, (r->time_step % r->dt_dti) == 0);
        if (rc < 0) return rc;
        merged = rc == 0;
        if (merged) r->fields_pending = true;   /* this step's field solve */
    }
    if (!merged && r->fields_pending) {
        if (pipe && !r->graph_f &&
            capture(r, step_fields, false, &r->graph_f, &r->graph_f_launches, &r->tmpl_f))
            r->use_graphs = 0;
        if (pipe && r->graph_f && pipelined(r)) {
            PGB_CK(r, cudaEventRecord(r->ev_fork, r->stream));
            PGB_CK(r, cudaStreamWaitEvent(r->side, r->ev_fork, 0));
            PGB_CK(r, cudaGraphLaunch(r->graph_f, r->side));
            r->launches += r->graph_f_launches;
            PGB_CK(r, cudaEventRecord(r->ev_join, r->side));
            r->fields_pending = false;
            forked = true;
        } else if ((rc = flush_fields(r))) {
            return rc;
        }
    }
    if (merged) {
        /* no sort or compaction is due: the step is queued */
    } else if (r->p.sort_interval > 0) {
        /* spatial sort (drops tombstones too): electrons every sort_interval
         * steps, ions every PGB_ION_SORT_FACTOR * sort_interval           */
        for (int s = 0; s < 2; ++s)
            if (r->time_step % ((long long)r->p.sort_interval * (s ? PGB_ION_SORT_FACTOR : 1)) == 0) {
                /* the padded layout needs n + pad slots; grow first if the
                 * (lazily read) count comes near the capacity              */
                const long long pad = sort_pad_slots(&r->p);
                if (r->hs->n[s] + r->hs->n[s] / 8 + pad > r->sp[s].cap) {
                    if ((rc = sync_state(r))) return rc;
                    const long long need = 2 * r->hs->n[s] + 65536 + pad;   /* > n + n/8 + pad */
                    if (r->hs->n[s] + r->hs->n[s] / 8 + pad > r->sp[s].cap &&
                        (rc = ensure_capacity(r, s, std::min<long long>(need, 0x7fffffffLL))))
                        return rc;
                }
                if (pgb_launch_sort(r, s)) return PGB_ERR_CUDA;
                r->orient[s] ^= 1;
            }
    } else {
        /* compact when tombstones exceed 1/8 of the slots (counts read lazily) */
        for (int s = 0; s < 2; ++s)
            if (r->hs->dead[s] * 8 > r->hs->n[s] && r->hs->dead[s] > 0) {
                if (pgb_launch_compact(r, s)) return PGB_ERR_CUDA;
                r->orient[s] ^= 1;
                r->hs->dead[s] = 0;
            }
    }
    if (r->prof_on) {
        if ((rc = sync_state(r))) return rc;
        r->prof.slots_e += r->hs->n[0];
        r->prof.slots_i += r->hs->n[1];
    }
    const bool ion_step = (r->time_step % r->dt_dti) == 0;
    if (merged) {
        /* A and B went with F in the step graph */
    } else if (pipe || forked) {
        const int key = graph_key(r, ion_step);
        if ((rc = replay(r, step_mcc_beside, ion_step, &r->graph_a[key], &r->graph_a_launches[key], &r->tmpl_a[key])))
            return rc;
        if (forked) PGB_CK(r, cudaStreamWaitEvent(r->stream, r->ev_join, 0));
        if ((rc = replay(r, step_particles, ion_step, &r->graph_b[key], &r->graph_b_launches[key], &r->tmpl_b[key])))
            return rc;
        r->fields_pending = true;
    } else {
        if ((rc = launch_step(r, ion_step))) return rc;
        if (r->prof_on && (rc = profile_collect(r))) return rc;
    }
    /* the graphs class sums after the field solve (pic.cpp:1189-1207) */
    if (r->gr.on && r->time_step >= r->gr.g.start_step && r->time_step < r->gr.g.end_step) {
        if ((rc = flush_fields(r)) || (rc = pgb_launch_graphs(r))) return rc;
    }
    r->time_step += 1;
    /* counters come back asynchronously; the host reads them only to
     * decide when to compact, which never changes results          */
    PGB_CK(r, cudaMemcpyAsync(r->hs, r->ds, sizeof(DevState), cudaMemcpyDeviceToHost, r->stream));
    return 0;
}

extern "C" int pgb_step(pgb_run* r, int32_t nsteps) {
    Range range("pgb_step");
    if (!r || nsteps < 0) return fail(r, PGB_ERR_ARG, "pgb_step: bad argument");
    int rc = need_particles(r);
    if (rc) return rc;
    int done = 0;
    while (done < nsteps) {
        int chunk = std::min<int>(nsteps - done, (int)r->phi_tab_cap);
        if ((rc = set_device_step(r, r->time_step, chunk))) return rc;
        for (int k = 0; k < chunk; ++k)
            if ((rc = issue_one_step(r))) return rc;
        if ((rc = flush_fields(r))) return rc;
        done += chunk;
    }
    return sync_state(r);
}

extern "C" int pgb_step_async(pgb_run* r, int32_t nsteps) {
    Range range("pgb_step_async");
    if (!r || nsteps < 0) return fail(r, PGB_ERR_ARG, "pgb_step_async: bad argument");
    int rc = need_particles(r);
    if (rc) return rc;
    int done = 0;
    while (done < nsteps) {
        int chunk = std::min<int>(nsteps - done, (int)r->phi_tab_cap);
        if ((rc = set_device_step(r, r->time_step, chunk))) return rc;
        for (int k = 0; k < chunk; ++k)
            if ((rc = issue_one_step(r))) return rc;
        if ((rc = flush_fields(r))) return rc;
        done += chunk;
    }
    return 0;
}

extern "C" int pgb_query(pgb_run* r, int32_t* idle) {
    if (!r || !idle) return fail(r, PGB_ERR_ARG, "pgb_query: bad argument");
    cudaError_t e = cudaStreamQuery(r->stream);
    if (e == cudaErrorNotReady) {
        *idle = 0;
        return 0;
    }
    if (e != cudaSuccess) return pgb_cuda_ok(r, e, "cudaStreamQuery") ? 0 : PGB_ERR_CUDA;
    *idle = 1;
    return sync_state(r);   /* idle: cheap, and reports device errors */
}

extern "C" int pgb_step_batch(pgb_run* const* runs, int32_t nruns, int32_t nsteps) {
    Range range("pgb_step_batch");
    if (!runs || nruns < 0 || nsteps < 0) return fail(nullptr, PGB_ERR_ARG, "pgb_step_batch: bad argument");
    for (int a = 0; a < nruns; ++a) {
        if (!runs[a]) return fail(nullptr, PGB_ERR_ARG, "pgb_step_batch: null run handle");
        for (int b = 0; b < a; ++b)
            if (runs[b] == runs[a]) return fail(nullptr, PGB_ERR_ARG, "pgb_step_batch: a run handle appears twice");
        int rc = need_particles(runs[a]);
        if (rc) return rc;
    }
    int done = 0;
    while (done < nsteps) {
        int chunk = nsteps - done;
        for (int a = 0; a < nruns; ++a) chunk = std::min<int>(chunk, (int)runs[a]->phi_tab_cap);
        for (int a = 0; a < nruns; ++a) {
            int rc = set_device_step(runs[a], runs[a]->time_step, chunk);
            if (rc) return rc;
        }
        /* one step of every run in turn: each run's work goes to its own
         * stream, so the kernels of different runs overlap on the GPU    */
        for (int k = 0; k < chunk; ++k)
            for (int a = 0; a < nruns; ++a) {
                int rc = issue_one_step(runs[a]);
                if (rc) return rc;
            }
        for (int a = 0; a < nruns; ++a) {
            int rc = flush_fields(runs[a]);
            if (rc) return rc;
        }
        done += chunk;
    }
    int first = 0;
    for (int a = 0; a < nruns; ++a) {
        int rc = sync_state(runs[a]);
        if (rc && !first) first = rc;
    }
    return first;
}

/* ------------------------------------------------------------ grids */
extern "C" int pgb_get_grid(pgb_run* r, int which, double* out, int64_t n) {
    if (!r || !out) return fail(r, PGB_ERR_ARG, "pgb_get_grid: bad argument");
    int64_t G = (int64_t)r->nx * r->ny, GE = (int64_t)(r->nx + 1) * (r->ny + 1);
    const double* src = nullptr;
    int64_t cnt = G;
    switch (which) {
        case PGB_GRID_Q_E: src = r->q[0]; break;
        case PGB_GRID_Q_I: src = r->q[1]; break;
        case PGB_GRID_RHO: src = r->rho; break;
        case PGB_GRID_PHI: src = r->phi; break;
        case PGB_GRID_EX: src = r->ex; cnt = GE; break;
        case PGB_GRID_EY: src = r->ey; cnt = GE; break;
        default: return fail(r, PGB_ERR_ARG, "pgb_get_grid: unknown grid");
    }
    if (n < cnt) return fail(r, PGB_ERR_ARG, "pgb_get_grid: buffer too small");
    PGB_CK(r, cudaMemcpyAsync(out, src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, r->stream));
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    return 0;
}

extern "C" int pgb_set_rho(pgb_run* r, const double* rho, int64_t n) {
    if (!r || !rho) return fail(r, PGB_ERR_ARG, "pgb_set_rho: bad argument");
    int64_t G = (int64_t)r->nx * r->ny;
    if (n < G) return fail(r, PGB_ERR_ARG, "pgb_set_rho: buffer too small");
    PGB_CK(r, cudaMemcpyAsync(r->rho, rho, sizeof(double) * G, cudaMemcpyHostToDevice, r->stream));
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    return 0;
}

extern "C" int pgb_get_counters(pgb_run* r, pgb_counters* c) {
    if (!r || !c) return fail(r, PGB_ERR_ARG, "pgb_get_counters: bad argument");
    int rc = sync_state(r);
    if (rc) return rc;
    const DevState& h = *r->hs;
    memset(c, 0, sizeof(*c));
    c->n_e = h.n[0] - h.dead[0];
    c->n_i = h.n[1] - h.dead[1];
    c->step = r->time_step;
    c->absorbed_e = h.stats[ST_ABS_E];
    c->absorbed_i = h.stats[ST_ABS_I];
    c->plopped = h.stats[ST_PLOP];
    c->reflected = h.stats[ST_REFL];
    c->backscattered = h.stats[ST_BACK];
    c->see_events = h.stats[ST_SEE_EV];
    c->see_emitted = h.stats[ST_SEE_EM];
    c->ion_see_emitted = h.stats[ST_ISEE_EM];
    c->elastic = h.stats[ST_ELASTIC];
    c->ionization = h.stats[ST_IONIZE];
    c->charge_exchange = h.stats[ST_CX];
    c->injected_e = h.stats[ST_INJ_E];
    c->injected_i = h.stats[ST_INJ_I];
    c->reductions_e = h.stats[ST_RED_E];
    c->reductions_i = h.stats[ST_RED_I];
    return 0;
}

extern "C" int pgb_get_stream(pgb_run* r, void** stream) {
    if (!r || !stream) return fail(r, PGB_ERR_ARG, "pgb_get_stream: bad argument");
    *stream = (void*)r->stream;
    return 0;
}

/* ------------------------------------------------------ launch shapes */
extern "C" int pgb_get_launch_config(pgb_run* r, pgb_launch_config* out) {
    if (!r || !out) return fail(r, PGB_ERR_ARG, "pgb_get_launch_config: bad argument");
    out->push_blocks_per_sm = r->tune_push_per_sm;
    out->field_sms = r->tune_field_sms;
    return 0;
}

extern "C" int pgb_set_launch_config(pgb_run* r, const pgb_launch_config* c) {
    if (!r || !c) return fail(r, PGB_ERR_ARG, "pgb_set_launch_config: bad argument");
    if (c->push_blocks_per_sm < 1 || c->push_blocks_per_sm > 64 || c->field_sms < 0 || c->field_sms >= r->sms)
        return fail(r, PGB_ERR_ARG, "pgb_set_launch_config: push_blocks_per_sm in [1, 64], field_sms in [0, SMs)");
    int rc = flush_fields(r);   /* a pending field solve was captured with the old shapes */
    if (rc) return rc;
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    r->tune_push_per_sm = c->push_blocks_per_sm;
    r->tune_field_sms = c->field_sms;
    drop_graphs(r);
    return 0;
}

extern "C" int pgb_autotune(pgb_run* r, int32_t steps, pgb_launch_config* best, double* ms_best, double* ms_all) {
    if (!r || steps < 1 || !best) return fail(r, PGB_ERR_ARG, "pgb_autotune: bad argument");
    static const int pushes[3] = {4, 8, 12}, fields[4] = {8, 16, 32, 48};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PGB_CK(r, cudaEventCreate(&e0));
    PGB_CK(r, cudaEventCreate(&e1));
    pgb_launch_config keep;
    pgb_get_launch_config(r, &keep);
    double bm = 1e300;
    int rc = 0, k = 0;
    for (int a = 0; a < 3 && !rc; ++a)
        for (int b = 0; b < 4 && !rc; ++b, ++k) {
            pgb_launch_config c;
            c.push_blocks_per_sm = pushes[a];
            c.field_sms = std::min(fields[b], r->sms - 1);
            if ((rc = pgb_set_launch_config(r, &c)) || (rc = pgb_step(r, 2))) break;   /* graphs captured */
            if (cudaEventRecord(e0, r->stream) != cudaSuccess) { rc = fail(r, PGB_ERR_CUDA, "pgb_autotune: event"); break; }
            if ((rc = pgb_step_async(r, steps))) break;
            float ms = 0.0f;
            if (cudaEventRecord(e1, r->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
                rc = fail(r, PGB_ERR_CUDA, "pgb_autotune: event");
                break;
            }
            const double per = (double)ms / steps;
            if (ms_all) ms_all[k] = per;
            if (per < bm) { bm = per; keep = c; }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc) rc = sync_state(r);
    int rc2 = pgb_set_launch_config(r, &keep);
    if (rc) return rc;
    if (rc2) return rc2;
    *best = keep;
    if (ms_best) *ms_best = bm;
    return 0;
}

extern "C" int pgb_set_profiling(pgb_run* r, int on) {
    if (!r) return PGB_ERR_ARG;
    if (on && !r->prof_ev_ok) {
        for (int k = 0; k < 13; ++k) PGB_CK(r, cudaEventCreate(&r->prof_ev[k]));
        r->prof_ev_ok = true;
    }
    memset(&r->prof, 0, sizeof(r->prof));
    r->prof_on = on ? 1 : 0;
    return 0;
}

extern "C" int pgb_get_profile(pgb_run* r, pgb_profile* out) {
    if (!r || !out) return fail(r, PGB_ERR_ARG, "pgb_get_profile: bad argument");
    *out = r->prof;
    out->launches = r->launches;
    return 0;
}

extern "C" int pgb_sync(pgb_run* r) {
    if (!r) return PGB_ERR_ARG;
    return sync_state(r);
}

