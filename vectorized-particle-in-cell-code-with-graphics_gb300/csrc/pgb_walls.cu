/*
 * Wall kernels and ion-neutral charge exchange.
 *
 * Reference path: boundary::ion_boundary (boundary.cpp:765-824),
 * boundary::e_boundary (boundary.cpp:581-677) with its yields
 * (boundary.cpp:281-337), reflect_electron, secondary_vel,
 * secondary_electrons, i_secondary_vel (boundary.cpp:374-756), the
 * steady-state pair re-insertion (boundary.cpp:854-1097) and
 * ion_collisions::collision (ion_collisions.cpp:255-308).
 *
 * The walls work from the ordered lists of outside particles that the push
 * kernels produced.  Pass 1 decides each wall event from the particle's own
 * random stream and applies the ones that modify a particle in place
 * (absorb, reflect, backscatter); an exclusive scan of the secondary counts
 * gives every new electron its slot and id in list order; pass 2 writes
 * the secondaries and removes their parents.  Results therefore do not
 * depend on thread scheduling.
 *
 * Event arithmetic (energies, angles, yields, speeds) is FP32, like the
 * particle state it starts from; positions are placed in FP64.  A wall
 * kernel handles a few wall hits per thread, so its time is the latency
 * of the longest event chain, and FP64 acos/pow/exp chains made it three
 * to four times longer.  Random numbers are the same in either precision
 * (pgb_u01f and pgb_u01d give the same value), so every comparison with a
 * draw sees the same draw.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "pgb_internal.h"
#include "pgb_physics.cuh"

struct WallArgs {
    Species e, i;
    DevState* ds;
    const int* list_e;
    const int* list_i;
    int* aux;                  /* per list entry: secondary count  */
    int* off;                  /* exclusive scan of aux            */
    unsigned long long* qacc_e;
    unsigned long long* qacc_i;
    int nx, ny;
    int ps;                    /* fraction bits of the positions */
    double dx, dy, dt;         /* boundary objects use DT (boundary.h:62) */
    double me, mi;
    double threshold, work_function;
    double e0, emax0, max_yield;
    int e_see, refl, back, ion_see;
    double vte, vti, xlength, ylength;
    uint64_t seed;
};

__device__ __forceinline__ void store_particle(const Species& S, long long slot, double x, double y, double vx,
                                               double vy, double vz, double dx, double dy, int ps) {
    S.xv[slot] = make_float4(pos_from_m(x, dx, ps), pos_from_m(y, dy, ps), (float)vx, (float)vy);
    S.vz[slot] = (float)vz;
}

/* boundary::secondary_vel (boundary.cpp:427-486) on a particle state */
__device__ void secondary_vel_f(const WallArgs& a, pgb_stream* st, double& x, double& y, float& vx, float& vy,
                                float& vz, float velocity, int jp, int kp) {
    const double lengthX = a.dx * a.nx, lengthY = a.dy * a.ny;
    const float two_pi = (float)(2.0 * PGB_PI);
    if (jp < 0 || jp >= a.nx) {
        float R = pgb_u01f(pgb_stream_u32(st)), Rphi = pgb_u01f(pgb_stream_u32(st)), Rchi = pgb_u01f(pgb_stream_u32(st));
        float chi = asinf(sqrtf(Rchi)), phi = two_pi * Rphi;
        float sc, cc, sp, cp;
        sincosf(chi, &sc, &cc);
        sincosf(phi, &sp, &cp);
        vx = fabsf(velocity * cc);
        vy = velocity * sc * cp;
        vz = velocity * sc * sp;
        x = (double)R * a.dt * fabs((double)vx);
        if (jp >= a.nx) { x = lengthX - x; vx = -fabsf(velocity * cc); }
    }
    if (kp < 0 || kp >= a.ny) {
        float R = pgb_u01f(pgb_stream_u32(st)), Rphi = pgb_u01f(pgb_stream_u32(st)), Rchi = pgb_u01f(pgb_stream_u32(st));
        float chi = asinf(sqrtf(Rchi)), phi = two_pi * Rphi;
        float sc, cc, sp, cp;
        sincosf(chi, &sc, &cc);
        sincosf(phi, &sp, &cp);
        vy = fabsf(velocity * cc);
        vx = velocity * sc * cp;
        vz = velocity * sc * sp;
        y = (double)R * a.dt * fabs((double)vy);
        if (kp >= a.ny) { y = lengthY - y; vy = -fabsf(velocity * cc); }
    }
}

/* sqrt(2 R q (THRESHOLD - 2 WORK_FUNCTION) / me) (boundary.cpp:510-512, 700-702) */
__device__ __forceinline__ float see_velocity(const WallArgs& a, float R) {
    return sqrtf(R * (float)(2.0 * PGB_CHARGE * (a.threshold - 2.0 * a.work_function) / a.me));
}

/* --------------------------------------------------------- ion walls */
/* i_impact_see_yield_Ar (boundary.cpp:310-317) */
__device__ __forceinline__ float ion_yield(const WallArgs& a, float energy) {
    if (!a.ion_see) return 0.0f;
    float y = 0.0f;
    if (energy >= 80.0f)
        y = 0.006f * energy / (1.0f + (energy / 10.0f)) +
            1.05e-4f * (sqrtf((energy - 80.0f)) / (1.0f + powf((energy / 8000.0f), 1.5f)));
    return y;
}

__global__ void k_iwall1(WallArgs a) {
    pgb_pdl_entry();
    const long long m = a.ds->list_n[LIST_OUT_I];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
        int slot = a.list_i[k];
        float4 p = a.i.xv[slot];
        float vx = p.z, vy = p.w, vz = a.i.vz[slot];
        float energy = (float)((0.5 / PGB_CHARGE) * a.mi) * (vx * vx + vy * vy + vz * vz);
        float yield = ion_yield(a, energy);
        pgb_stream st;
        pgb_stream_init(&st, a.seed, a.i.id[slot], (unsigned int)a.ds->t, PGB_STREAM_IWALL, 1);
        float R = pgb_u01f(pgb_stream_u32(&st));
        a.aux[k] = (R < yield) ? (int)floorf(yield) + 1 : 0;
    }
}

/* boundary::i_secondary_vel (boundary.cpp:687-756) */
__global__ void k_iwall2(WallArgs a) {
    pgb_pdl_entry();
    const long long m = a.ds->list_n[LIST_OUT_I];
    const long long ne0 = a.ds->n[0];
    const unsigned int id0 = a.ds->next_id[0];
    const double lengthX = a.dx * a.nx, lengthY = a.dy * a.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
        int slot = a.list_i[k];
        float4 p = a.i.xv[slot];
        int c = a.aux[k];
        if (c > 0) {
            double w = a.i.w[slot];
            int jp = pcell(p.x, a.ps), kp = pcell(p.y, a.ps);
            for (int j = 0; j < c; ++j) {
                long long es = ne0 + a.off[k] + j;
                if (es >= a.e.cap) { atomicOr(&a.ds->err, ERR_CAP_E); break; }
                unsigned int id = id0 + (unsigned int)(a.off[k] + j);
                pgb_stream st;
                pgb_stream_init(&st, a.seed, id, (unsigned int)a.ds->t, PGB_STREAM_SEE, 0);
                double x = 0.0, y = 0.0;
                float vx = 0.0f, vy = 0.0f, vz = 0.0f, ww = 1.0f;
                const float two_pi = (float)(2.0 * PGB_PI);
                if (jp < 0 || jp >= a.nx) {
                    float R = pgb_u01f(pgb_stream_u32(&st));
                    float velocity = see_velocity(a, R);
                    float Rphi = pgb_u01f(pgb_stream_u32(&st)), Rchi = pgb_u01f(pgb_stream_u32(&st));
                    float chi = asinf(sqrtf(Rchi)), phi = two_pi * Rphi;
                    float sc, cc, sp, cp;
                    sincosf(chi, &sc, &cc);
                    sincosf(phi, &sp, &cp);
                    vx = fabsf(velocity * cc);
                    vy = velocity * sc * cp;
                    vz = velocity * sc * sp;
                    ww = (float)w;
                    x = (double)R * a.dt * fabs((double)vx);
                    if (jp >= a.nx) { x = lengthX - x; vx = -fabsf(velocity * cc); }
                }
                if (kp < 0 || kp >= a.ny) {
                    float R = pgb_u01f(pgb_stream_u32(&st));
                    float velocity = see_velocity(a, R);
                    float Rphi = pgb_u01f(pgb_stream_u32(&st)), Rchi = pgb_u01f(pgb_stream_u32(&st));
                    float chi = asinf(sqrtf(Rchi)), phi = two_pi * Rphi;
                    float sc, cc, sp, cp;
                    sincosf(chi, &sc, &cc);
                    sincosf(phi, &sp, &cp);
                    vy = fabsf(velocity * cc);
                    vx = velocity * sc * cp;
                    vz = velocity * sc * sp;
                    ww = (float)w;
                    y = (double)R * a.dt * fabs((double)vy);
                    if (kp >= a.ny) { y = lengthY - y; vy = -fabsf(velocity * cc); }
                }
                store_particle(a.e, es, x, y, vx, vy, vz, a.dx, a.dy, a.ps);
                a.e.w[es] = ww;
                a.e.id[es] = id;
                float4 q = a.e.xv[es];
                maybe_deposit(a.qacc_e, a.nx, a.ny, a.ps, q.x, q.y, (float)ww);
            }
        }
        a.i.xv[slot].x = pos_dead();
    }
}

/* ---------------------------------------------------- electron walls */
struct WallState { float energy, angleX, angleY; int onX; };
/* e_impact_see_yield_v (boundary.cpp:281-300) */
__device__ __forceinline__ float e_yield(const WallArgs& a, const WallState& w) {
    if (!a.e_see) return 0.0f;
    const float twoPi = (float)(2.0 * PGB_PI);
    const float e0 = (float)a.e0, emax0 = (float)a.emax0;
    float v = (w.energy - e0) / (emax0 - e0);
    float k = (v > 1.0f) ? 0.25f : 0.62f;
    float ang = w.onX ? w.angleX : w.angleY;
    float ww = (w.energy - e0) / (emax0 * (1.0f + k * (ang * ang / twoPi)) - e0);
    return (float)a.max_yield * (1.0f + k * (ang * ang / twoPi)) * powf((ww * expf((1.0f - ww))), k);
}

/* outcome codes of one electron wall interaction */
enum { EW_STAY = 0, EW_ABSORB = 1, EW_SEE = 2, EW_RETRY = -1 };

__device__ int e_wall_event(const WallArgs& a, pgb_stream* st, double& x, double& y, float& vx, float& vy,
                            float& vz, int jp, int kp, int& nsec, int& kind) {
    const double lengthX = a.dx * a.nx, lengthY = a.dy * a.ny;
    const float me = (float)a.me;
    WallState w;
    w.onX = (jp < 0 || jp >= a.nx);
    float u2 = vx * vx + vy * vy + vz * vz;
    w.energy = (float)((0.5 / PGB_CHARGE) * a.me) * u2;
    float uu = 2.0f * w.energy / me;
    w.angleX = acosf(vx / (sqrtf(uu) + 1.0e-6f));
    w.angleY = acosf(vy / (sqrtf(uu) + 1.0e-6f));
    float yield = e_yield(a, w);
    float R = pgb_u01f(pgb_stream_u32(st));
    if (R < yield) {
        float refl = (a.refl && w.energy > 50.0f) ? 0.1f * yield : 0.0f;
        float back = (a.back && w.energy > 50.0f) ? 0.1f * yield : 0.0f;
        int no_inject = (int)floorf(fabsf((yield - refl - back))) + 1;
        const float offset = 1.0e-6f;
        R = pgb_u01f(pgb_stream_u32(st));
        if (R < refl / (yield + offset)) {
            /* reflect_electron (boundary.cpp:374-417) */
            double Rr = pgb_u01d(pgb_stream_u32(st));
            if (jp >= a.nx) { vx = -vx; x = lengthX - Rr * a.dt * fabs((double)vx); }
            else if (jp < 0) { vx = -vx; x = Rr * a.dt * fabs((double)vx); }
            if (kp >= a.ny) { vy = -vy; y = lengthY - Rr * a.dt * fabs((double)vy); }
            else if (kp < 0) { vy = -vy; y = Rr * a.dt * fabs((double)vy); }
            kind = ST_REFL;
            return EW_STAY;
        } else if (R > refl / yield && R < (refl + back) / (yield + offset)) {
            float R3 = (float)(pgb_stream_u32(st) % 10000u) / 10000.0f;
            float velocity = R3 * sqrtf((float)(2.0 * PGB_CHARGE / a.me) * w.energy);
            secondary_vel_f(a, st, x, y, vx, vy, vz, velocity, jp, kp);
            kind = ST_BACK;
            return EW_STAY;
        } else if (R > (refl + back) / (yield + offset)) {
            nsec = no_inject;
            return EW_SEE;
        }
        return EW_RETRY;
    }
    return EW_ABSORB;
}

__global__ void k_ewall1(WallArgs a) {
    pgb_pdl_entry();
    const long long m = a.ds->list_n[LIST_OUT_E];
    int cnt[4] = {0, 0, 0, 0};   /* absorbed, reflected, backscattered, see events */
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
        int slot = a.list_e[k];
        float4 p = a.e.xv[slot];
        double x = pos_m(p.x, a.ps, a.dx), y = pos_m(p.y, a.ps, a.dy);
        float vx = p.z, vy = p.w, vz = a.e.vz[slot];
        pgb_stream st;
        pgb_stream_init(&st, a.seed, a.e.id[slot], (unsigned int)a.ds->t, PGB_STREAM_EWALL, 0);
        int res = EW_RETRY, nsec = 0, kind = 0;
        const int jp = pcell(p.x, a.ps), kp = pcell(p.y, a.ps);
        for (int attempt = 0; attempt < 64 && res == EW_RETRY; ++attempt)
            res = e_wall_event(a, &st, x, y, vx, vy, vz, jp, kp, nsec, kind);
        if (res == EW_RETRY) res = EW_ABSORB;
        int c = 0;
        if (res == EW_STAY) {
            store_particle(a.e, slot, x, y, vx, vy, vz, a.dx, a.dy, a.ps);
            float4 q = a.e.xv[slot];
            maybe_deposit(a.qacc_e, a.nx, a.ny, a.ps, q.x, q.y, a.e.w[slot]);
            cnt[kind == ST_REFL ? 1 : 2]++;
        } else if (res == EW_ABSORB) {
            a.e.xv[slot].x = pos_dead();
            cnt[0]++;
        } else {
            c = nsec;
            cnt[3]++;
        }
        a.aux[k] = c;
    }
    const int idx[4] = {ST_ABS_E, ST_REFL, ST_BACK, ST_SEE_EV};
    int dead = cnt[0] + cnt[3];
    for (int d = 16; d; d >>= 1) dead += __shfl_down_sync(0xffffffffu, dead, d);
    if ((threadIdx.x & 31) == 0 && dead) atomicAdd((unsigned long long*)&a.ds->dead[0], (unsigned long long)dead);
    for (int q = 0; q < 4; ++q) {
        int v = cnt[q];
        for (int d = 16; d; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd((unsigned long long*)&a.ds->stats[idx[q]], (unsigned long long)v);
    }
}

/* boundary::secondary_electrons (boundary.cpp:494-529) */
__global__ void k_ewall2(WallArgs a) {
    pgb_pdl_entry();
    const long long m = a.ds->list_n[LIST_OUT_E];
    const long long ne0 = a.ds->n[0];
    const unsigned int id0 = a.ds->next_id[0];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
        int c = a.aux[k];
        if (c == 0) continue;
        int slot = a.list_e[k];
        float4 p = a.e.xv[slot];
        double px = pos_m(p.x, a.ps, a.dx), py = pos_m(p.y, a.ps, a.dy);
        float w = a.e.w[slot];
        int jpp = pcell(p.x, a.ps);
        for (int j = 0; j < c; ++j) {
            long long es = ne0 + a.off[k] + j;
            if (es >= a.e.cap) { atomicOr(&a.ds->err, ERR_CAP_E); break; }
            unsigned int id = id0 + (unsigned int)(a.off[k] + j);
            double x = 0.0, y = 0.0;
            float vx = 0.0f, vy = 0.0f, vz = 0.0f;
            if (jpp < 0 || jpp >= a.nx) x = px;
            else y = py;
            pgb_stream st;
            pgb_stream_init(&st, a.seed, id, (unsigned int)a.ds->t, PGB_STREAM_SEE, 0);
            float R = pgb_u01f(pgb_stream_u32(&st));
            float velocity = see_velocity(a, R);
            /* the new electron sits at the parent's x (left/right wall) or y */
            int jp = (jpp < 0 || jpp >= a.nx) ? jpp : 0;
            int kp = (jpp < 0 || jpp >= a.nx) ? 0 : pcell(p.y, a.ps);
            secondary_vel_f(a, &st, x, y, vx, vy, vz, velocity, jp, kp);
            store_particle(a.e, es, x, y, vx, vy, vz, a.dx, a.dy, a.ps);
            a.e.w[es] = w;
            a.e.id[es] = id;
            float4 q = a.e.xv[es];
            maybe_deposit(a.qacc_e, a.nx, a.ny, a.ps, q.x, q.y, w);
        }
        a.e.xv[slot].x = pos_dead();
    }
}

/* n, next id and statistics after a wall pass that appended `total` electrons */
__global__ void k_wall_commit(DevState* ds, const long long* total, int which, long long cap_e, int stat_emit) {
    pgb_pdl_entry();
    long long t = *total;
    long long v = ds->n[0] + t;
    ds->n[0] = v < cap_e ? v : cap_e;
    ds->next_id[0] += (unsigned int)t;
    long long m = ds->list_n[which == 0 ? LIST_OUT_I : LIST_OUT_E];
    if (which == 0) { ds->stats[ST_ABS_I] += m; ds->dead[1] += m; }
    ds->stats[stat_emit] += t;
}

/* ------------------------------------------------- steady-state walls */
/* boundary::steadyBoundaryX/Y (boundary.cpp:890-1082): per wall, the r-th
 * outside electron in list order is paired with the r-th outside ion, and
 * both are re-inserted at one random point (plop_particles,
 * boundary.cpp:854-878).  One CTA; lists are a small fraction of N.       */
__device__ __forceinline__ int steady_class(float c, int ncells, int ps) {
    if (pos_lt0(c)) return 1;               /* left / bottom  */
    if (pcell(c, ps) >= ncells) return 2;   /* right / top    */
    return 0;
}

__device__ __forceinline__ void block_scan2(int a, int b, int& ea, int& eb, int& ta, int& tb) {
    /* exclusive scans of two 0/1 flags over the block, plus totals */
    __shared__ int s_a[32], s_b[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned ma = __ballot_sync(0xffffffffu, a), mb = __ballot_sync(0xffffffffu, b);
    unsigned lt = (1u << lane) - 1u;
    if (lane == 0) { s_a[warp] = __popc(ma); s_b[warp] = __popc(mb); }
    __syncthreads();
    int pa = 0, pb = 0, sa = 0, sb = 0;
    for (int w = 0; w < nw; ++w) {
        if (w < warp) { pa += s_a[w]; pb += s_b[w]; }
        sa += s_a[w]; sb += s_b[w];
    }
    ea = pa + __popc(ma & lt);
    eb = pb + __popc(mb & lt);
    ta = sa; tb = sb;
    __syncthreads();
}

__global__ void __launch_bounds__(1024) k_steady(WallArgs a, int* ion_by_rank) {
    pgb_pdl_entry();
    const long long me_ = a.ds->list_n[LIST_OUT_E], mi_ = a.ds->list_n[LIST_OUT_I];
    __shared__ int s_plops;
    if (threadIdx.x == 0) s_plops = 0;
    for (int axis = 0; axis < 2; ++axis) {
        const int nc = axis == 0 ? a.nx : a.ny;
        /* ions: record slots by (class, rank); lo from the front, hi from the back */
        int cnt_lo = 0, cnt_hi = 0;
        for (long long b = 0; b < mi_; b += blockDim.x) {
            long long k = b + threadIdx.x;
            int cls = 0, slot = -1;
            if (k < mi_) {
                slot = a.list_i[k];
                float4 p = a.i.xv[slot];
                cls = steady_class(axis == 0 ? p.x : p.y, nc, a.ps);
            }
            int ea, eb, ta, tb;
            block_scan2(cls == 1, cls == 2, ea, eb, ta, tb);
            if (cls == 1) ion_by_rank[cnt_lo + ea] = slot;
            if (cls == 2) ion_by_rank[mi_ - 1 - (cnt_hi + eb)] = slot;
            cnt_lo += ta;
            cnt_hi += tb;
        }
        __syncthreads();
        /* electrons: pair by rank */
        int rlo = 0, rhi = 0;
        for (long long b = 0; b < me_; b += blockDim.x) {
            long long k = b + threadIdx.x;
            int cls = 0, slot = -1;
            if (k < me_) {
                slot = a.list_e[k];
                float4 p = a.e.xv[slot];
                cls = steady_class(axis == 0 ? p.x : p.y, nc, a.ps);
            }
            int ea, eb, ta, tb;
            block_scan2(cls == 1, cls == 2, ea, eb, ta, tb);
            int partner = -1;
            if (cls == 1 && rlo + ea < cnt_lo) partner = ion_by_rank[rlo + ea];
            if (cls == 2 && rhi + eb < cnt_hi) partner = ion_by_rank[mi_ - 1 - (rhi + eb)];
            if (partner >= 0) {
                pgb_stream st;
                pgb_stream_init(&st, a.seed, a.e.id[slot], (unsigned int)a.ds->t, PGB_STREAM_PLOP, 0);
                double rx = pgb_u01d(pgb_stream_u32(&st)), ry = pgb_u01d(pgb_stream_u32(&st));
                double x = (a.dx + rx * (a.xlength - 2.0 * a.dx));
                double y = (a.dy + ry * (a.ylength - 2.0 * a.dy));
                double evx = maxwell_fp64(&st, a.vte), ivx = maxwell_fp64(&st, a.vti);
                double evy = maxwell_fp64(&st, a.vte), ivy = maxwell_fp64(&st, a.vti);
                double evz = maxwell_fp64(&st, a.vte), ivz = maxwell_fp64(&st, a.vti);
                store_particle(a.e, slot, x, y, evx, evy, evz, a.dx, a.dy, a.ps);
                store_particle(a.i, partner, x, y, ivx, ivy, ivz, a.dx, a.dy, a.ps);
                float4 q = a.e.xv[slot];
                maybe_deposit(a.qacc_e, a.nx, a.ny, a.ps, q.x, q.y, a.e.w[slot]);
                q = a.i.xv[partner];
                maybe_deposit(a.qacc_i, a.nx, a.ny, a.ps, q.x, q.y, a.i.w[partner]);
                atomicAdd(&s_plops, 1);
            }
            rlo += ta;
            rhi += tb;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) a.ds->stats[ST_PLOP] += s_plops;
}

/* ================================================================ CX */
/* ion_collisions::collision (ion_collisions.cpp:255-308): per x column jp,
 * the probabilities of the eligible ions accumulate in slot order; the ion
 * that takes the column above 1 exchanges charge (its velocity becomes a
 * random neutral's) and the column restarts from 0.  The accumulator is
 * kept in fixed point (2^40 per unit), so sums are exact and independent
 * of summation order.  Pass 1: per tile of CX_TILE slots, per-column sums.
 * Pass 2: one warp per column walks the tiles, skipping whole tiles whose
 * sum cannot cross 1 and scanning the others element by element.
 * The tile sums are built in shared memory from two 32-bit atomics per ion
 * (the low 20 bits of its fixed-point probability, then the rest): 64-bit
 * shared atomics are compare-and-swap loops on this GPU, and the ions of a
 * sorted tile share a few dozen columns, so those loops contended (argon,
 * where every ion has a probability: 0.22 ms of a 0.46 ms step at 129^2).
 * A probability is at most 2^40, so with 2048 ions a tile neither 32-bit
 * sum can reach 2^32.                                                     */
#define CX_TILE PGB_CX_TILE
#define CX_ONE (1ll << 40)
static_assert((long long)CX_TILE << 20 <= (1ll << 31), "32-bit halves of the tile sums must not overflow");

struct CxArgs {
    Species i;
    DevState* ds;
    int nx, ny;
    int ps;                  /* fraction bits of the positions */
    float pcoef, ecoef;      /* DTI*1e-20*n_g, (0.5/CHARGE)*MI */
    CollConsts cc;
    long long* tile_sum;     /* [column][tile] fixed point, written where non-zero */
    long long ntl;           /* tiles capacity (row length of tile_sum) */
    unsigned long long* mask;   /* [column][mw]: bit t of the tiles with a non-zero sum */
    long long* total;        /* per-column sum of the pass                */
    int mw;
    long long* col_acc;      /* per-column accumulator carried across steps (fixed point) */
    const float* neut_i;     /* ion-neutral table (FP32) */
    uint64_t seed;
    int tail;                /* 0: slots [0, n), recording n in ds->n_cx;
                                1: the slots appended since, [ds->n_cx, n)  */
};

/* The slots one pass tests.  Charge exchange (ion_collisions.cpp:255-308)
 * walks the ions in slot order with one accumulator per column, so a pass
 * over the ions present when the step starts, run beside the previous
 * step's field solve, followed by a pass over the ions appended by
 * ionization and injection, continues every column's sum in the same order
 * and makes the same decisions as one pass over all of them.             */
__device__ __forceinline__ void cx_range(const CxArgs& a, long long& i0, long long& n) {
    n = a.ds->n[1];
    i0 = a.tail ? a.ds->n_cx : 0;
    if (i0 > n) i0 = n;
}

__device__ __forceinline__ long long cx_prob_fixed(const CxArgs& a, float4 p, float vz, int& col) {
    col = -1;
    if (is_dead(p.x)) return 0;
    int jp = pcell(p.x, a.ps), kp = pcell(p.y, a.ps);
    if (!(jp >= 0 && jp < a.nx && kp >= 0 && kp < a.ny)) return 0;
    col = jp;
    float u2 = __fadd_rn(__fadd_rn(__fmul_rn(p.z, p.z), __fmul_rn(p.w, p.w)), __fmul_rn(vz, vz));
    float energy = __fmul_rn(a.ecoef, u2);
    float s = sigma_cx(a.cc, energy);
    if (s == 0.0f) return 0;   /* P = -expm1f(-0) = 0 */
    float u = sqrtf(u2);
    /* no contraction: both CX passes must compute the same bits */
    float P = -expm1f(-__fmul_rn(__fmul_rn(u, a.pcoef), s));
    return __float2ll_rn(P * 1099511627776.0f);   /* P * 2^40, exact scaling */
}

/* charge_exchange_velocity (ion_collisions.cpp:209-221): ion i takes a
 * neutral's velocity from the table, picked by its CX stream            */
__device__ __forceinline__ void cx_exchange(const CxArgs& a, long long i) {
    pgb_stream st;
    pgb_stream_init(&st, a.seed, a.i.id[i], (unsigned int)a.ds->t, PGB_STREAM_CX, 1);
    (void)pgb_stream_u32(&st);
    int nn = a.cc.n_neutral;
    int index = (int)(pgb_stream_u32(&st) % (uint32_t)(nn - 1));
    float4 p = a.i.xv[i];
    p.z = a.neut_i[index];
    p.w = a.neut_i[nn + index];
    a.i.xv[i] = p;
    a.i.vz[i] = a.neut_i[2 * nn + index];
}

__global__ void __launch_bounds__(256) k_cx_tiles(CxArgs a) {
    pgb_pdl_entry();
    extern __shared__ unsigned int s_sum32[];
    unsigned int* const s_lo = s_sum32;          /* low 20 bits of the probabilities */
    unsigned int* const s_hi = s_sum32 + a.nx;   /* the rest (>> 20)                  */
    long long i0, n;
    cx_range(a, i0, n);
    const int ntiles = (int)((n - i0 + CX_TILE - 1) / CX_TILE);
    /* H+-H with the fit: vz is read only for the rare ion that needs it */
    const bool h_fit = a.cc.species == PGB_HYDROGEN && !a.cc.cx_const;
    /* the sums start at zero, and the scan of each tile zeroes what it reads */
    for (int c = threadIdx.x; c < a.nx; c += blockDim.x) {
        s_lo[c] = 0u;
        s_hi[c] = 0u;
    }
    __syncthreads();
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int any = 0;   /* an ion of this tile has a non-zero probability */
        /* four ions per thread in flight at a time */
        for (int k0 = threadIdx.x; k0 < CX_TILE; k0 += 4 * blockDim.x) {
            float4 p[4];
            float vz[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                long long i = i0 + (long long)t * CX_TILE + k0 + q * blockDim.x;
                p[q] = make_float4(pos_dead(), 0.f, 0.f, 0.f);
                vz[q] = 0.f;
                if (k0 + q * blockDim.x < CX_TILE && i < n) {
                    p[q] = a.i.xv[i];
                    if (!h_fit) vz[q] = a.i.vz[i];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (h_fit) {
                    /* the H fit is 0 where e / (1000 AMU) >= 2e10 (sig_h_cx),
                     * and e >= e_xy = ecoef (vx^2 + vy^2) also after rounding
                     * (adding vz^2 >= 0 and scaling by ecoef > 0 are monotone):
                     * such an ion's probability is 0 without its vz            */
                    const float e_xy = __fmul_rn(a.ecoef, __fadd_rn(__fmul_rn(p[q].z, p[q].z), __fmul_rn(p[q].w, p[q].w)));
                    if (e_xy * (1.0f / (1000.0f * 1.66054e-27f)) >= 2.0e10f) continue;
                    const long long i = i0 + (long long)t * CX_TILE + k0 + q * blockDim.x;
                    if (k0 + q * blockDim.x < CX_TILE && i < n) vz[q] = a.i.vz[i];
                }
                int col;
                long long pf = cx_prob_fixed(a, p[q], vz[q], col);
                if (col >= 0 && pf) {
                    atomicAdd(&s_lo[col], (unsigned int)(pf & 0xFFFFF));
                    const unsigned int hi = (unsigned int)(pf >> 20);
                    if (hi) atomicAdd(&s_hi[col], hi);
                    any = 1;
                }
            }
        }
        /* only non-zero sums are stored (marked in the column's bit mask and
         * added to its total): where no ion can exchange (the H fit is 0 at
         * any ion energy above 1e-14 eV) a tile has none and is not scanned */
        if (__syncthreads_or(any)) {
            for (int c = threadIdx.x; c < a.nx; c += blockDim.x) {
                const unsigned long long v = ((unsigned long long)s_hi[c] << 20) + s_lo[c];
                s_lo[c] = 0u;
                s_hi[c] = 0u;
                if (v) {
                    a.tile_sum[(long long)c * a.ntl + t] = (long long)v;
                    atomicOr(&a.mask[(long long)c * a.mw + (t >> 6)], 1ull << (t & 63));
                    atomicAdd((unsigned long long*)&a.total[c], v);
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(256) k_cx_walk(CxArgs a) {
    pgb_pdl_entry();
    const int lane = threadIdx.x & 31;
    const int col = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    long long i0, n;
    cx_range(a, i0, n);
    /* the tail pass starts where this one ends (k_cx_tiles has read n) */
    if (!a.tail && blockIdx.x == 0 && threadIdx.x == 0) a.ds->n_cx = n;
    if (col >= a.nx) return;
    const int ntiles = (int)((n - i0 + CX_TILE - 1) / CX_TILE);
    long long acc = a.col_acc[col];
    int fired = 0;
    const long long* row = a.tile_sum + (long long)col * a.ntl;
    unsigned long long* const mrow = a.mask + (long long)col * a.mw;
    /* most columns do not reach 1 in a step: test the column total first */
    const long long tot = a.total[col];
    if (acc + tot <= CX_ONE) {
        if (lane == 0) {
            a.col_acc[col] = acc + tot;
            a.total[col] = 0;
        }
        if (tot)
            for (int w = lane; w < (ntiles + 63) / 64; w += 32) mrow[w] = 0ull;
        return;
    }
    for (int t0 = 0; t0 < ntiles; t0 += 32) {
        int t = t0 + lane;
        long long s = (t < ntiles && ((mrow[t >> 6] >> (t & 63)) & 1ull)) ? row[t] : 0;
        /* inclusive prefix over the 32 tiles */
        long long ps = s;
        for (int d = 1; d < 32; d <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, ps, d);
            if (lane >= d) ps += y;
        }
        unsigned cross = __ballot_sync(0xffffffffu, acc + ps > CX_ONE);
        if (!cross) {
            acc += __shfl_sync(0xffffffffu, ps, 31);
            continue;
        }
        /* tiles before the first crossing cannot fire */
        int first = __ffs(cross) - 1;
        long long before = first ? __shfl_sync(0xffffffffu, ps, first - 1) : 0;
        acc += before;
        /* scan tile t0+first element by element, then continue after it */
        int tt = t0 + first;
        for (int b = 0; b < CX_TILE; b += 32) {
            long long i = i0 + (long long)tt * CX_TILE + b + lane;
            int c = -1;
            long long pf = 0;
            if (i < n) pf = cx_prob_fixed(a, a.i.xv[i], a.i.vz[i], c);
            unsigned match = __ballot_sync(0xffffffffu, c == col && pf > 0);
            while (match) {
                int l = __ffs(match) - 1;
                match &= match - 1;
                long long v = __shfl_sync(0xffffffffu, pf, l);
                acc += v;
                if (acc > CX_ONE) {
                    acc = 0;
                    if (lane == l) cx_exchange(a, i);
                    fired++;
                }
            }
        }
        /* resume with the tiles after tt */
        t0 = tt + 1 - 32;
    }
    __syncwarp();
    for (int w = lane; w < (ntiles + 63) / 64; w += 32) mrow[w] = 0ull;
    if (lane == 0) {
        a.col_acc[col] = acc;
        a.total[col] = 0;
        if (fired) atomicAdd((unsigned long long*)&a.ds->stats[ST_CX], (unsigned long long)fired);
    }
}

/* The charge exchange of the few ions appended since pass 1 (the injected
 * ones), in one block: their probabilities go to shared memory 256 at a
 * time, then each column's accumulator continues over them in slot order,
 * as k_cx_tiles + k_cx_walk would take it.                               */
__global__ void __launch_bounds__(256) k_cx_tail_small(CxArgs a) {
    pgb_pdl_entry();
    __shared__ long long s_pf[256];
    __shared__ int s_col[256];
    long long i0, n;
    cx_range(a, i0, n);
    int fired = 0;
    for (long long b = i0; b < n; b += 256) {
        const long long i = b + threadIdx.x;
        int col = -1;
        long long pf = 0;
        if (i < n) pf = cx_prob_fixed(a, a.i.xv[i], a.i.vz[i], col);
        s_pf[threadIdx.x] = pf;
        s_col[threadIdx.x] = pf ? col : -1;
        __syncthreads();
        const int cnt = (int)(n - b < 256 ? n - b : 256);
        for (int c = threadIdx.x; c < a.nx; c += blockDim.x) {
            long long acc = a.col_acc[c];
            for (int j = 0; j < cnt; ++j)
                if (s_col[j] == c) {
                    acc += s_pf[j];
                    if (acc > CX_ONE) {
                        acc = 0;
                        cx_exchange(a, b + j);
                        fired++;
                    }
                }
            a.col_acc[c] = acc;
        }
        __syncthreads();
    }
    for (int d = 16; d; d >>= 1) fired += __shfl_down_sync(0xffffffffu, fired, d);
    if ((threadIdx.x & 31) == 0 && fired) atomicAdd((unsigned long long*)&a.ds->stats[ST_CX], (unsigned long long)fired);
}

/* the ion walls without ion-impact emission: every listed ion is removed
 * (k_iwall1's yield is 0 there, so no secondary and nothing to scan)     */
__global__ void k_iwall_absorb(WallArgs a) {
    pgb_pdl_entry();
    const long long m = a.ds->list_n[LIST_OUT_I];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
        a.i.xv[a.list_i[k]].x = pos_dead();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ds->stats[ST_ABS_I] += m;
        a.ds->dead[1] += m;
    }
}

/* =========================================================== launchers */
static WallArgs wall_args(pgb_run* r) {
    WallArgs a;
    a.e = r->sp[0]; a.i = r->sp[1]; a.ds = r->ds;
    a.list_e = r->list[LIST_OUT_E]; a.list_i = r->list[LIST_OUT_I];
    a.aux = r->aux_i; a.off = r->aux_j;
    a.qacc_e = r->qacc[0]; a.qacc_i = r->qacc[1];
    a.nx = r->nx; a.ny = r->ny; a.ps = r->ps; a.dx = r->dx; a.dy = r->dy; a.dt = r->p.dt;
    a.me = r->p.electron_mass; a.mi = r->p.ion_mass;
    a.threshold = r->p.threshold; a.work_function = r->p.work_function;
    a.e0 = r->p.see_e0; a.emax0 = r->p.see_emax0; a.max_yield = r->p.see_max_yield;
    a.e_see = r->p.e_impact_see; a.refl = r->p.reflection; a.back = r->p.backscatter;
    a.ion_see = (r->p.species == PGB_ARGON && r->p.ion_impact_see) ? 1 : 0;
    a.vte = r->p.vte; a.vti = r->p.vti; a.xlength = r->p.xlength; a.ylength = r->p.ylength;
    a.seed = r->p.seed;
    return a;
}

__global__ void k_scan_list(const int* cnt, int* off, const long long* m_ptr, long long* total);

int pgb_launch_walls(pgb_run* r, int which) {
    WallArgs a = wall_args(r);
    int g = r->sms * 4;
    if (r->p.steadystate) {
        if (which == PGB_BOUNDARY_ELECTRONS) {
            PGB_CK(r, pgb_launch_pdl(k_steady, dim3(1), dim3(1024), 0, r->stream, a, r->aux_i));
            r->launches++;
            PGB_CK(r, cudaGetLastError());
        }
        return 0;
    }
    if (which == PGB_BOUNDARY_IONS && !a.ion_see) {
        PGB_CK(r, pgb_launch_pdl(k_iwall_absorb, dim3(g), dim3(256), 0, r->stream, a));
        r->launches++;
    } else if (which == PGB_BOUNDARY_IONS) {
        PGB_CK(r, pgb_launch_pdl(k_iwall1, dim3(g), dim3(256), 0, r->stream, a));
        r->launches++;
        PGB_CK(r, pgb_launch_pdl(k_scan_list, dim3(1), dim3(1024), 0, r->stream, r->aux_i, r->aux_j, &r->ds->list_n[LIST_OUT_I], &r->ds->list_n[LIST_SPARE]));
        r->launches++;
        PGB_CK(r, pgb_launch_pdl(k_iwall2, dim3(g), dim3(256), 0, r->stream, a));
        r->launches++;
        PGB_CK(r, pgb_launch_pdl(k_wall_commit, dim3(1), dim3(1), 0, r->stream, r->ds, &r->ds->list_n[LIST_SPARE], 0, r->sp[0].cap, ST_ISEE_EM));
        r->launches++;
    } else {
        PGB_CK(r, pgb_launch_pdl(k_ewall1, dim3(g), dim3(256), 0, r->stream, a));
        r->launches++;
        PGB_CK(r, pgb_launch_pdl(k_scan_list, dim3(1), dim3(1024), 0, r->stream, r->aux_i, r->aux_j, &r->ds->list_n[LIST_OUT_E], &r->ds->list_n[LIST_SPARE]));
        r->launches++;
        PGB_CK(r, pgb_launch_pdl(k_ewall2, dim3(g), dim3(256), 0, r->stream, a));
        r->launches++;
        PGB_CK(r, pgb_launch_pdl(k_wall_commit, dim3(1), dim3(1), 0, r->stream, r->ds, &r->ds->list_n[LIST_SPARE], 1, r->sp[0].cap, ST_SEE_EM));
        r->launches++;
    }
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_cx(pgb_run* r, int tail, int leave_sms) {
    CxArgs a;
    a.tail = tail ? 1 : 0;
    a.i = r->sp[1]; a.ds = r->ds; a.nx = r->nx; a.ny = r->ny; a.ps = r->ps;
    a.cc = pgb_coll_consts(r);
    a.pcoef = a.cc.i_pcoef; a.ecoef = a.cc.i_energy_coef;
    a.tile_sum = (long long*)r->cx_tile_sum;
    a.ntl = r->cx_tiles_cap;
    a.mask = r->cx_mask;
    a.total = r->cx_total;
    a.mw = r->cx_mask_words;
    a.col_acc = (long long*)r->prob_cx;
    a.neut_i = r->neut[1];
    a.seed = r->p.seed;
    if (tail == 2) {
        PGB_CK(r, pgb_launch_pdl(k_cx_tail_small, dim3(1), dim3(256), 0, r->stream, a));
        r->launches++;
        PGB_CK(r, cudaGetLastError());
        return 0;
    }
    const int sms = r->sms - leave_sms > 8 ? r->sms - leave_sms : 8;
    PGB_CK(r, pgb_launch_pdl(k_cx_tiles, dim3(sms * 4), dim3(256), 2 * sizeof(unsigned int) * r->nx, r->stream, a));
    r->launches++;
    int warps = 8;
    PGB_CK(r, pgb_launch_pdl(k_cx_walk, dim3((r->nx + warps - 1) / warps), dim3(warps * 32), 0, r->stream, a));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}
