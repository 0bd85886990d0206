/*
 * Particle kernels: electron-neutral collisions, gather + push + deposit,
 * ordered event lists, injection, ionization products, compaction, load
 * and dump.
 *
 * Reference path: e_collisions::collision (e_collisions.cpp:480-597),
 * particle::get_particle_electric_field + move_particles
 * (particle.cpp:870-1341, pic.cl:56-149), particle::collect_charge
 * (particle.cpp:663-858, pic.cl:22-52), particle::inject_more_particles
 * (particle.cpp:491-510).
 *
 * k_mcc reads each electron (16 B position/velocity, 4 B vz, 4 B id) for
 * the collision test and writes back only the ~5% whose velocity changes;
 * it reads no field, so it runs beside the previous step's field solve.
 * One pass of k_push then reads a particle once (16 B, plus 4 B vz with a
 * magnetic field and 4 B weight), gathers E bilinearly from the FP32 node
 * grid (L2 resident), pushes, deposits the new position into the int64
 * fixed-point charge grid and records wall crossings as per-tile ballot
 * words that keep slot order.  Grids are sized from the SM count and loop over
 * tiles, reading the particle count from device memory, so a step needs
 * no host round trip.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "pgb_internal.h"
#include "pgb_physics.cuh"

/* ------------------------------------------------------------ device state */
struct PushArgs {
    float4* xv;
    float* vz;
    float* w;
    const unsigned int* id;
    const float2* exy;
    unsigned long long* qacc;
    DevState* ds;
    int s;
    PushConsts pc;
    CollConsts cc;
    const float* neut;          /* electron-neutral table (FP32), 3 x N */
    const int4* pieces;         /* bin pieces of the last sort              */
    int nbx;                    /* bins per row                             */
    int* tl_out;                /* per-tile outside list              */
    int* tc_out;
    int* tl_ev;                 /* per-tile ionization-event list     */
    int* tc_ev;
};

/* gather (pic.cl:56-92) + push (pic.cl:95-149) of one particle in cell units */
__device__ __forceinline__ void gather_push_one(const PushConsts& pc, const float2* exy, float4& p, float& vz,
                                                bool& moved) {
    moved = false;
    /* jp < nx && x > 0 && kp < ny && y > 0; then the cell is a shift */
    if (pos_open_in(p.x, pc.nx, pc.ps) && pos_open_in(p.y, pc.ny, pc.ps)) {
        const int jp = pbits(p.x) >> pc.ps, kp = pbits(p.y) >> pc.ps;
        float wj = pfrac(p.x, pc.ps), wk = pfrac(p.y, pc.ps);
        float a4 = (1.0f - wj) * (1.0f - wk), a3 = wj * (1.0f - wk);
        float a2 = wk * (1.0f - wj), a1 = wj * wk;
        const float2* e = exy + (long long)kp * pc.nx + jp;
        float2 e0 = __ldg(e), e1 = __ldg(e + 1), e2 = __ldg(e + pc.nx), e3 = __ldg(e + pc.nx + 1);
        float Exp = a4 * e0.x + a3 * e1.x + a2 * e2.x + a1 * e3.x;
        float Eyp = a4 * e0.y + a3 * e1.y + a2 * e2.y + a1 * e3.y;
        float vx = p.z + pc.coef * Exp;
        float vy = p.w + pc.coef * Eyp;
        if (pc.bfield) {
            float vpar = pc.ca * vx + pc.sa * vy;
            float vperp = -pc.sa * vx + pc.ca * vy;
            float vperp_after = vperp * pc.co + pc.so * vz;
            vz = -vperp * pc.so + pc.co * vz;
            vx = pc.ca * vpar - pc.sa * vperp_after;
            vy = pc.sa * vpar + pc.ca * vperp_after;
        }
        vx += pc.coef * Exp;
        vy += pc.coef * Eyp;
        p.x = pos_step(p.x, pc.dtdx * vx);
        p.y = pos_step(p.y, pc.dtdy * vy);
        p.z = vx;
        p.w = vy;
        moved = true;
    }
}

/* electron-neutral collision test (e_collisions.cpp:504-551): both
 * probabilities come from the energy before any event; the decisions are
 * a bit set MCC_SCATTER | MCC_IONIZE.  The scattering continues the EMCC
 * stream after the test's first draw.                                    */
#define MCC_SCATTER 1
#define MCC_IONIZE 2
/* |v|^2 with its roundings spelled out: the collision test and the
 * scattering kernel must derive the same energy from the same velocity */
__device__ __forceinline__ float speed2(const float4& p, float vz) {
    return __fmaf_rn(vz, vz, __fmaf_rn(p.w, p.w, __fmul_rn(p.z, p.z)));
}
/* The test in two parts.  mcc_draw: in the domain (0 <= jp < nx,
 * 0 <= kp < ny), |v|^2 and the elastic test's uniform R, the first draw
 * of the electron's EMCC stream; false outside (no event).              */
__device__ __forceinline__ bool mcc_draw(const CollConsts& cc, unsigned int id, unsigned int step, int nx, int ny,
                                         int ps, const float4& p, float vz, float& u2, float& R) {
    if (!(pos_trunc_in(p.x, nx, ps) && pos_trunc_in(p.y, ny, ps))) return false;
    u2 = speed2(p, vz);
    pgb_stream st;
    pgb_stream_init(&st, cc.seed, id, step, PGB_STREAM_EMCC, 0);
    R = pgb_u01f(pgb_stream_u32(&st));
    return true;
}
/* whether mcc_decide can find an event: the elastic bound below with a
 * margin of 1e-5 over its own (about 3e-7 of FP32 rounding, the square
 * root included), written without the square root as u^2 K^2 > 4 R^2
 * (K^2 = cc.el_bound2), or an energy at or above the lowest at which the
 * ionization fit is non-zero (cc.ion_emin).  A false here is a decision
 * of no event that mcc_decide would take too.                           */
__device__ __forceinline__ bool mcc_candidate(const CollConsts& cc, float u2, float R) {
    return (R < 0.5f && u2 * cc.el_bound2 > (2.0f * R) * (2.0f * R)) || cc.e_energy_coef * u2 >= cc.ion_emin;
}
/* the decisions from |v|^2 and R (bit set MCC_SCATTER | MCC_IONIZE) */
__device__ __forceinline__ int mcc_decide(const CollConsts& cc, float u2, float R) {
    float energy = cc.e_energy_coef * u2;
    float u = sqrtf(u2);
    int ev = 0;
    /* P = 1 - exp(-x) is at most 1, so P > 2R cannot hold for R >= 1/2;
     * and P <= x <= u*pcoef*el_max, so with that bound (times 1 + 1e-6,
     * above the FP32 roundings of x and of expm1) at most 2R the event is
     * ruled out: the cross-section and the exponential are needed only
     * for the few electrons left, and every decision is the one the full
     * test would take                                                    */
    if (R < 0.5f && (u * cc.e_pcoef) * cc.el_max * 1.000001f > 2.0f * R) {
        float sel = sigma_el(cc, energy);
        float P = -expm1f(-(u * cc.e_pcoef * sel));
        if (P > 2.0f * R) ev |= MCC_SCATTER;
    }
    /* the ionization test is P = 1 - exp(-x) > 0 (e_collisions.cpp:546-551),
     * which holds exactly when x > 0 (for NaN x neither holds)          */
    float sio = sigma_ion(cc, energy);
    if (u * cc.e_pcoef * sio > 0.0f) ev |= MCC_IONIZE;
    return ev;
}

/* the full ionization of a parent electron (never reached while the
 * reference's energy units make the excess negative): kept out of line so
 * that it does not weigh on the push kernels' registers                  */
__device__ __noinline__ void mcc_ionize_full(const CollConsts& cc, const float* neut, unsigned int id, unsigned int step,
                                             float4& p, float& vz) {
    pgb_stream si;
    pgb_stream_init(&si, cc.seed, id, step, PGB_STREAM_IONIZE, 0);
    /* positions enter only the products; the parent keeps its position */
    IonizeOut o = ionize_f32(&si, neut, cc.n_neutral, cc, 0.0, 0.0, p.z, p.w, vz);
    p.z = (float)o.evx; p.w = (float)o.evy; vz = (float)o.evz;
}

/* e_collisions::ionization's effect on the parent electron, from its
 * velocity after any scattering (e_collisions.cpp:319-443)              */
__device__ __forceinline__ void mcc_ionize(const CollConsts& cc, const float* neut, unsigned int id, unsigned int step,
                                           float4& p, float& vz) {
    if (p.z * p.z + p.w * p.w + vz * vz < cc.ion_vcap * cc.ion_vcap) {
        /* (rm/2)(ve-vn)^2 - THRESHOLD < 0 at this speed for every neutral
         * of the table, so ionize_f32 would return NaN velocities from
         * sqrt of a negative number whatever it draws                   */
        p.z = p.w = vz = __int_as_float(0x7fffffff);
    } else {
        mcc_ionize_full(cc, neut, id, step, p, vz);
    }
}

/* add per-thread event counts (elastic, ionization) with one atomic per warp */
__device__ __forceinline__ void flush_stats(int (&st)[2], long long* stats) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        int v = st[k];
        for (int d = 16; d; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd((unsigned long long*)&stats[ST_ELASTIC + k], (unsigned long long)v);
    }
}

/* A tile's ordered list as bit masks: item k of thread t is slot
 * tile*TILE + k*THREADS + t, so word k*warps + w of the tile (the ballot of
 * warp w's item k) holds its slots in slot order, and the words in order
 * are the tile's list.  The tile's count goes through a shared counter:
 * one barrier per tile, and no scan (k_gather_lists expands the words).
 * s_cnt: two shared counters, zero at the kernel's start, used by turns
 * (it counts the calls of the block), so that a block's next tile can
 * count while thread 0 reads and clears this one's after the barrier.   */
static_assert(PGB_ITEMS * (PGB_PUSH_THREADS / 32) == 32, "a tile's list is 32 mask words");
__device__ __forceinline__ void tile_masks(const bool (&f)[PGB_ITEMS], int tile, unsigned* masks, int* tc,
                                           int* s_cnt, int& it) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int c = 0;
#pragma unroll
    for (int k = 0; k < PGB_ITEMS; ++k) {
        const unsigned m = __ballot_sync(0xffffffffu, f[k]);
        if (lane == 0) {
            masks[(long long)tile * 32 + k * (PGB_PUSH_THREADS / 32) + warp] = m;
            c += __popc(m);
        }
    }
    int* const cnt = &s_cnt[it & 1];
    if (lane == 0 && c) atomicAdd(cnt, c);
    __syncthreads();
    if (threadIdx.x == 0) {
        tc[tile] = *cnt;
        *cnt = 0;
    }
    ++it;
}

/* The shared deposit window holds each node's sum as one 32-bit word
 * (32-bit shared atomics are native, 64-bit ones are not).  A piece holds
 * at most PGB_PIECE_TILES * PGB_TILE = 4096 particles, and a contribution
 * of weight w < 1.99 is at most 1.99 * 2^19 + 1/2, so a node's sum stays
 * below 2^32.
 * Other weights deposit straight into the global int64 grid.  Both paths
 * add the same integer round(a*w*2^19).                                  */
#define WIN_NODES (PGB_WIN * PGB_WIN)
#define WIN_MAX_WEIGHT 1.99f
static_assert(PGB_PIECE_TILES * PGB_TILE <= 4096, "window sums are sized for 4096 particles per piece");
static_assert((PGB_FIX_SCALE * 1.99 + 1.0) * 4096.0 < 4294967296.0, "window sums must fit 32 bits");

/* round(v) to nearest even for 0 <= v < 2^22, as __float2int_rn: adding
 * 1.5 * 2^23 leaves v's integer part in the low mantissa bits, rounded by
 * the addition itself (1.5 * 2^23 is even, so ties go the same way)      */
__device__ __forceinline__ unsigned int round_small(float v) {
    return (unsigned int)__float_as_int(__fadd_rn(v, 12582912.0f)) - 0x4b400000u;
}

/* deposit into the CTA's shared window when the four nodes fall inside it,
 * else into the global grid.  Caller checks deposit_ok (x, y > 0).       */
__device__ __forceinline__ void deposit_win(unsigned long long* qacc, unsigned int* win, int ox, int oy, int nx,
                                            int ps, float xs, float ys, float w) {
    const int jp = pbits(xs) >> ps, kp = pbits(ys) >> ps;
    const int lx = jp - ox, ly = kp - oy;
    if (win && (unsigned)lx < (unsigned)(PGB_WIN - 1) && (unsigned)ly < (unsigned)(PGB_WIN - 1) && w >= 0.0f &&
        w < WIN_MAX_WEIGHT) {
        float wj = pfrac(xs, ps), wk = pfrac(ys, ps);
        float a4 = (1.0f - wj) * (1.0f - wk), a3 = wj * (1.0f - wk);
        float a2 = wk * (1.0f - wj), a1 = wj * wk;
        /* (a*w)*2^19 == a*(w*2^19) exactly: scaling by a power of two
         * commutes with rounding (w < 2: no overflow; a product below
         * FP32's normal range rounds to 0 either way)                     */
        const float wS = w * PGB_FIX_SCALE_F;
        const int k = ly * PGB_WIN + lx;
        /* below 2^21: the same integer as __float2ll_rn in deposit_cell */
        atomicAdd(&win[k], round_small(__fmul_rn(a4, wS)));
        atomicAdd(&win[k + 1], round_small(__fmul_rn(a3, wS)));
        atomicAdd(&win[k + PGB_WIN], round_small(__fmul_rn(a2, wS)));
        atomicAdd(&win[k + PGB_WIN + 1], round_small(__fmul_rn(a1, wS)));
    } else {
        deposit_cell(qacc, nx, ps, xs, ys, w);
    }
}

template <bool DEP>
__device__ __forceinline__ void push_tile(const PushArgs& a, const PushConsts& pc, int tile, long long n,
                                          unsigned int* win, int ox, int oy, int* s_cnt, int& it) {
    const long long base = (long long)tile * PGB_TILE;
    bool f[PGB_ITEMS];
    /* all loads of the thread's items first, so that they are in flight
     * together, then the pushes                                          */
    float4 p[PGB_ITEMS];
    float vz[PGB_ITEMS], w[PGB_ITEMS];
#pragma unroll
    for (int k = 0; k < PGB_ITEMS; ++k) {
        long long i = base + k * PGB_PUSH_THREADS + threadIdx.x;
        p[k] = make_float4(pos_dead(), 0.0f, 0.0f, 0.0f);
        vz[k] = 0.0f;
        w[k] = 0.0f;
        if (i < n) {
            p[k] = a.xv[i];
            if (pc.bfield) vz[k] = a.vz[i];
            if (DEP) w[k] = a.w[i];
        }
    }
#pragma unroll
    for (int k = 0; k < PGB_ITEMS; ++k) {
        f[k] = false;
        long long i = base + k * PGB_PUSH_THREADS + threadIdx.x;
        if (is_dead(p[k].x)) continue;
        bool moved;
        gather_push_one(pc, a.exy, p[k], vz[k], moved);
        if (moved) a.xv[i] = p[k];
        if (pc.bfield && moved) a.vz[i] = vz[k];
        if (DEP && deposit_ok(p[k].x, p[k].y, pc.nx, pc.ny, pc.ps))
            deposit_win(a.qacc, win, ox, oy, pc.nx, pc.ps, p[k].x, p[k].y, w[k]);
        f[k] = pc.steady ? outside_steady(p[k].x, p[k].y, pc.nx, pc.ny, pc.ps)
                         : outside_absorbing(p[k].x, p[k].y, pc.nx, pc.ny, pc.ps);
    }
    tile_masks(f, tile, (unsigned*)a.tl_out, a.tc_out, s_cnt, it);
}

/* Work items: the bin pieces of the last sort (tiles of one bin, deposited
 * through a shared window), then every tile after the sorted region.     */
template <bool DEP>
__global__ void __launch_bounds__(PGB_PUSH_THREADS, 4) k_push(PushArgs a) {
    pgb_pdl_entry();
    __shared__ unsigned int s_win[WIN_NODES];
    const long long n = a.ds->n[a.s];
    const int ntiles = (int)((n + PGB_TILE - 1) / PGB_TILE);
    const int npieces = a.ds->n_pieces[a.s];
    const int tile0 = (int)a.ds->sorted_tiles[a.s];
    const int nitems = npieces + (ntiles > tile0 ? ntiles - tile0 : 0);
    const PushConsts pc = a.pc;
    __shared__ int s_cnt[2];
    int it = 0;
    if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
    /* the window starts zeroed; each flush leaves it zeroed again */
    if (DEP && npieces > 0)
        for (int k = threadIdx.x; k < WIN_NODES; k += blockDim.x) s_win[k] = 0u;
    __syncthreads();
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        if (item < npieces) {
            int4 pc4 = a.pieces[item];
            unsigned int* win = nullptr;
            int ox = 0, oy = 0;
            if (DEP && pc4.z >= 0) {
                win = s_win;
                ox = (pc4.z % a.nbx) * PGB_BIN - PGB_HALO;
                oy = (pc4.z / a.nbx) * PGB_BIN - PGB_HALO;
            }
            for (int t = pc4.x; t < pc4.x + pc4.y && t < ntiles; ++t)
                push_tile<DEP>(a, pc, t, n, win, ox, oy, s_cnt, it);
            if (win) {
                __syncthreads();
                /* a warp per window row, a lane per node: add the non-zero
                 * sums to the grid and zero them for the next piece        */
                const int lane = threadIdx.x & 31;
                for (int ry = threadIdx.x >> 5; ry < PGB_WIN; ry += PGB_PUSH_THREADS / 32) {
                    const int gy = oy + ry;
                    unsigned long long* qrow = a.qacc + (long long)gy * pc.nx;
                    for (int rx = lane; rx < PGB_WIN; rx += 32) {
                        const unsigned int v = s_win[ry * PGB_WIN + rx];
                        if (v) {
                            s_win[ry * PGB_WIN + rx] = 0u;
                            const int gx = ox + rx;
                            if (gx >= 0 && gy >= 0 && gx < pc.nx && gy < pc.ny)
                                atomicAdd(qrow + gx, (unsigned long long)v);
                        }
                    }
                }
                __syncthreads();
            }
        } else {
            push_tile<DEP>(a, pc, tile0 + (item - npieces), n, nullptr, 0, 0, s_cnt, it);
        }
    }
}

/* flag-only pass (wall classification without a push) */
__global__ void __launch_bounds__(PGB_PUSH_THREADS) k_flag(const float4* xv, DevState* ds, int s, int nx, int ny,
                                                           int ps, int steady, int* tl, int* tc) {
    pgb_pdl_entry();
    const long long n = ds->n[s];
    const int ntiles = (int)((n + PGB_TILE - 1) / PGB_TILE);
    __shared__ int s_cnt[2];
    int it = 0;
    if (threadIdx.x < 2) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long base = (long long)tile * PGB_TILE;
        bool f[PGB_ITEMS];
#pragma unroll
        for (int k = 0; k < PGB_ITEMS; ++k) {
            long long i = base + k * PGB_PUSH_THREADS + threadIdx.x;
            f[k] = false;
            if (i >= n) continue;
            float4 p = xv[i];
            if (is_dead(p.x)) continue;
            f[k] = steady ? outside_steady(p.x, p.y, nx, ny, ps) : outside_absorbing(p.x, p.y, nx, ny, ps);
        }
        tile_masks(f, tile, (unsigned*)tl, tc, s_cnt, it);
    }
}

/* standalone deposit (particle::collect_charge) */
__global__ void __launch_bounds__(256) k_deposit(const float4* xv, const float* w, DevState* ds, int s, int nx, int ny,
                                                 int ps, unsigned long long* qacc) {
    pgb_pdl_entry();
    const long long n = ds->n[s];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 p = xv[i];
        if (deposit_ok(p.x, p.y, nx, ny, ps)) deposit_cell(qacc, nx, ps, p.x, p.y, w[i]);
    }
}

/* e_collisions::collision (e_collisions.cpp:480-597) in two kernels, the
 * first of a step.  They read no field, so they run while the previous
 * step's field solve is still in flight.
 *   k_mcc      the collision test of every electron; the ionizations of
 *              electrons that do not also scatter; the ordered per-tile
 *              list of ionization events; the scattering events (about one
 *              electron in twenty) appended, unordered, to a dense list
 *   k_scatter  one thread per listed event: the scattering, then the
 *              ionization of the parent if it also ionizes
 * Each event touches only its own electron and draws from that electron's
 * stream, so the order of the scattering list changes nothing.
 *
 * A block is MCC_GROUPS independent groups of 256 threads, each with its
 * own list scratch and named barrier, each taking one tile at a time.  At
 * 64 registers a thread the block fills an SM's register file, so a grid
 * of sms - k blocks leaves k SMs wholly free: the field solve's one-CTA
 * multigrid (1024 threads) needs an SM of its own.                       */
#define MCC_GROUPS 4
#define MCC_THREADS (MCC_GROUPS * PGB_PUSH_THREADS)
#define MCC_ION_BIT 0x80000000u
struct MccGroupSmem {
    int off[PGB_ITEMS][PGB_PUSH_THREADS / 32];    /* ionization events per (item, warp) */
    int soff[PGB_ITEMS][PGB_PUSH_THREADS / 32];   /* scattering events per (item, warp) */
    unsigned long long sbase;                      /* the tile's first scattering-list entry */
    int qn;                                        /* candidates queued                      */
    float qu2[PGB_TILE];                           /* candidate |v|^2, R and tile position   */
    float qr[PGB_TILE];
    unsigned short qi[PGB_TILE];
    unsigned char ev[PGB_TILE];                    /* decisions by tile position             */
};
static_assert(MCC_GROUPS * sizeof(MccGroupSmem) <= 48 * 1024, "static shared memory");
__device__ __forceinline__ void group_sync(int g) {
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "n"(PGB_PUSH_THREADS) : "memory");
}
/* A tile in three passes.  (1) Every electron: the domain test, |v|^2,
 * the Philox draw R and mcc_candidate; the candidates (about one in ten
 * at a few eV) are queued.  (2) The queue, one candidate per thread: the
 * cross-sections, the exponential and the decisions of mcc_decide, so
 * that the fits run densely instead of in every warp that holds one
 * candidate.  (3) Every electron takes its decisions back in slot order
 * for the lists.                                                         */
__global__ void __launch_bounds__(MCC_THREADS, 1) k_mcc(PushArgs a, int* scat) {
    pgb_pdl_entry();
    __shared__ MccGroupSmem s_grp[MCC_GROUPS];
    const int g = threadIdx.x / PGB_PUSH_THREADS, t = threadIdx.x % PGB_PUSH_THREADS;
    const int lane = t & 31, warp = t >> 5;
    const unsigned lt = (1u << lane) - 1u;
    MccGroupSmem& S = s_grp[g];
    const long long n = a.ds->n[0];
    const int ntiles = (int)((n + PGB_TILE - 1) / PGB_TILE);
    const unsigned step = (unsigned)a.ds->t;
    int st_loc[2] = {0, 0};
    if (t == 0) S.qn = 0;
    group_sync(g);
    for (int tile = blockIdx.x * MCC_GROUPS + g; tile < ntiles; tile += gridDim.x * MCC_GROUPS) {
        const long long base = (long long)tile * PGB_TILE;
        /* (1) all loads of the thread's items first, then the draws */
        float4 pa[PGB_ITEMS];
        float vza[PGB_ITEMS];
        unsigned int ida[PGB_ITEMS];
#pragma unroll
        for (int k = 0; k < PGB_ITEMS; ++k) {
            long long i = base + k * PGB_PUSH_THREADS + t;
            pa[k] = make_float4(pos_dead(), 0.0f, 0.0f, 0.0f);
            vza[k] = 0.0f;
            ida[k] = 0u;
            if (i < n) {
                pa[k] = a.xv[i];
                vza[k] = a.vz[i];
                ida[k] = a.id[i];
            }
        }
        unsigned cand = 0;   /* bit k: item k is queued */
#pragma unroll
        for (int k = 0; k < PGB_ITEMS; ++k) {
            float u2 = 0.0f, R = 1.0f;
            bool c = false;
            if (!is_dead(pa[k].x) && mcc_draw(a.cc, ida[k], step, a.pc.nx, a.pc.ny, a.pc.ps, pa[k], vza[k], u2, R))
                c = mcc_candidate(a.cc, u2, R);
            const unsigned cm = __ballot_sync(0xffffffffu, c);
            int qb = 0;
            if (lane == 0 && cm) qb = atomicAdd(&S.qn, __popc(cm));
            qb = __shfl_sync(0xffffffffu, qb, 0);
            if (c) {
                const int q = qb + __popc(cm & lt);
                S.qu2[q] = u2;
                S.qr[q] = R;
                S.qi[q] = (unsigned short)(k * PGB_PUSH_THREADS + t);
                cand |= 1u << k;
            }
        }
        group_sync(g);
        /* (2) the queued candidates, densely */
        {
            const int qn = S.qn;
            for (int q = t; q < qn; q += PGB_PUSH_THREADS) S.ev[S.qi[q]] = (unsigned char)mcc_decide(a.cc, S.qu2[q], S.qr[q]);
        }
        group_sync(g);
        /* (3) decisions back in slot order */
        if (t == 0) S.qn = 0;   /* every thread has read it before the barrier */
        bool f[PGB_ITEMS], sc[PGB_ITEMS];
#pragma unroll
        for (int k = 0; k < PGB_ITEMS; ++k) {
            const int i = (int)(base + k * PGB_PUSH_THREADS + t);
            const int ev = (cand >> k) & 1u ? S.ev[k * PGB_PUSH_THREADS + t] : 0;
            sc[k] = (ev & MCC_SCATTER) != 0;
            f[k] = (ev & MCC_IONIZE) != 0;
            st_loc[0] += sc[k] ? 1 : 0;
            st_loc[1] += f[k] ? 1 : 0;
            /* an ionization without scattering is applied here (rare: the
             * electron is read again rather than held through the passes) */
            if (f[k] && !sc[k]) {
                float4 p = a.xv[i];
                float vz = a.vz[i];
                mcc_ionize(a.cc, a.neut, a.id[i], step, p, vz);
                a.xv[i] = p;
                a.vz[i] = vz;
            }
        }
        /* the tile's ionization events in slot order (as tile_masks), and its
         * scattering events appended to the dense list with one counter
         * update for the tile (a counter update per warp serialised some
         * 400k atomics on one address per launch)                        */
        unsigned m[PGB_ITEMS], ms[PGB_ITEMS];
#pragma unroll
        for (int k = 0; k < PGB_ITEMS; ++k) {
            m[k] = __ballot_sync(0xffffffffu, f[k]);
            ms[k] = __ballot_sync(0xffffffffu, sc[k]);
            if (lane == 0) {
                S.off[k][warp] = __popc(m[k]);
                S.soff[k][warp] = __popc(ms[k]);
            }
        }
        group_sync(g);
        /* exclusive scans of the group's 32 (item, warp) counts by its first
         * warp, in (item, warp) order, which is slot order                */
        static_assert(PGB_ITEMS * (PGB_PUSH_THREADS / 32) == 32, "one count per lane");
        if (warp == 0) {
            int* const io = &S.off[0][0];
            int* const so = &S.soff[0][0];
            const int c = io[lane], d = so[lane];
            int x = c, y = d;
#pragma unroll
            for (int dd = 1; dd < 32; dd <<= 1) {
                const int xu = __shfl_up_sync(0xffffffffu, x, dd), yu = __shfl_up_sync(0xffffffffu, y, dd);
                if (lane >= dd) { x += xu; y += yu; }
            }
            io[lane] = x - c;
            so[lane] = y - d;
            if (lane == 31) {
                a.tc_ev[tile] = x;
                S.sbase = y ? atomicAdd(&a.ds->scat_n, (unsigned long long)y) : 0ull;
            }
        }
        group_sync(g);
#pragma unroll
        for (int k = 0; k < PGB_ITEMS; ++k) {
            const int i = (int)(base + k * PGB_PUSH_THREADS + t);
            /* the ionization events as the tile's mask words (tile_masks) */
            if (lane == 0) ((unsigned*)a.tl_ev)[(long long)tile * 32 + k * (PGB_PUSH_THREADS / 32) + warp] = m[k];
            if (sc[k]) scat[S.sbase + S.soff[k][warp] + __popc(ms[k] & lt)] = (int)((unsigned)i | (f[k] ? MCC_ION_BIT : 0u));
        }
        group_sync(g);
    }
    flush_stats(st_loc, a.ds->stats);
}

__global__ void __launch_bounds__(MCC_THREADS, 1) k_scatter(PushArgs a, const int* scat) {
    pgb_pdl_entry();
    const long long m = (long long)a.ds->scat_n;
    const unsigned step = (unsigned)a.ds->t;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < m; r += (long long)gridDim.x * blockDim.x) {
        const unsigned e = (unsigned)scat[r];
        const int slot = (int)(e & ~MCC_ION_BIT);
        float4 p = a.xv[slot];
        float vz = a.vz[slot];
        const unsigned int id = a.id[slot];
        const float energy = a.cc.e_energy_coef * speed2(p, vz);
        pgb_stream st;
        pgb_stream_init(&st, a.cc.seed, id, step, PGB_STREAM_EMCC, 0);
        (void)pgb_stream_u32(&st);   /* the collision test's draw */
        scatter_f32(&st, a.neut, a.cc.n_neutral, energy, (float)a.cc.reduced_mass, p.z, p.w, vz);
        if (e & MCC_ION_BIT) mcc_ionize(a.cc, a.neut, id, step, p, vz);
        a.xv[slot] = p;
        a.vz[slot] = vz;
    }
}

/* the last kernel of a step's particle phases moves the step counter on */
__global__ void k_step_advance(DevState* ds) {
    pgb_pdl_entry();
    ds->t += 1;
}

/* ------------------------------------------------------------ scans */
/* exclusive scan of cnt[0..m) into off[]; returns the total.  One block of
 * 1024 threads, 8 consecutive items per thread and 8192 entries per pass.
 * (32 items per thread, one pass for the bench's 16.7K tiles, measured
 * slower: a warp's load then touches 32 lines instead of 8.)            */
#define SCAN_ITEMS 8
__device__ __forceinline__ long long block_excl_scan(const int* cnt, int* off, long long m, long long carry0) {
    __shared__ long long s_warp[32];
    __shared__ long long s_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = carry0;
    __syncthreads();
    for (long long b = 0; b < m; b += SCAN_ITEMS * 1024) {
        long long i0 = b + SCAN_ITEMS * (long long)threadIdx.x;
        int v[SCAN_ITEMS];
        long long sum = 0;
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS; ++q) v[q] = (i0 + q < m) ? cnt[i0 + q] : 0;
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS; ++q) sum += v[q];
        long long x = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, d);
            if (lane >= d) x += y;
        }
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            long long t = s_warp[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, t, d);
                if (lane >= d) t += y;
            }
            s_warp[lane] = t;
        }
        __syncthreads();
        long long excl = s_carry + (warp ? s_warp[warp - 1] : 0) + x - sum;
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS; ++q) {
            if (i0 + q < m) off[i0 + q] = (int)excl;
            excl += v[q];
        }
        __syncthreads();
        if (threadIdx.x == 0) s_carry += s_warp[31];
        __syncthreads();
    }
    return s_carry;
}

__global__ void __launch_bounds__(1024) k_scan_small(const int* cnt, int* off, const long long* n_ptr, long long m_const,
                                                     long long* total) {
    pgb_pdl_entry();
    /* n_ptr: particle count whose tiles are scanned; else m_const entries */
    const long long m = n_ptr ? (*n_ptr + PGB_TILE - 1) / PGB_TILE : m_const;
    long long t = block_excl_scan(cnt, off, m, 0);
    if (threadIdx.x == 0) *total = t;
}

/* exclusive scan of a list-length array (length read from device memory) */
__global__ void __launch_bounds__(1024) k_scan_list(const int* cnt, int* off, const long long* m_ptr, long long* total) {
    pgb_pdl_entry();
    long long t = block_excl_scan(cnt, off, *m_ptr, 0);
    if (threadIdx.x == 0) *total = t;
}

/* gather per-tile lists (32 mask words a tile, see tile_masks) into one
 * dense list in slot order.  A warp per tile, a lane per word: a shuffle
 * scan of the words' counts gives each word's place, then each lane writes
 * the slots of its set bits.                                             */
__global__ void k_gather_lists(const int* tl, const int* tc, const int* toff, const long long* n_ptr, int* out) {
    pgb_pdl_entry();
    const long long n = *n_ptr;
    const int ntiles = (int)((n + PGB_TILE - 1) / PGB_TILE);
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const unsigned* masks = (const unsigned*)tl;
    for (int t = blockIdx.x * wpb + (threadIdx.x >> 5); t < ntiles; t += gridDim.x * wpb) {
        if (tc[t] == 0) continue;   /* the same for every lane */
        unsigned m = masks[(long long)t * 32 + lane];
        const int c = __popc(m);
        int incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        int pos = toff[t] + incl - c;
        /* word lane = k * warps + w holds slots tile*TILE + k*THREADS + w*32 + bit */
        const int sb = t * PGB_TILE + (lane / (PGB_PUSH_THREADS / 32)) * PGB_PUSH_THREADS +
                       (lane % (PGB_PUSH_THREADS / 32)) * 32;
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            out[pos++] = sb + b;
        }
    }
}

/* ------------------------------------------------------------ inject */
/* particle::inject_more_particles (particle.cpp:491-510): uniform position
 * in [DX, L-DX]^2, velocities from get_particle_velocity, weight 0.0.  For
 * electrons the new particles are pushed here too (they are created before
 * the electron push in pic_run, after the collision loop).               */
struct InjectArgs {
    Species e, i;
    DevState* ds;
    int k;                       /* NUMBER_TO_INJECT */
    double dx, dy, xlength, ylength;
    uint64_t seed;
    PushConsts pce;
    const float2* exy;
    unsigned long long* qacc_e;
    int push_e;                  /* push the new electrons (inside pgb_step) */
    int species_mask;            /* 1 = electrons, 2 = ions                  */
    int* list_out_e;             /* append outside electrons (ordered)       */
    long long list_cap;
    int* flag;                   /* per new electron: outside after its push */
};
__global__ void k_inject(InjectArgs a) {
    pgb_pdl_entry();
    /* one thread per new particle; electrons first, then ions, in id order */
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = a.k * ((a.species_mask & 1) + ((a.species_mask >> 1) & 1));
    if (j >= total) return;
    const int s = ((a.species_mask & 1) && j < a.k) ? 0 : 1;
    const int jj = (s == 0 || !(a.species_mask & 1)) ? j : j - a.k;
    const Species& S = s == 0 ? a.e : a.i;
    const long long n0 = a.ds->n[s];
    const long long slot = n0 + jj;
    if (slot >= S.cap) { atomicOr(&a.ds->err, s == 0 ? ERR_CAP_E : ERR_CAP_I); return; }
    const unsigned int id = a.ds->next_id[s] + (unsigned int)jj;
    pgb_stream st;
    pgb_stream_init(&st, a.seed, id, (unsigned int)a.ds->t, PGB_STREAM_INJECT, (uint32_t)s);
    double rx = pgb_u01d(pgb_stream_u32(&st));
    double ry = pgb_u01d(pgb_stream_u32(&st));
    double x = (a.dx + rx * (a.xlength - 2.0 * a.dx));
    double y = (a.dy + ry * (a.ylength - 2.0 * a.dy));
    float vt = (float)S.vt;
    float vx = maxwell_f32(&st, vt), vy = maxwell_f32(&st, vt), vz = maxwell_f32(&st, vt);
    float4 p = make_float4(pos_from_m(x, a.dx, a.pce.ps), pos_from_m(y, a.dy, a.pce.ps), vx, vy);
    bool out = false;
    if (s == 0 && a.push_e) {
        bool moved;
        gather_push_one(a.pce, a.exy, p, vz, moved);
        /* weight 0: the deposit adds nothing (particle.cpp:497) */
        out = a.pce.steady ? outside_steady(p.x, p.y, a.pce.nx, a.pce.ny, a.pce.ps)
                           : outside_absorbing(p.x, p.y, a.pce.nx, a.pce.ny, a.pce.ps);
    }
    S.xv[slot] = p;
    S.vz[slot] = vz;
    S.w[slot] = 0.0f;
    S.id[slot] = id;
    /* outside electrons join the end of the wall list in slot order */
    if (out) a.flag[jj] = 1;
}

/* after k_inject: counts, ids, and the wall list entries of new electrons */
__global__ void k_inject_commit(InjectArgs a) {
    pgb_pdl_entry();
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int s = 0; s < 2; ++s) {
        if (!(a.species_mask & (1 << s))) continue;
        const Species& S = s == 0 ? a.e : a.i;
        long long n0 = a.ds->n[s];
        int k = a.k;
        if (n0 + k > S.cap) k = (int)(S.cap - n0 > 0 ? S.cap - n0 : 0);
        if (s == 0 && a.push_e) {
            for (int j = 0; j < k; ++j)
                if (a.flag[j]) {
                    long long pos = a.ds->list_n[LIST_OUT_E];
                    if (pos < a.list_cap) { a.list_out_e[pos] = (int)(n0 + j); a.ds->list_n[LIST_OUT_E] = pos + 1; }
                    else a.ds->err |= ERR_LIST;
                    a.flag[j] = 0;
                }
        }
        a.ds->n[s] = n0 + k;
        a.ds->next_id[s] += (unsigned int)k;
        a.ds->stats[s == 0 ? ST_INJ_E : ST_INJ_I] += k;
    }
}

/* ------------------------------------------------- ionization products */
/* e_collisions::ionization appends one ion and one electron per event
 * (e_collisions.cpp:406-441); both are NaN (see ionize_fp64).  With
 * absorbing walls the electron is removed by the wall pass of the same
 * step, and so is the ion on an ion step, so those are counted without
 * being stored; otherwise they are stored in event order.                 */
struct IonizeAppendArgs {
    Species e, i;
    DevState* ds;
    const int* ev;               /* dense event list (electron slots)      */
    CollConsts cc;
    const float* neut;
    double dx, dy;
    int ps;
    int store_e, store_i;
};
__global__ void k_ionize_append(IonizeAppendArgs a) {
    pgb_pdl_entry();
    const long long m = a.ds->list_n[LIST_ION_EV];
    const long long ne0 = a.ds->n[0], ni0 = a.ds->n[1];
    const unsigned int ide0 = a.ds->next_id[0], idi0 = a.ds->next_id[1];
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < m; r += (long long)gridDim.x * blockDim.x) {
        if (!a.store_e && !a.store_i) break;
        int slot = a.ev[r];
        unsigned int pid = a.e.id[slot];
        /* recompute the event's products from the parent's stream; the
         * parent's pre-event velocity is not needed because every product
         * is NaN (the excess energy is negative)                           */
        pgb_stream si;
        pgb_stream_init(&si, a.cc.seed, pid, (unsigned int)a.ds->t, PGB_STREAM_IONIZE, 0);
        float4 pp = a.e.xv[slot];
        double xe = pos_m(pp.x, a.ps, a.dx), ye = pos_m(pp.y, a.ps, a.dy);
        IonizeOut o = ionize_f32(&si, a.neut, a.cc.n_neutral, a.cc, xe, ye, 0.0f, 0.0f, 0.0f);
        if (a.store_i) {
            long long s2 = ni0 + r;
            if (s2 < a.i.cap) {
                a.i.xv[s2] = make_float4(pos_from_m(o.ix, a.dx, a.ps), pos_from_m(o.iy, a.dy, a.ps), (float)o.ivx,
                                         (float)o.ivy);
                a.i.vz[s2] = (float)o.ivz;
                a.i.w[s2] = a.e.w[slot];
                a.i.id[s2] = idi0 + (unsigned int)r;
            } else {
                a.ds->err |= ERR_CAP_I;
            }
        }
        if (a.store_e) {
            long long s2 = ne0 + r;
            if (s2 < a.e.cap) {
                a.e.xv[s2] = make_float4(pos_from_m(o.nx_, a.dx, a.ps), pos_from_m(o.ny_, a.dy, a.ps), (float)o.nvx,
                                         (float)o.nvy);
                a.e.vz[s2] = (float)o.nvz;
                a.e.w[s2] = a.e.w[slot];
                a.e.id[s2] = ide0 + (unsigned int)r;
            } else {
                a.ds->err |= ERR_CAP_E;
            }
        }
    }
}
__global__ void k_ionize_commit(DevState* ds, int store_e, int store_i, long long cap_e, long long cap_i) {
    pgb_pdl_entry();
    long long m = ds->list_n[LIST_ION_EV];
    ds->next_id[0] += (unsigned int)m;
    ds->next_id[1] += (unsigned int)m;
    if (store_e) { long long v = ds->n[0] + m; ds->n[0] = v < cap_e ? v : cap_e; }
    else ds->stats[ST_ABS_E] += m;
    if (store_i) { long long v = ds->n[1] + m; ds->n[1] = v < cap_i ? v : cap_i; }
    else ds->stats[ST_ABS_I] += m;
}

/* ------------------------------------------------------------ compaction */
__global__ void __launch_bounds__(PGB_PUSH_THREADS) k_alive_count(const float4* xv, DevState* ds, int s, int* tc) {
    pgb_pdl_entry();
    const long long n = ds->n[s];
    const int ntiles = (int)((n + PGB_TILE - 1) / PGB_TILE);
    __shared__ int s_w[PGB_PUSH_THREADS / 32];
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        int c = 0;
        for (int k = 0; k < PGB_ITEMS; ++k) {
            long long i = (long long)tile * PGB_TILE + k * PGB_PUSH_THREADS + threadIdx.x;
            if (i < n && !is_dead(xv[i].x)) c++;
        }
        for (int d = 16; d; d >>= 1) c += __shfl_down_sync(0xffffffffu, c, d);
        if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = c;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < PGB_PUSH_THREADS / 32; ++w) t += s_w[w];
            tc[tile] = t;
        }
        __syncthreads();
    }
}
__global__ void __launch_bounds__(PGB_PUSH_THREADS) k_compact(Species S, DevState* ds, int s, const int* toff) {
    pgb_pdl_entry();
    const long long n = ds->n[s];
    const int ntiles = (int)((n + PGB_TILE - 1) / PGB_TILE);
    bool f[1][PGB_ITEMS];
    __shared__ int s_off[PGB_ITEMS][PGB_PUSH_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        unsigned m[PGB_ITEMS];
        for (int k = 0; k < PGB_ITEMS; ++k) {
            long long i = (long long)tile * PGB_TILE + k * PGB_PUSH_THREADS + threadIdx.x;
            f[0][k] = (i < n) && !is_dead(S.xv[i].x);
            m[k] = __ballot_sync(0xffffffffu, f[0][k]);
            if (lane == 0) s_off[k][warp] = __popc(m[k]);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = toff[tile];
            for (int k = 0; k < PGB_ITEMS; ++k)
                for (int w = 0; w < PGB_PUSH_THREADS / 32; ++w) { int c = s_off[k][w]; s_off[k][w] = acc; acc += c; }
        }
        __syncthreads();
        for (int k = 0; k < PGB_ITEMS; ++k)
            if (f[0][k]) {
                long long i = (long long)tile * PGB_TILE + k * PGB_PUSH_THREADS + threadIdx.x;
                int pos = s_off[k][warp] + __popc(m[k] & ((1u << lane) - 1u));
                S.xv2[pos] = S.xv[i];
                S.vz2[pos] = S.vz[i];
                S.w2[pos] = S.w[i];
                S.id2[pos] = S.id[i];
            }
        __syncthreads();
    }
}
__global__ void k_compact_commit(DevState* ds, int s, const long long* total) {
    pgb_pdl_entry();
    ds->n[s] = *total;
    ds->dead[s] = 0;
    ds->n_pieces[s] = 0;       /* slot order changed: the bin pieces are gone */
    ds->sorted_tiles[s] = 0;
}

/* ------------------------------------------------------------ load / dump */
/* slots [i0, i1) from records aos[6 i ..] */
__global__ void k_load(Species S, const double* aos, long long i0, long long i1, double dx, double dy, int ps) {
    pgb_pdl_entry();
    for (long long i = i0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < i1; i += (long long)gridDim.x * blockDim.x) {
        const double* r = aos + 6 * i;
        S.xv[i] = make_float4(pos_from_m(r[0], dx, ps), pos_from_m(r[1], dy, ps), (float)r[2], (float)r[3]);
        S.vz[i] = (float)r[4];
        S.w[i] = (float)r[5];
        S.id[i] = (unsigned int)i;
    }
}
/* dump live slots in order: out[j] for the j-th live slot; pos[] = exclusive
 * scan of the per-tile live counts                                        */
/* tiles [t0, t1) of the live-slot order */
/* out (6 doubles per particle) and ids (the particle's id) are each
 * written when not null                                                  */
__global__ void __launch_bounds__(PGB_PUSH_THREADS) k_dump(Species S, DevState* ds, int s, const int* toff, double dx,
                                                           double dy, int ps, double* out, unsigned int* ids,
                                                           long long cap, int t0, int t1) {
    pgb_pdl_entry();
    const long long n = ds->n[s];
    const int ntiles = min(t1, (int)((n + PGB_TILE - 1) / PGB_TILE));
    __shared__ int s_off[PGB_ITEMS][PGB_PUSH_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int tile = t0 + blockIdx.x; tile < ntiles; tile += gridDim.x) {
        bool f[PGB_ITEMS];
        unsigned m[PGB_ITEMS];
        for (int k = 0; k < PGB_ITEMS; ++k) {
            long long i = (long long)tile * PGB_TILE + k * PGB_PUSH_THREADS + threadIdx.x;
            f[k] = (i < n) && !is_dead(S.xv[i].x);
            m[k] = __ballot_sync(0xffffffffu, f[k]);
            if (lane == 0) s_off[k][warp] = __popc(m[k]);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = toff[tile];
            for (int k = 0; k < PGB_ITEMS; ++k)
                for (int w = 0; w < PGB_PUSH_THREADS / 32; ++w) { int c = s_off[k][w]; s_off[k][w] = acc; acc += c; }
        }
        __syncthreads();
        for (int k = 0; k < PGB_ITEMS; ++k)
            if (f[k]) {
                long long i = (long long)tile * PGB_TILE + k * PGB_PUSH_THREADS + threadIdx.x;
                long long pos = s_off[k][warp] + __popc(m[k] & ((1u << lane) - 1u));
                if (pos < cap && out) {
                    float4 p = S.xv[i];
                    double* o = out + 6 * pos;
                    o[0] = pos_m(p.x, ps, dx); o[1] = pos_m(p.y, ps, dy);
                    o[2] = p.z; o[3] = p.w; o[4] = S.vz[i]; o[5] = S.w[i];
                }
                if (pos < cap && ids) ids[pos] = S.id[i];
            }
        __syncthreads();
    }
}

/* ====================================================== host launchers */
static int grid_for(pgb_run* r, int per_sm) { return r->sms * per_sm; }

static PushConsts push_consts(pgb_run* r, int s) {
    PushConsts pc;
    const Species& S = r->sp[s];
    pc.nx = r->nx; pc.ny = r->ny;
    pc.ps = r->ps;
    pc.dtdx = (float)ldexp(S.dt / r->dx, r->ps);
    pc.dtdy = (float)ldexp(S.dt / r->dy, r->ps);
    pc.coef = (float)(0.5 * S.dt * S.q_over_m);
    double omega_dt = S.dt * S.q_over_m * r->p.magnetic_field;
    pc.ca = (float)cos(r->p.angle); pc.sa = (float)sin(r->p.angle);
    pc.co = (float)cos(omega_dt); pc.so = (float)sin(omega_dt);
    pc.bfield = r->p.magnetic_field > 0.0;
    pc.steady = r->p.steadystate;
    return pc;
}

/* the FP32 fits at the given energies (pgb_cross_sections) */
__global__ void k_cross_sections(int which, const double* e, long long n, double* out) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const float x = (float)e[k];
        float s = 0.0f;
        switch (which) {
            case PGB_XS_AR_ELASTIC: s = sig_ar_el(x); break;
            case PGB_XS_AR_IONIZE: s = sig_ar_ion(x); break;
            case PGB_XS_H_ELASTIC: s = sig_h_el(x); break;
            case PGB_XS_H_IONIZE: s = sig_h_ion(x); break;
            case PGB_XS_AR_CX: s = sig_ar_cx(x); break;
            default: s = sig_h_cx(x); break;
        }
        out[k] = (double)s;
    }
}
int pgb_launch_cross_sections(int which, const double* d_e, long long n, double* d_out, cudaStream_t st) {
    k_cross_sections<<<(int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, st>>>(which, d_e, n, d_out);
    return cudaGetLastError() == cudaSuccess ? 0 : PGB_ERR_CUDA;
}

CollConsts pgb_coll_consts(pgb_run* r) {
    CollConsts c;
    const pgb_params& p = r->p;
    c.species = p.species;
    c.el_const = p.sigma_elastic_mode == PGB_SIGMA_CONSTANT;
    c.ion_const = p.sigma_ionization_mode == PGB_SIGMA_CONSTANT;
    c.cx_const = p.sigma_cx_mode == PGB_SIGMA_CONSTANT;
    c.el_value = (float)p.elastic_sigma_value;
    c.ion_value = (float)p.ionization_sigma_value;
    c.cx_value = (float)p.sigma_value;
    c.e_energy_coef = (float)((0.5 / PGB_CHARGE) * p.electron_mass);
    c.el_max = c.el_const ? c.el_value : (c.species == PGB_ARGON ? 25.5f : 50.5f);
    c.i_energy_coef = (float)((0.5 / PGB_CHARGE) * p.ion_mass);
    c.e_pcoef = (float)(p.dt * 1.0e-20 * p.neutral_density);
    c.i_pcoef = (float)(p.dti * 1.0e-20 * p.neutral_density);
    {
        const double k = (double)c.e_pcoef * (double)c.el_max * 1.000001 * (1.0 + 1.0e-5);
        c.el_bound2 = (float)(k * k * (1.0 + 1.0e-6));
        if (!(c.el_bound2 >= 0.0f)) c.el_bound2 = INFINITY;   /* a negative or NaN bound tests everyone */
    }
    if (c.ion_const) c.ion_emin = c.ion_value > 0.0f ? -INFINITY : INFINITY;
    else c.ion_emin = c.species == PGB_ARGON ? 15.755f : 13.6f;
    c.me = p.electron_mass; c.mi = p.ion_mass; c.dt = p.dt; c.dti = p.dti;
    c.threshold = p.threshold;
    c.reduced_mass = p.ion_mass / (p.electron_mass + p.ion_mass);
    c.n_neutral = p.init_no_neutrals;
    c.seed = p.seed;
    /* (ve + vn) < sqrt(THRESHOLD/rm)/2 makes (rm/2)(ve-vn)^2 at most
     * THRESHOLD/8, far from THRESHOLD whatever the FP32 rounding         */
    {
        double rm = (double)(float)(c.reduced_mass * c.me);
        double cap = 0.5 * sqrt((double)(float)p.threshold / rm) - 1.001 * (double)r->vn_max[0];
        c.ion_vcap = cap > 0.0 ? (float)cap : 0.0f;
    }
    return c;
}

static PushArgs push_args(pgb_run* r, int s) {
    PushArgs a;
    Species& S = r->sp[s];
    a.xv = S.xv; a.vz = S.vz; a.w = S.w; a.id = S.id;
    a.exy = r->exy; a.qacc = r->qacc[s]; a.ds = r->ds; a.s = s;
    a.pc = push_consts(r, s);
    a.cc = pgb_coll_consts(r);
    a.neut = r->neut[0];
    a.pieces = r->pieces[s];
    {
        int nby;
        pgb_bins(r, &a.nbx, &nby);
    }
    a.tl_out = r->tile_list[s == 0 ? LIST_OUT_E : LIST_OUT_I];
    a.tc_out = r->tile_cnt[s == 0 ? LIST_OUT_E : LIST_OUT_I];
    a.tl_ev = r->tile_list[LIST_ION_EV];
    a.tc_ev = r->tile_cnt[LIST_ION_EV];
    return a;
}

int pgb_launch_push(pgb_run* r, int s, bool deposit) {
    PushArgs a = push_args(r, s);
    int g = grid_for(r, r->tune_push_per_sm);
    void (*kp)(PushArgs) = deposit ? k_push<true> : k_push<false>;
    PGB_CK(r, pgb_launch_pdl(kp, dim3(g), dim3(PGB_PUSH_THREADS), 0, r->stream, a));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_flag_outside(pgb_run* r, int s) {
    int l = s == 0 ? LIST_OUT_E : LIST_OUT_I;
    PGB_CK(r, pgb_launch_pdl(k_flag, dim3(grid_for(r, 8)), dim3(PGB_PUSH_THREADS), 0, r->stream, r->sp[s].xv, r->ds, s, r->nx, r->ny, r->ps, r->p.steadystate,
                                                               r->tile_list[l], r->tile_cnt[l]));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}


int pgb_launch_step_advance(pgb_run* r) {
    PGB_CK(r, pgb_launch_pdl(k_step_advance, dim3(1), dim3(1), 0, r->stream, r->ds));
    r->launches++;
    return 0;
}

/* leave_sms: SMs the collision kernels leave free (one block fills an SM).
 * Small runs take fewer blocks: one per MCC_GROUPS tiles for k_mcc, one per
 * 16 Ki electrons for k_scatter (about a scattering per thread), from the
 * electron count last read back; both kernels loop grid-stride.
 * The scattering list is the spare dense list (capacity >= electron slots). */
static int mcc_blocks(pgb_run* r, int leave_sms, long long per_block) {
    const long long n = std::max<long long>(r->hs->n[0], 0);
    const long long want = std::max<long long>(1, (n + per_block - 1) / per_block);
    return (int)std::min<long long>(std::max(1, r->sms - leave_sms), want);
}
int pgb_launch_mcc(pgb_run* r, int leave_sms) {
    PushArgs a = push_args(r, 0);
    const int g = mcc_blocks(r, leave_sms, (long long)MCC_GROUPS * PGB_TILE);
    PGB_CK(r, cudaMemsetAsync(&r->ds->scat_n, 0, sizeof(unsigned long long), r->stream));
    PGB_CK(r, pgb_launch_pdl(k_mcc, dim3(g), dim3(MCC_THREADS), 0, r->stream, a, r->list[LIST_SPARE]));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_scatter(pgb_run* r, int leave_sms) {
    PushArgs a = push_args(r, 0);
    const int g = mcc_blocks(r, leave_sms, 16384);
    PGB_CK(r, pgb_launch_pdl(k_scatter, dim3(g), dim3(MCC_THREADS), 0, r->stream, a, (const int*)r->list[LIST_SPARE]));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

/* per-tile list `which` (tiles of species s) -> dense list + count */
int pgb_build_list(pgb_run* r, int which, int s, bool count_only) {
    int* toff = r->aux_j;
    PGB_CK(r, pgb_launch_pdl(k_scan_small, dim3(1), dim3(1024), 0, r->stream, r->tile_cnt[which], toff, &r->ds->n[s], 0, &r->ds->list_n[which]));
    r->launches++;
    if (count_only) return 0;
    PGB_CK(r, pgb_launch_pdl(k_gather_lists, dim3(grid_for(r, 4)), dim3(256), 0, r->stream, r->tile_list[which], r->tile_cnt[which], toff,
                                                           &r->ds->n[s], r->list[which]));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_deposit(pgb_run* r, int s) {
    PGB_CK(r, pgb_launch_pdl(k_deposit, dim3(grid_for(r, 8)), dim3(256), 0, r->stream, r->sp[s].xv, r->sp[s].w, r->ds, s, r->nx, r->ny, r->ps, r->qacc[s]));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_inject(pgb_run* r, int species_mask, bool push_e) {
    InjectArgs a;
    a.e = r->sp[0]; a.i = r->sp[1]; a.ds = r->ds; a.k = r->p.number_to_inject;
    a.dx = r->dx; a.dy = r->dy; a.xlength = r->p.xlength; a.ylength = r->p.ylength;
    a.seed = r->p.seed;
    a.pce = push_consts(r, 0); a.exy = r->exy; a.qacc_e = r->qacc[0];
    a.push_e = push_e; a.species_mask = species_mask;
    a.list_out_e = r->list[LIST_OUT_E]; a.list_cap = r->list_cap;
    a.flag = r->inject_flag;
    int tot = 2 * a.k;
    if (tot <= 0) return 0;
    PGB_CK(r, pgb_launch_pdl(k_inject, dim3((tot + 127) / 128), dim3(128), 0, r->stream, a));
    PGB_CK(r, pgb_launch_pdl(k_inject_commit, dim3(1), dim3(32), 0, r->stream, a));
    r->launches += 2;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_ionize_appends(pgb_run* r, int store_e, int store_i) {
    IonizeAppendArgs a;
    a.e = r->sp[0]; a.i = r->sp[1]; a.ds = r->ds; a.ev = r->list[LIST_ION_EV];
    a.cc = pgb_coll_consts(r); a.neut = r->neut[0];
    a.dx = r->dx; a.dy = r->dy; a.ps = r->ps;
    a.store_e = store_e;
    a.store_i = store_i;
    if (store_e || store_i) {   /* else the products are only counted */
        PGB_CK(r, pgb_launch_pdl(k_ionize_append, dim3(r->sms * 2), dim3(256), 0, r->stream, a));
        r->launches++;
        PGB_CK(r, cudaGetLastError());
    }
    PGB_CK(r, pgb_launch_pdl(k_ionize_commit, dim3(1), dim3(1), 0, r->stream, r->ds, a.store_e, a.store_i, r->sp[0].cap, r->sp[1].cap));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_compact(pgb_run* r, int s) {
    Species& S = r->sp[s];
    int* tc = r->tile_cnt[LIST_SPARE];
    int* toff = r->aux_j;
    PGB_CK(r, cudaMemsetAsync(tc, 0, sizeof(int) * r->ntiles_cap, r->stream));
    PGB_CK(r, pgb_launch_pdl(k_alive_count, dim3(grid_for(r, 8)), dim3(PGB_PUSH_THREADS), 0, r->stream, S.xv, r->ds, s, tc));
    r->launches++;
    PGB_CK(r, pgb_launch_pdl(k_scan_small, dim3(1), dim3(1024), 0, r->stream, tc, toff, &r->ds->n[s], 0, &r->ds->list_n[LIST_SPARE]));
    r->launches++;
    PGB_CK(r, pgb_launch_pdl(k_compact, dim3(grid_for(r, 8)), dim3(PGB_PUSH_THREADS), 0, r->stream, S, r->ds, s, toff));
    r->launches++;
    PGB_CK(r, pgb_launch_pdl(k_compact_commit, dim3(1), dim3(1), 0, r->stream, r->ds, s, &r->ds->list_n[LIST_SPARE]));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    std::swap(S.xv, S.xv2);
    std::swap(S.vz, S.vz2);
    std::swap(S.w, S.w2);
    std::swap(S.id, S.id2);
    return 0;
}

int pgb_launch_load(pgb_run* r, int s, const double* d_aos, long long i0, long long i1) {
    PGB_CK(r, pgb_launch_pdl(k_load, dim3(grid_for(r, 4)), dim3(256), 0, r->stream, r->sp[s], d_aos, i0, i1, r->dx, r->dy, r->ps));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

/* live-slot offsets per tile (into r->aux_j) for pgb_launch_dump */
int pgb_launch_dump_offsets(pgb_run* r, int s) {
    int* tc = r->tile_cnt[LIST_SPARE];
    PGB_CK(r, cudaMemsetAsync(tc, 0, sizeof(int) * r->ntiles_cap, r->stream));
    PGB_CK(r, pgb_launch_pdl(k_alive_count, dim3(grid_for(r, 8)), dim3(PGB_PUSH_THREADS), 0, r->stream, r->sp[s].xv, r->ds, s, tc));
    r->launches++;
    PGB_CK(r, pgb_launch_pdl(k_scan_small, dim3(1), dim3(1024), 0, r->stream, tc, r->aux_j, &r->ds->n[s], 0, &r->ds->list_n[LIST_SPARE]));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_dump(pgb_run* r, int s, double* d_out, unsigned int* d_ids, long long cap, int t0, int t1) {
    PGB_CK(r, pgb_launch_pdl(k_dump, dim3(grid_for(r, 8)), dim3(PGB_PUSH_THREADS), 0, r->stream, r->sp[s], r->ds, s, r->aux_j, r->dx, r->dy, r->ps, d_out,
                             d_ids, cap, t0, t1));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

