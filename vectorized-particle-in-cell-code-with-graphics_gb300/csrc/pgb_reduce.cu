/*
 * Kunhardt population control: particle::contain_particle_growth and
 * reduce_population (particle.cpp:520-653).
 *
 * When a species holds more than SIZE_TO_CHECK particles, each particle is
 * put in a speed group by |v_xy| against V_LIMIT (particle.cpp:556-566).
 * A group holding more than GROUP_LIMIT particles is cut to
 * NEW_GROUP_SIZE.  The group's survivors are re-weighted by
 * Ngroup/(Ngroup - removed), so the group keeps its charge
 * (particle.cpp:612-653).
 *
 * The reference picks the removed particles one at a time with rand().
 * Here every particle gets a priority, the first 32-bit word of its Philox
 * stream (id, step, REDUCE, species).  In each over-full group the Nremove
 * particles with the smallest (priority, id) are removed.  The set removed
 * does not depend on the slot order, and the oracle's library mode applies
 * the same rule.
 *
 * The selection is an exact radix select on the 64-bit key (priority, id),
 * eight passes of 8 bits.  Each pass histograms the particles whose key
 * matches the digits fixed so far; the host then fixes the next digit of
 * each group.  Keys are unique because ids are, so exactly Nremove
 * particles of the group have a key <= the selected one.  Removed
 * particles become tombstones in place; the next compaction or spatial
 * sort drops them.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "pgb_internal.h"
#include "pgb_physics.cuh"

#define KH_GROUPS 3

struct KhState {
    unsigned long long ngroup[KH_GROUPS];
    unsigned long long removed;
    unsigned int hist[KH_GROUPS][256];
};

struct KhArgs {
    Species S;
    DevState* ds;
    KhState* st;
    int s;
    int ng;
    double vlim[KH_GROUPS];
    uint64_t seed;
    int active[KH_GROUPS];                 /* group has particles to remove   */
    unsigned long long prefix[KH_GROUPS];  /* digits fixed so far             */
    int shift;                             /* bit position of this pass's digit */
    double gwd[KH_GROUPS];                 /* survivor re-weighting           */
};

/* speed group: while (|v_xy| > V_LIMIT[g]) g++, capped at the last group
 * (particle.cpp:556-566)                                                  */
__device__ __forceinline__ int kh_group(float4 p, const KhArgs& a) {
    double vx = (double)p.z, vy = (double)p.w;
    double vxy = sqrt(vx * vx + vy * vy);
    int g = 0;
    while (g < a.ng - 1 && vxy > a.vlim[g]) g++;
    return g;
}

__device__ __forceinline__ unsigned long long kh_key(const KhArgs& a, unsigned int id, unsigned int step) {
    pgb_stream st;
    pgb_stream_init(&st, a.seed, id, step, PGB_STREAM_REDUCE, (uint32_t)a.s);
    return ((unsigned long long)pgb_stream_u32(&st) << 32) | id;
}

__global__ void __launch_bounds__(256) k_kh_count(KhArgs a) {
    __shared__ unsigned long long s_cnt[KH_GROUPS];
    if (threadIdx.x < KH_GROUPS) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    const long long n = a.ds->n[a.s];
    unsigned int c[KH_GROUPS] = {0, 0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 p = a.S.xv[i];
        if (is_dead(p.x)) continue;
        c[kh_group(p, a)]++;
    }
    for (int g = 0; g < KH_GROUPS; ++g)
        if (c[g]) atomicAdd(&s_cnt[g], (unsigned long long)c[g]);
    __syncthreads();
    if (threadIdx.x < KH_GROUPS && s_cnt[threadIdx.x]) atomicAdd(&a.st->ngroup[threadIdx.x], s_cnt[threadIdx.x]);
}

/* histogram of this pass's digit over the keys that match the prefix */
__global__ void __launch_bounds__(256) k_kh_hist(KhArgs a) {
    __shared__ unsigned int s_h[KH_GROUPS][256];
    for (int k = threadIdx.x; k < KH_GROUPS * 256; k += blockDim.x) (&s_h[0][0])[k] = 0;
    __syncthreads();
    const long long n = a.ds->n[a.s];
    const unsigned int step = (unsigned int)a.ds->t;
    const int hi = a.shift + 8;   /* bits above this digit must match */
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 p = a.S.xv[i];
        if (is_dead(p.x)) continue;
        int g = kh_group(p, a);
        if (!a.active[g]) continue;
        unsigned long long key = kh_key(a, a.S.id[i], step);
        if (hi < 64 && (key >> hi) != (a.prefix[g] >> hi)) continue;
        atomicAdd(&s_h[g][(key >> a.shift) & 255u], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < KH_GROUPS * 256; k += blockDim.x) {
        unsigned int v = (&s_h[0][0])[k];
        if (v) atomicAdd(&(&a.st->hist[0][0])[k], v);
    }
}

/* remove keys <= the selected key of an active group; re-weight the rest */
__global__ void __launch_bounds__(256) k_kh_apply(KhArgs a) {
    __shared__ unsigned long long s_rm;
    if (threadIdx.x == 0) s_rm = 0;
    __syncthreads();
    const long long n = a.ds->n[a.s];
    const unsigned int step = (unsigned int)a.ds->t;
    unsigned int rm = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float4 p = a.S.xv[i];
        if (is_dead(p.x)) continue;
        int g = kh_group(p, a);
        if (a.active[g] && kh_key(a, a.S.id[i], step) <= a.prefix[g]) {
            a.S.xv[i].x = pos_dead();
            rm++;
        } else if (a.gwd[g] != 1.0) {
            a.S.w[i] = (float)((double)a.S.w[i] * a.gwd[g]);
        }
    }
    if (rm) atomicAdd(&s_rm, (unsigned long long)rm);
    __syncthreads();
    if (threadIdx.x == 0 && s_rm) {
        atomicAdd((unsigned long long*)&a.ds->dead[a.s], s_rm);
        atomicAdd(&a.st->removed, s_rm);
    }
}

__global__ void k_kh_count_event(DevState* ds, int s) {
    ds->stats[s == 0 ? ST_RED_E : ST_RED_I] += 1;
}

/* ============================================================ host side */
static int kh_fail(pgb_run* r, cudaError_t e, const char* what) {
    pgb_cuda_ok(r, e, what);
    return PGB_ERR_CUDA;
}

/* The caller has synchronised r->hs with the device and found the species
 * above its SIZE_TO_CHECK.  Waits for the stream (the group counts and the
 * digit histograms are read on the host).                                 */
int pgb_launch_reduce(pgb_run* r, int s) {
    cudaError_t e;
    if (!r->kh) {
        e = cudaMalloc((void**)&r->kh, sizeof(KhState));
        if (e != cudaSuccess) return kh_fail(r, e, "pgb_launch_reduce: cudaMalloc");
    }
    KhState* st = (KhState*)r->kh;
    KhArgs a;
    a.S = r->sp[s]; a.ds = r->ds; a.st = st; a.s = s;
    a.ng = r->p.no_groups < 1 ? 1 : (r->p.no_groups > KH_GROUPS ? KH_GROUPS : r->p.no_groups);
    const double* vl = s == 0 ? r->p.v_limit_e : r->p.v_limit_i;
    const int32_t* glim = s == 0 ? r->p.group_limit_e : r->p.group_limit_i;
    const int32_t* gnew = s == 0 ? r->p.new_group_size_e : r->p.new_group_size_i;
    for (int g = 0; g < KH_GROUPS; ++g) {
        a.vlim[g] = vl[g];
        a.active[g] = 0;
        a.prefix[g] = 0;
        a.gwd[g] = 1.0;
    }
    a.seed = r->p.seed;
    a.shift = 56;
    const int blocks = r->sms * 8;

    if ((e = cudaMemsetAsync(st, 0, sizeof(KhState), r->stream)) != cudaSuccess) return kh_fail(r, e, "kh memset");
    k_kh_count<<<blocks, 256, 0, r->stream>>>(a);
    r->launches++;
    k_kh_count_event<<<1, 1, 0, r->stream>>>(r->ds, s);
    r->launches++;
    KhState h;
    if ((e = cudaMemcpyAsync(&h, st, sizeof(KhState), cudaMemcpyDeviceToHost, r->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(r->stream)) != cudaSuccess)
        return kh_fail(r, e, "pgb_launch_reduce: group counts");

    long long ngroup[KH_GROUPS], nremove[KH_GROUPS] = {0, 0, 0}, to_remove = 0;
    for (int g = 0; g < KH_GROUPS; ++g) ngroup[g] = (long long)h.ngroup[g];
    for (int g = 0; g < a.ng; ++g) {
        if (ngroup[g] > glim[g]) nremove[g] = ngroup[g] - gnew[g];
        to_remove += nremove[g];
    }
    if (to_remove <= 0) return 0;
    long long need[KH_GROUPS] = {0, 0, 0};
    bool any = false;
    for (int g = 0; g < a.ng; ++g)
        if (nremove[g] > 0) {
            a.active[g] = 1;
            need[g] = nremove[g] < ngroup[g] ? nremove[g] : ngroup[g];   /* rank of the last removed key */
            any = true;
        }
    if (!any) return 0;

    for (int pass = 0; pass < 8; ++pass) {
        a.shift = 56 - 8 * pass;
        if ((e = cudaMemsetAsync(st->hist, 0, sizeof(st->hist), r->stream)) != cudaSuccess) return kh_fail(r, e, "kh memset");
        k_kh_hist<<<blocks, 256, 0, r->stream>>>(a);
        r->launches++;
        if ((e = cudaMemcpyAsync(h.hist, st->hist, sizeof(st->hist), cudaMemcpyDeviceToHost, r->stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(r->stream)) != cudaSuccess)
            return kh_fail(r, e, "pgb_launch_reduce: digit histogram");
        for (int g = 0; g < a.ng; ++g) {
            if (!a.active[g]) continue;
            long long cum = 0;
            int d = 0;
            for (; d < 256; ++d) {
                if (cum + (long long)h.hist[g][d] >= need[g]) break;
                cum += h.hist[g][d];
            }
            if (d == 256) {   /* counts changed under us: cannot happen on a quiet stream */
                pgb_cuda_ok(r, cudaErrorUnknown, "pgb_launch_reduce: radix select lost its rank");
                return PGB_ERR_STATE;
            }
            need[g] -= cum;
            a.prefix[g] |= (unsigned long long)d << a.shift;
        }
    }
    for (int g = 0; g < a.ng; ++g)
        if (a.active[g]) {
            long long removed = nremove[g] < ngroup[g] ? nremove[g] : ngroup[g];
            if (ngroup[g] - removed > 0) a.gwd[g] = (double)ngroup[g] / (double)(ngroup[g] - removed);
        }
    k_kh_apply<<<blocks, 256, 0, r->stream>>>(a);
    r->launches++;
    if ((e = cudaGetLastError()) != cudaSuccess) return kh_fail(r, e, "pgb_launch_reduce: launch");
    return 0;
}
