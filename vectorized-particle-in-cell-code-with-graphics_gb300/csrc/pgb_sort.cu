/*
 * Spatial binning of the particles (stable counting sort by bin).
 *
 * The deposit (particle::collect_charge, pic.cl:22-52) scatters four adds
 * per particle; on particles in arbitrary order they land on random grid
 * nodes and the adds go to L2 as global atomics.  Every sort_interval steps
 * the particles of a species are re-ordered by bin (BIN x BIN cells), each
 * bin starting on a 1024-slot tile boundary, so the push kernel can give a
 * CTA a run of tiles of one bin and accumulate its deposit in a shared-
 * memory window of the bin's nodes plus a halo.
 *
 * The sort is stable (particles keep their relative order within a bin),
 * so the resulting order -- and every order-dependent rule that follows it
 * (charge-exchange accumulation, wall-list order) -- is deterministic.  It
 * also drops removed particles (tombstones).  Passes:
 *   count    per chunk of SORT_CHUNK slots, a shared histogram of bin keys
 *   scan     per bin over chunks, then over bins with tile padding
 *   scatter  one warp per chunk walks its slots in order and writes each
 *            particle to its bin at a running per-bin cursor
 *   pieces   tile -> bin map and work pieces (runs of tiles of one bin)
 */
#include <cuda_runtime.h>
#include "pgb_internal.h"
#include "pgb_physics.cuh"

#define SORT_CHUNK PGB_SORT_CHUNK

struct SortArgs {
    Species S;
    DevState* ds;
    int s;
    int nx, ny;              /* nodes */
    int ps;                  /* fraction bits of the positions */
    int nbx, nby, nbins;     /* bins; key nbins = not in the deposit region */
    long long nchunks_cap;
    int* counts;             /* [key][chunk] */
    int* offs;               /* [key][chunk] exclusive within the key */
    int* key_total;          /* [key] */
    long long* key_start;    /* [key+1] padded starts */
    int* tile_bin;           /* [tile] */
    int4* pieces;            /* {first tile, tiles, bin, 0} */
    int piece_tiles;
};

__device__ __forceinline__ int bin_key(float4 p, int nx, int ny, int ps, int nbx, int nbins) {
    if (is_dead(p.x)) return -1;
    int jp = pcell(p.x, ps), kp = pcell(p.y, ps);
    /* the deposit region of collectCharge (pic.cl:35) */
    if (!deposit_ok(p.x, p.y, nx, ny, ps)) return nbins;
    return (kp / PGB_BIN) * nbx + (jp / PGB_BIN);
}

__global__ void __launch_bounds__(256) k_sort_count(SortArgs a) {
    pgb_pdl_entry();
    extern __shared__ int s_hist[];
    const long long n = a.ds->n[a.s];
    const int nch = (int)((n + SORT_CHUNK - 1) / SORT_CHUNK);
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        for (int k = threadIdx.x; k <= a.nbins; k += blockDim.x) s_hist[k] = 0;
        __syncthreads();
        for (int k = threadIdx.x; k < SORT_CHUNK; k += blockDim.x) {
            long long i = (long long)c * SORT_CHUNK + k;
            if (i >= n) break;
            int key = bin_key(a.S.xv[i], a.nx, a.ny, a.ps, a.nbx, a.nbins);
            if (key >= 0) atomicAdd(&s_hist[key], 1);
        }
        __syncthreads();
        for (int k = threadIdx.x; k <= a.nbins; k += blockDim.x) a.counts[(long long)k * a.nchunks_cap + c] = s_hist[k];
        __syncthreads();
    }
}

/* exclusive scan of one value per thread over the CTA; *total = the sum.
 * Every thread of the CTA must call it.                                  */
__device__ __forceinline__ long long block_excl_scan_ll(long long v, long long* s_w, long long& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long x = v;
    for (int d = 1; d < 32; d <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < nw ? s_w[lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        if (lane < nw) s_w[lane] = w;   /* inclusive over warps */
    }
    __syncthreads();
    long long before = warp ? s_w[warp - 1] : 0;
    total = s_w[nw - 1];
    __syncthreads();
    return before + x - v;
}

/* per key: exclusive scan over the live chunks (one CTA per key) */
__global__ void __launch_bounds__(1024) k_sort_scan_keys(SortArgs a) {
    pgb_pdl_entry();
    const long long n = a.ds->n[a.s];
    const int nch = (int)((n + SORT_CHUNK - 1) / SORT_CHUNK);
    __shared__ long long s_w[32];
    for (int key = blockIdx.x; key <= a.nbins; key += gridDim.x) {
        const int* row = a.counts + (long long)key * a.nchunks_cap;
        int* out = a.offs + (long long)key * a.nchunks_cap;
        long long carry = 0;
        for (int b = 0; b < nch; b += blockDim.x) {
            int c = b + threadIdx.x;
            long long v = c < nch ? row[c] : 0, tot;
            long long ex = block_excl_scan_ll(v, s_w, tot);
            if (c < nch) out[c] = (int)(carry + ex);
            carry += tot;
        }
        if (threadIdx.x == 0) a.key_total[key] = (int)carry;
    }
}

/* over keys: padded starts (each key begins on a tile boundary), pieces.
 * One CTA scans the keys 1024 at a time (tiles and pieces per key), each
 * key's thread writes its pieces, then every tile finds its key by binary
 * search over the starts.                                               */
__global__ void __launch_bounds__(1024) k_sort_scan_bins(SortArgs a) {
    pgb_pdl_entry();
    __shared__ long long s_w[32];
    long long carry_t = 0, carry_p = 0;
    for (int base = 0; base <= a.nbins; base += blockDim.x) {
        const int key = base + threadIdx.x;
        long long tiles = 0, np = 0;
        if (key <= a.nbins) {
            long long c = a.key_total[key];
            tiles = (c + PGB_TILE - 1) / PGB_TILE;
            np = (tiles + a.piece_tiles - 1) / a.piece_tiles;
        }
        long long tot_t, tot_p;
        long long t0 = carry_t + block_excl_scan_ll(tiles, s_w, tot_t);
        long long p0 = carry_p + block_excl_scan_ll(np, s_w, tot_p);
        if (key <= a.nbins) {
            a.key_start[key] = t0 * PGB_TILE;
            const int bin = key < a.nbins ? key : -1;
            for (long long q = 0; q < np; ++q) {
                long long t = q * a.piece_tiles;
                int len = (int)((tiles - t) < a.piece_tiles ? (tiles - t) : a.piece_tiles);
                a.pieces[p0 + q] = make_int4((int)(t0 + t), len, bin, 0);
            }
        }
        carry_t += tot_t;
        carry_p += tot_p;
    }
    /* every bin starts on a tile boundary: the padded layout needs carry_t
     * tiles.  If they do not fit the capacity, the sort copies the
     * particles in their current order instead (no pieces, no padding) and
     * the step reports the capacity error.                              */
    __shared__ int s_over;
    if (threadIdx.x == 0) {
        const int over = carry_t * PGB_TILE > a.S.cap ? 1 : 0;
        s_over = over;
        a.ds->sort_overflow = over;
        a.key_start[a.nbins + 1] = carry_t * PGB_TILE;
        a.ds->n_pieces[a.s] = over ? 0 : (int)carry_p;
        a.ds->sorted_tiles[a.s] = over ? 0 : carry_t;
        if (over) atomicOr(&a.ds->err, a.s == 0 ? ERR_CAP_E : ERR_CAP_I);
    }
    __syncthreads();
    if (s_over) return;
    /* tile -> bin map: the key whose [start, next start) holds the tile */
    for (long long t = threadIdx.x; t < carry_t; t += blockDim.x) {
        const long long slot = t * PGB_TILE;
        int lo = 0, hi = a.nbins;   /* largest key with key_start <= slot */
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (a.key_start[mid] <= slot) lo = mid;
            else hi = mid - 1;
        }
        a.tile_bin[t] = lo < a.nbins ? lo : -1;
    }
}

/* one warp per chunk: stable placement at per-key cursors.  Four batches of
 * 32 slots are loaded at once (memory-level parallelism), then placed in
 * slot order.                                                           */
#define SCATTER_BATCHES 4
__global__ void __launch_bounds__(256) k_sort_scatter(SortArgs a) {
    pgb_pdl_entry();
    extern __shared__ long long s_cur[];   /* [warp][key] */
    const long long n = a.ds->n[a.s];
    const int nch = (int)((n + SORT_CHUNK - 1) / SORT_CHUNK);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long* cur = s_cur + (long long)warp * (a.nbins + 1);
    const unsigned lt = (1u << lane) - 1u;
    if (a.ds->sort_overflow) {
        /* the padded layout does not fit: keep the order (and the slots) */
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
            a.S.xv2[i] = a.S.xv[i];
            a.S.vz2[i] = a.S.vz[i];
            a.S.w2[i] = a.S.w[i];
            a.S.id2[i] = a.S.id[i];
        }
        return;
    }
    for (int c = blockIdx.x * nw + warp; c < nch; c += gridDim.x * nw) {
        for (int k = lane; k <= a.nbins; k += 32) cur[k] = a.key_start[k] + a.offs[(long long)k * a.nchunks_cap + c];
        __syncwarp();
        for (int b = 0; b < SORT_CHUNK; b += 32 * SCATTER_BATCHES) {
            float4 p[SCATTER_BATCHES];
            float vz[SCATTER_BATCHES], w[SCATTER_BATCHES];
            unsigned int id[SCATTER_BATCHES];
            int key[SCATTER_BATCHES];
#pragma unroll
            for (int u = 0; u < SCATTER_BATCHES; ++u) {
                long long i = (long long)c * SORT_CHUNK + b + u * 32 + lane;
                key[u] = -1;
                if (i < n) {
                    p[u] = a.S.xv[i];
                    vz[u] = a.S.vz[i];
                    w[u] = a.S.w[i];
                    id[u] = a.S.id[i];
                    key[u] = bin_key(p[u], a.nx, a.ny, a.ps, a.nbx, a.nbins);
                }
            }
#pragma unroll
            for (int u = 0; u < SCATTER_BATCHES; ++u) {
                unsigned peers = __match_any_sync(0xffffffffu, key[u]);
                long long pos = -1;
                if (key[u] >= 0) pos = cur[key[u]] + __popc(peers & lt);
                __syncwarp();
                if (key[u] >= 0 && (peers & lt) == 0) cur[key[u]] += __popc(peers);
                __syncwarp();
                if (key[u] >= 0 && pos < a.S.cap) {
                    a.S.xv2[pos] = p[u];
                    a.S.vz2[pos] = vz[u];
                    a.S.w2[pos] = w[u];
                    a.S.id2[pos] = id[u];
                }
            }
        }
        __syncwarp();
    }
}

/* tombstones in the padding after each key's particles; new counts */
__global__ void k_sort_pad(SortArgs a) {
    pgb_pdl_entry();
    if (a.ds->sort_overflow) return;   /* the copy kept n and the tombstones */
    for (int key = blockIdx.x; key <= a.nbins; key += gridDim.x) {
        long long s0 = a.key_start[key] + a.key_total[key], s1 = a.key_start[key + 1];
        for (long long i = s0 + threadIdx.x; i < s1; i += blockDim.x) {
            a.S.xv2[i] = make_float4(pos_dead(), 0.f, 0.f, 0.f);
            a.S.vz2[i] = 0.f;
            a.S.w2[i] = 0.f;
            a.S.id2[i] = 0u;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        long long live = 0;
        for (int key = 0; key <= a.nbins; ++key) live += a.key_total[key];
        long long tot = a.key_start[a.nbins + 1];
        a.ds->n[a.s] = tot;
        a.ds->dead[a.s] = tot - live;
    }
}

/* ============================================================ host side */
void pgb_bins(pgb_run* r, int* nbx, int* nby) {
    *nbx = (r->nx - 1 + PGB_BIN - 1) / PGB_BIN;
    *nby = (r->ny - 1 + PGB_BIN - 1) / PGB_BIN;
}

int pgb_launch_sort(pgb_run* r, int s) {
    SortArgs a;
    a.S = r->sp[s]; a.ds = r->ds; a.s = s; a.nx = r->nx; a.ny = r->ny; a.ps = r->ps;
    pgb_bins(r, &a.nbx, &a.nby);
    a.nbins = a.nbx * a.nby;
    a.nchunks_cap = r->sort_chunks_cap;
    a.counts = r->sort_counts; a.offs = r->sort_offs; a.key_total = r->sort_key_total;
    a.key_start = r->sort_key_start; a.tile_bin = r->tile_bin[s]; a.pieces = r->pieces[s];
    a.piece_tiles = PGB_PIECE_TILES;
    size_t hist = sizeof(int) * (a.nbins + 1);
    PGB_CK(r, pgb_launch_pdl(k_sort_count, dim3(r->sms * 4), dim3(256), hist, r->stream, a));
    r->launches++;
    PGB_CK(r, pgb_launch_pdl(k_sort_scan_keys, dim3(r->sms * 2), dim3(1024), 0, r->stream, a));
    r->launches++;
    PGB_CK(r, pgb_launch_pdl(k_sort_scan_bins, dim3(1), dim3(1024), 0, r->stream, a));
    r->launches++;
    size_t cur = sizeof(long long) * (a.nbins + 1) * 8;
    PGB_CK(r, pgb_launch_pdl(k_sort_scatter, dim3(r->sms * 4), dim3(256), cur, r->stream, a));
    r->launches++;
    PGB_CK(r, pgb_launch_pdl(k_sort_pad, dim3(r->sms), dim3(256), 0, r->stream, a));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    Species& S = r->sp[s];
    std::swap(S.xv, S.xv2);
    std::swap(S.vz, S.vz2);
    std::swap(S.w, S.w2);
    std::swap(S.id, S.id2);
    return 0;
}

int pgb_sort_setup(pgb_run* r) {
    int nbx, nby;
    pgb_bins(r, &nbx, &nby);
    int nbins = nbx * nby;
    size_t cur = sizeof(long long) * (nbins + 1) * 8;
    if (cur > 48 * 1024) PGB_CK(r, cudaFuncSetAttribute(k_sort_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cur));
    size_t hist = sizeof(int) * (nbins + 1);
    if (hist > 48 * 1024) PGB_CK(r, cudaFuncSetAttribute(k_sort_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hist));
    return 0;
}
