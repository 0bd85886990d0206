/*
 * Headless viewer plots: the plots of the reference's OpenGL viewer
 * (graphics.cpp:245-607) rasterised by CUDA into an RGB8 image owned by the
 * run.  The GL window itself needs a graphics stack; the plots are plain
 * rasterisation and need none.
 *
 * Particle plots (two order-independent passes over the particle arrays):
 *   - a particle is plotted when it is live, in the sample (a hash of its
 *     id, see rd_keep) and strictly inside the domain in FP32 cell units
 *     (the |x| < boxLength/2 test of graphics.cpp:432-436, 593-595);
 *   - vx-vy: k_rd_vmax takes the largest |vx| and |vy| of those particles
 *     (atomicMax on the float bits, exact), k_rd_points truncates it to an
 *     int, at least 1 (graphics.cpp:421-452), and plots the particles with
 *     |vx|, |vy| below it (graphics.cpp:499-503);
 *   - a point is 2 x 2 pixels (glPointSize(2), graphics.cpp:483).  Points
 *     mark a one-byte-per-pixel layer (1 electrons, 2 ions; the ion pass
 *     runs second and overwrites), storing only where the byte changes:
 *     dense plasma puts tens of points on a pixel, and unconditional
 *     stores to the same lines serialise.  k_rd_resolve turns the layer
 *     into colours, one thread per pixel.
 *   - Blocks take 1024-particle tiles in a scrambled order (tile t * P mod
 *     ntiles, P a prime above any tile count): spatially sorted particles
 *     would otherwise put every block in flight on the same few bins, and
 *     so on the same few lines of the layer.
 * Field plots (k_rd_field, one thread per pixel): the pixel's grid
 * coordinate picks a cell; the cell's quad is inset by a tenth of a cell,
 * and its colour is the ramp of drawField (graphics.cpp:303-356) applied to
 * |mean of the four corners / max|.  The maximum comes from k_rd_fmax, an
 * order-independent max over the field (NaN values ignored).
 *
 * The unit is compiled with --fmad=false so that every pixel and colour
 * equals the oracle's C restatement of the same rules bit for bit.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include "pgb_internal.h"
#include "pgb_physics.cuh"

namespace {

struct Rgb { unsigned char r, g, b; };

/* colour byte of a [0,1] component */
__device__ __forceinline__ unsigned char rd_byte(float c) {
    float v = c * 255.0f + 0.5f;
    v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
    return (unsigned char)(int)v;
}

/* lowbias32 integer hash (C. Wellons, hash-prospector) of id and seed */
__device__ __forceinline__ uint32_t rd_hash(uint32_t id, uint32_t seed) {
    uint32_t x = id ^ (seed * 0x9E3779B9u);
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

/* in the sample: all particles when max_points <= 0 or n <= max_points,
 * else hash < max_points/n of the 32-bit range                          */
__device__ __forceinline__ bool rd_keep(uint32_t id, uint32_t seed, long long nlive, int max_points) {
    if (max_points <= 0 || nlive <= max_points) return true;
    const unsigned long long thresh = (unsigned long long)((double)max_points / (double)nlive * 4294967296.0);
    return (unsigned long long)rd_hash(id, seed) < thresh;
}

struct PointArgs {
    const float4* xv;
    const unsigned int* id;
    const DevState* ds;
    int s, nx, ny, ps, width, height, max_points, phase;
    uint32_t seed;
    const unsigned int* vmax;   /* phase: bits of max |vx|, |vy| */
    unsigned int* vmax_out;     /* k_rd_vmax */
    unsigned char* layer;       /* one byte per pixel */
    unsigned char mark;         /* 1 electrons, 2 ions */
};

#define RD_TILE 1024
#define RD_SCRAMBLE 2147483647ull   /* 2^31-1, prime and above any tile count (at most 2^21):
                                      t -> t * P mod ntiles is a permutation */

__device__ __forceinline__ long long rd_tile(long long t, long long ntiles) {
    return (long long)(((unsigned long long)t * RD_SCRAMBLE) % (unsigned long long)ntiles);
}

__device__ __forceinline__ bool rd_candidate(const PointArgs& a, long long i, long long nlive, float4& p) {
    p = a.xv[i];
    if (is_dead(p.x)) return false;
    /* the position in FP32 cells (NaN for a NaN position) */
    p.x = pos_cellsf(p.x, a.ps);
    p.y = pos_cellsf(p.y, a.ps);
    if (!(p.x > 0.0f && p.x < (float)(a.nx - 1) && p.y > 0.0f && p.y < (float)(a.ny - 1))) return false;
    return rd_keep(a.id[i], a.seed, nlive, a.max_points);
}

__global__ void __launch_bounds__(256) k_rd_vmax(PointArgs a) {
    const long long n = a.ds->n[a.s], nlive = n - a.ds->dead[a.s];
    unsigned int mx = 0u, my = 0u;
    const long long ntiles = (n + RD_TILE - 1) / RD_TILE;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x)
    for (long long i = rd_tile(t, ntiles) * RD_TILE + threadIdx.x, e = min(n, rd_tile(t, ntiles) * RD_TILE + RD_TILE);
         i < e; i += blockDim.x) {
        float4 p;
        if (!rd_candidate(a, i, nlive, p)) continue;
        const float ax = fabsf(p.z), ay = fabsf(p.w);
        if (ax == ax) mx = max(mx, __float_as_uint(ax));   /* non-negative floats order as their bits */
        if (ay == ay) my = max(my, __float_as_uint(ay));
    }
    for (int d = 16; d; d >>= 1) {
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, d));
        my = max(my, __shfl_down_sync(0xffffffffu, my, d));
    }
    if ((threadIdx.x & 31) == 0) {
        if (mx) atomicMax(&a.vmax_out[0], mx);
        if (my) atomicMax(&a.vmax_out[1], my);
    }
}

/* (int) of a non-negative float, at least 1 (int maxVx, graphics.cpp:421-452) */
__device__ __forceinline__ int rd_vscale(unsigned int bits) {
    float v = __uint_as_float(bits);
    int m = v < 2147483520.0f ? (int)v : 2147483647;
    return m < 1 ? 1 : m;
}

__device__ __forceinline__ void rd_splat(const PointArgs& a, int px, int py) {
    for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
            const int x = px + dx, y = py - dy;
            if (x < 0 || x >= a.width || y < 0 || y >= a.height) continue;
            unsigned char* q = a.layer + (long long)y * a.width + x;
            if (*q != a.mark) *q = a.mark;   /* a racing store writes the same byte */
        }
}

/* layer byte -> colour: 0 black, 1 electron colour, 2 ion colour */
__global__ void k_rd_resolve(const unsigned char* layer, long long npx, Rgb c1, Rgb c2, unsigned char* img) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx; k += (long long)gridDim.x * blockDim.x) {
        const unsigned char m = layer[k];
        const Rgb c = m == 1 ? c1 : (m == 2 ? c2 : Rgb{0, 0, 0});
        img[3 * k] = c.r;
        img[3 * k + 1] = c.g;
        img[3 * k + 2] = c.b;
    }
}

__global__ void __launch_bounds__(256) k_rd_points(PointArgs a) {
    const long long n = a.ds->n[a.s], nlive = n - a.ds->dead[a.s];
    int mvx = 1, mvy = 1;
    if (a.phase) {
        mvx = rd_vscale(a.vmax[0]);
        mvy = rd_vscale(a.vmax[1]);
    }
    const float W = (float)a.width, H = (float)a.height;
    const long long ntiles = (n + RD_TILE - 1) / RD_TILE;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x)
    for (long long i = rd_tile(t, ntiles) * RD_TILE + threadIdx.x, e = min(n, rd_tile(t, ntiles) * RD_TILE + RD_TILE);
         i < e; i += blockDim.x) {
        float4 p;
        if (!rd_candidate(a, i, nlive, p)) continue;
        float fx, fy;
        if (a.phase) {
            if (!(fabsf(p.z) < (float)mvx && fabsf(p.w) < (float)mvy)) continue;
            fx = (p.z / (float)mvx + 1.0f) * 0.5f;
            fy = (p.w / (float)mvy + 1.0f) * 0.5f;
        } else {
            fx = p.x / (float)(a.nx - 1);
            fy = p.y / (float)(a.ny - 1);
        }
        int px = (int)(fx * W), py = a.height - 1 - (int)(fy * H);
        px = px < 0 ? 0 : (px > a.width - 1 ? a.width - 1 : px);
        py = py < 0 ? 0 : (py > a.height - 1 ? a.height - 1 : py);
        rd_splat(a, px, py);
    }
}

/* doubles as ordered 64-bit keys: max of keys = max of values */
__device__ __forceinline__ unsigned long long rd_key(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double rd_unkey(unsigned long long k) {
    unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    double v;
    memcpy(&v, &b, sizeof v);
    return v;
}

/* max over src[k] / div (the field the plot shows), NaN ignored */
__global__ void k_rd_fmax(const double* src, double div, int count, unsigned long long* out) {
    unsigned long long m = 0ull;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        double v = src[k] / div;
        if (v == v) m = max(m, rd_key(v));
    }
    for (int d = 16; d; d >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, d));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

/* the colour ramp of drawField (graphics.cpp:303-356): red, orange,
 * yellow, green, blue, purple; band b mixes colours b and b+1           */
__constant__ float c_ramp[6][3] = {{1.0f, 0.0f, 0.0f}, {1.0f, 0.396f, 0.0f}, {1.0f, 1.0f, 0.0f},
                                   {0.0f, 1.0f, 0.0f}, {0.0f, 0.0f, 1.0f}, {0.396f, 0.0f, 1.0f}};

__device__ __forceinline__ void rd_ramp(float zAv, float (&c)[3]) {
    const float rd = 0.2f;
    float alpha = zAv < 1.0f ? zAv : 1.0f;
    int b;
    if (zAv < rd) {
        alpha /= rd; b = 0;
    } else if ((double)zAv < 2.0 * (double)rd) {
        alpha = (alpha - rd) / rd; b = 1;
    } else if ((double)zAv < 3.0 * (double)rd) {
        alpha = (float)(((double)alpha - 2.0 * (double)rd) / (double)rd); b = 2;
    } else if ((double)zAv < 4.0 * (double)rd) {
        alpha = (float)(((double)alpha - 3.0 * (double)rd) / (double)rd); b = 3;
    } else {
        alpha = (float)(((double)alpha - 4.0 * (double)rd) / (double)rd); b = 4;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] = c_ramp[b][k] * (1.0f - alpha) + c_ramp[b + 1][k] * alpha;   /* glm::mix */
}

__global__ void k_rd_field(const double* src, double div, int n, int grid_start, const unsigned long long* fmax_key,
                           int width, int height, unsigned char* img) {
    double fmax = fabs(rd_unkey(*fmax_key));
    if (*fmax_key == 0ull || !(fmax >= 1.0)) fmax = 1.0;   /* if (fieldMax < 1.0) fieldMax = 1.0 */
    const long long npx = (long long)width * height;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < npx; k += (long long)gridDim.x * blockDim.x) {
        const int px = (int)(k % width), py = (int)(k / width);
        const float u = ((float)px + 0.5f) * (float)(n - 1) / (float)width;
        const float v = ((float)(height - 1 - py) + 0.5f) * (float)(n - 1) / (float)height;
        const int i = (int)u, j = (int)v;
        const float fu = u - (float)i, fv = v - (float)j;
        unsigned char* q = img + 3 * k;
        if (i < grid_start || i >= n - grid_start - 1 || j < grid_start || j >= n - grid_start - 1 || fu < 0.1f ||
            fu > 0.9f || fv < 0.1f || fv > 0.9f) {
            q[0] = q[1] = q[2] = 0;
            continue;
        }
        const float z0 = (float)(src[(long long)(j + 1) * n + i] / div / fmax);
        const float z1 = (float)(src[(long long)(j + 1) * n + i + 1] / div / fmax);
        const float z2 = (float)(src[(long long)j * n + i + 1] / div / fmax);
        const float z3 = (float)(src[(long long)j * n + i] / div / fmax);
        const float zAv = (float)fabs((double)(z0 + z1 + z2 + z3) / 4.0);
        float c[3];
        rd_ramp(zAv, c);
        q[0] = rd_byte(c[0]);
        q[1] = rd_byte(c[1]);
        q[2] = rd_byte(c[2]);
    }
}

int rd_fail(pgb_run* r, int code, const char* msg) {
    r->err = msg;
    return code;
}

const Rgb kLime = {142, 255, 29};      /* (0.557, 1.0, 0.114) x 255, rounded */
const Rgb kHotPink = {255, 29, 142};   /* (1.0, 0.114, 0.557) */

}  // namespace

extern "C" int pgb_render(pgb_run* r, int plot, int32_t width, int32_t height, int32_t max_points, uint32_t seed,
                          uint8_t* rgb, int64_t cap) {
    if (!r) return PGB_ERR_ARG;
    if (!rgb || width < 1 || height < 1 || width > 16384 || height > 16384 || plot < 0 || plot > PGB_PLOT_ION_DENSITY)
        return rd_fail(r, PGB_ERR_ARG, "pgb_render: bad argument (plot kind, or a size outside 1..16384)");
    const long long npx = (long long)width * height, bytes = 3 * npx;
    if (cap < bytes) return rd_fail(r, PGB_ERR_ARG, "pgb_render: rgb buffer smaller than width*height*3");
    if (plot <= PGB_PLOT_ION_VX_VY && (r->sp[0].cap == 0 || r->sp[1].cap == 0))
        return rd_fail(r, PGB_ERR_STATE, "pgb_render: load both species first");
    if (4 * npx > r->rd_cap) {   /* RGB image, then the point layer */
        PGB_CK(r, cudaStreamSynchronize(r->stream));
        cudaFree(r->rd_img);
        r->rd_img = nullptr;
        r->rd_cap = 0;
        if (cudaMalloc(&r->rd_img, (size_t)(4 * npx)) != cudaSuccess) {
            cudaGetLastError();
            return rd_fail(r, PGB_ERR_NOMEM, "pgb_render: image allocation failed");
        }
        r->rd_cap = 4 * npx;
    }
    if (!r->rd_scratch) {
        if (cudaMalloc(&r->rd_scratch, 16) != cudaSuccess) {
            cudaGetLastError();
            return rd_fail(r, PGB_ERR_NOMEM, "pgb_render: scratch allocation failed");
        }
    }
    unsigned char* img = (unsigned char*)r->rd_img;
    PGB_CK(r, cudaMemsetAsync(r->rd_scratch, 0, 16, r->stream));
    if (plot <= PGB_PLOT_ION_VX_VY) {
        unsigned char* layer = img + bytes;
        PGB_CK(r, cudaMemsetAsync(layer, 0, (size_t)npx, r->stream));
        PointArgs a;
        a.ds = r->ds; a.nx = r->nx; a.ny = r->ny; a.ps = r->ps; a.width = width; a.height = height;
        a.max_points = max_points; a.seed = seed; a.layer = layer;
        a.vmax = (const unsigned int*)r->rd_scratch;
        a.vmax_out = (unsigned int*)r->rd_scratch;
        const int blocks = r->sms * 8;
        if (plot == PGB_PLOT_PARTICLE_XY) {
            a.phase = 0;
            for (int s = 0; s < 2; ++s) {   /* electrons, then ions on top (graphics.cpp:560-606) */
                a.s = s; a.xv = r->sp[s].xv; a.id = r->sp[s].id;
                a.mark = (unsigned char)(s + 1);
                k_rd_points<<<blocks, 256, 0, r->stream>>>(a);
                r->launches++;
            }
        } else {
            const int s = plot == PGB_PLOT_ELECTRON_VX_VY ? 0 : 1;   /* lime / hot pink, graphics.cpp:692, 696 */
            a.phase = 1; a.s = s; a.xv = r->sp[s].xv; a.id = r->sp[s].id;
            a.mark = (unsigned char)(s + 1);
            k_rd_vmax<<<blocks, 256, 0, r->stream>>>(a);
            k_rd_points<<<blocks, 256, 0, r->stream>>>(a);
            r->launches += 2;
        }
        const int rb = (int)std::min<long long>((npx + 255) / 256, (long long)r->sms * 16);
        k_rd_resolve<<<rb, 256, 0, r->stream>>>(layer, npx, kLime, kHotPink, img);
        r->launches++;
    } else {
        const int nodes = r->nx * r->ny;
        const double* src = nullptr;
        double div = 1.0;
        int grid_start = 0;
        const bool averaged = r->gr.on;
        switch (plot) {
            case PGB_PLOT_PHI: src = averaged ? r->gr.f[1] : r->phi; break;
            case PGB_PLOT_EFIELD_X: src = averaged ? r->gr.f[2] : r->ex; break;
            case PGB_PLOT_EFIELD_Y: src = averaged ? r->gr.f[3] : r->ey; break;
            default: {
                const int s = plot == PGB_PLOT_E_DENSITY ? 0 : 1;
                grid_start = 1;   /* graphics.cpp:720, 727 */
                src = averaged ? r->gr.q[s] : r->q[s];
                if (!averaged) div = s == 0 ? -PGB_CHARGE : PGB_CHARGE;   /* q / qc */
            }
        }
        if (averaged) div = (double)r->gr.g.no_graph_steps;
        unsigned long long* key = (unsigned long long*)r->rd_scratch;
        k_rd_fmax<<<std::min((nodes + 255) / 256, r->sms * 4), 256, 0, r->stream>>>(src, div, nodes, key);
        const int pb = (int)std::min<long long>((npx + 255) / 256, (long long)r->sms * 16);
        k_rd_field<<<pb, 256, 0, r->stream>>>(src, div, r->nx, grid_start, key, width, height, img);
        r->launches += 2;
    }
    PGB_CK(r, cudaGetLastError());
    PGB_CK(r, cudaMemcpyAsync(rgb, img, (size_t)bytes, cudaMemcpyDeviceToHost, r->stream));
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    return 0;
}
