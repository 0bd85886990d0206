/*
 * FP32 Poisson solve by discrete sine transforms (the DST_DC mode's inner
 * solver).
 *
 * fields::grid_potential solves the 5-point discrete Poisson equation
 *   (u[i+1][j] + u[i-1][j] + u[i][j+1] + u[i][j-1] - 4 u[i][j]) / h^2 = f[i][j]
 * on the interior of an n x n grid with u = 0 on the walls (mglin.cpp:
 * 116-127 relaxes exactly this system; the walls' potentials are applied
 * afterwards).  With n = N + 1 nodes and N a power of two, the sine modes
 * sin(pi j k / N) sin(pi i l / N), 1 <= k, l <= N-1, are its eigenvectors,
 * with eigenvalues -(s_k + s_l) / h^2, s_k = 4 sin^2(pi k / 2N).  So
 *   u = (2/N)^2 DST( DST(f) * (-h^2) / (s_k + s_l) )
 * with DST the type-I sine transform along each axis,
 *   S_k = sum_{j=1}^{N-1} x_j sin(pi j k / N),
 * which is its own inverse up to the factor 2/N.  This is the exact
 * discrete solution that the multigrid approaches, up to FP32 rounding
 * (about 1e-6 of phi); an FP64 defect correction around it
 * (pgb_poisson_solve) removes that.
 *
 * A type-I sine transform of length N-1 is read off a complex FFT of
 * length M = 2N of the odd extension y = (0, x_1..x_{N-1}, 0, -x_{N-1}..
 * -x_1): Y_k = -2i S_k.  Two real sequences a, b share one FFT as
 * z = y_a + i y_b: Re Z_k = 2 S_b,k and Im Z_k = -2 S_a,k.  Three launches:
 *   k_dst_rows     row pairs (i, i+1): transform over j, stored transposed
 *                  t[k-1][i-1] (rows of N floats) for the next pass
 *   k_dst_columns  pairs of k: transform over i, division by the
 *                  eigenvalue, inverse transform over l
 *   k_dst_back     row pairs: inverse transform over k, written to u
 * Each CTA runs one radix-2 FFT of length M in shared memory (in-place,
 * decimation in time from a bit-reversed load), twiddles from a table made
 * in FP64 on the host.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <vector>
#include "pgb_internal.h"

struct DstArgs {
    const float* f;      /* n x n right-hand side (walls not read)       */
    float* u;            /* n x n solution (walls written 0)             */
    float* t;            /* (N-1) rows of N floats                       */
    const float2* tw;    /* M/2 twiddles exp(-2 pi i q / M)              */
    const float* s;      /* N values s_k = 4 sin^2(pi k / 2N)            */
    int n, N, logM;
    float scale;         /* -(2/N)^2 h^2                                 */
};

__device__ __forceinline__ int bitrev(int q, int logM) { return (int)(__brev((unsigned)q) >> (32 - logM)); }

/* stage the twiddles, then an in-place FFT of z (already bit-reversed) */
__device__ __forceinline__ void fft_inplace(float2* z, const float2* stw, int M, int logM) {
    for (int st = 0; st < logM; ++st) {
        const int h = 1 << st;
        for (int b = threadIdx.x; b < (M >> 1); b += blockDim.x) {
            const int pos = b & (h - 1);
            const int i0 = ((b >> st) << (st + 1)) + pos, i1 = i0 + h;
            const float2 w = stw[pos << (logM - 1 - st)];
            const float2 a = z[i0], c = z[i1];
            const float2 tt = make_float2(w.x * c.x - w.y * c.y, w.x * c.y + w.y * c.x);
            z[i0] = make_float2(a.x + tt.x, a.y + tt.y);
            z[i1] = make_float2(a.x - tt.x, a.y - tt.y);
        }
        __syncthreads();
    }
}

/* odd extension of the pair (a_q, b_q), q = 1..N-1, into z in bit-reversed
 * order; get(q) returns (a_q, b_q)                                       */
template <class G>
__device__ __forceinline__ void load_odd(float2* z, int N, int logM, G get) {
    const int M = 2 * N;
    for (int q = threadIdx.x; q < M; q += blockDim.x) {
        float2 v = make_float2(0.0f, 0.0f);
        if (q > 0 && q < N) v = get(q);
        else if (q > N) {
            v = get(M - q);
            v.x = -v.x;
            v.y = -v.y;
        }
        z[bitrev(q, logM)] = v;
    }
}

__device__ __forceinline__ float2* dst_smem(float2*& stw, int M) {
    extern __shared__ __align__(16) float2 smem[];
    stw = smem;              /* M/2 twiddles */
    return smem + M / 2;     /* then the FFT buffer(s) */
}

__device__ __forceinline__ void stage_twiddles(float2* stw, const float2* tw, int M) {
    for (int q = threadIdx.x; q < M / 2; q += blockDim.x) stw[q] = tw[q];
}

/* row pair p: rows i0 = 2p+1 and i0+1 (the wall row n-1 reads as 0) */
__global__ void k_dst_rows(DstArgs a) {
    pgb_pdl_entry();
    const int N = a.N, M = 2 * N, n = a.n;
    float2* stw;
    float2* z = dst_smem(stw, M);
    stage_twiddles(stw, a.tw, M);
    const int i0 = 2 * blockIdx.x + 1, i1 = i0 + 1;
    const float* ra = a.f + (size_t)i0 * n;
    const float* rb = i1 <= n - 2 ? a.f + (size_t)i1 * n : nullptr;
    load_odd(z, N, a.logM, [&](int j) { return make_float2(ra[j], rb ? rb[j] : 0.0f); });
    __syncthreads();
    fft_inplace(z, stw, M, a.logM);
    /* S_a,k = -Im Z_k / 2 (row i0), S_b,k = Re Z_k / 2 (row i1); for the
     * wall row an exact 0, not the rounding of row i0 that Re Z_k holds  */
    for (int k = 1 + threadIdx.x; k < N; k += blockDim.x) {
        const float2 Z = z[k];
        *reinterpret_cast<float2*>(a.t + (size_t)(k - 1) * N + (i0 - 1)) = make_float2(-0.5f * Z.y, rb ? 0.5f * Z.x : 0.0f);
    }
}

/* pair q of frequencies k0 = 2q+1, k1 = k0+1 (k1 = N reads as 0, not written) */
__global__ void k_dst_columns(DstArgs a) {
    pgb_pdl_entry();
    const int N = a.N, M = 2 * N;
    float2* stw;
    float2* z = dst_smem(stw, M);
    float2* z2 = z + M;
    stage_twiddles(stw, a.tw, M);
    const int k0 = 2 * blockIdx.x + 1, k1 = k0 + 1;
    float* const ta = a.t + (size_t)(k0 - 1) * N;
    float* const tb = k1 <= N - 1 ? a.t + (size_t)(k1 - 1) * N : nullptr;
    load_odd(z, N, a.logM, [&](int i) { return make_float2(ta[i - 1], tb ? tb[i - 1] : 0.0f); });
    __syncthreads();
    fft_inplace(z, stw, M, a.logM);
    /* the solution's coefficients, then their odd extension over l */
    const float sa = a.s[k0], sb = a.s[k1 < N ? k1 : 1];
    load_odd(z2, N, a.logM, [&](int l) {
        const float2 Z = z[l];
        const float sl = a.s[l];
        return make_float2((-0.5f * Z.y) * a.scale / (sa + sl), tb ? (0.5f * Z.x) * a.scale / (sb + sl) : 0.0f);
    });
    __syncthreads();
    fft_inplace(z2, stw, M, a.logM);
    for (int i = 1 + threadIdx.x; i < N; i += blockDim.x) {
        const float2 Z = z2[i];
        ta[i - 1] = -0.5f * Z.y;
        if (tb) tb[i - 1] = 0.5f * Z.x;
    }
}

/* row pair p: u rows i0 = 2p+1 and i0+1 from t's columns i0-1 and i0 */
__global__ void k_dst_back(DstArgs a) {
    pgb_pdl_entry();
    const int N = a.N, M = 2 * N, n = a.n;
    float2* stw;
    float2* z = dst_smem(stw, M);
    stage_twiddles(stw, a.tw, M);
    const int i0 = 2 * blockIdx.x + 1, i1 = i0 + 1;
    /* the wall row's slot (column N-1 of t) is never written by the column
     * pass: read it as 0, or its values would leak into row i0 through the
     * rounding of the shared transform                                    */
    const bool wall = i1 > n - 2;
    load_odd(z, N, a.logM, [&](int k) {
        const float2 v = *reinterpret_cast<const float2*>(a.t + (size_t)(k - 1) * N + (i0 - 1));
        return make_float2(v.x, wall ? 0.0f : v.y);
    });
    __syncthreads();
    fft_inplace(z, stw, M, a.logM);
    float* const ua = a.u + (size_t)i0 * n;
    float* const ub = a.u + (size_t)i1 * n;   /* i1 <= n-1: the top wall row is written 0 */
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        float va = 0.0f, vb = 0.0f;
        if (j > 0 && j < n - 1) {
            const float2 Z = z[j];
            va = -0.5f * Z.y;
            vb = i1 <= n - 2 ? 0.5f * Z.x : 0.0f;
        }
        ua[j] = va;
        ub[j] = vb;
        if (blockIdx.x == 0) a.u[j] = 0.0f;   /* the bottom wall row */
    }
}

static int dst_threads(int M) { return M / 2 < 32 ? 32 : (M / 2 > 512 ? 512 : M / 2); }

int pgb_dst_setup(pgb_run* r) {
    const int n = r->nx, N = n - 1;
    if (n != r->ny || N < 4 || (N & (N - 1))) return 0;   /* not a (2^k+1)^2 grid: the mode is refused at solve time */
    const int M = 2 * N;
    std::vector<float2> tw(M / 2);
    for (int q = 0; q < M / 2; ++q) {
        const double ang = -2.0 * M_PI * (double)q / (double)M;
        tw[q] = make_float2((float)cos(ang), (float)sin(ang));
    }
    std::vector<float> s(N);
    for (int k = 0; k < N; ++k) {
        const double v = sin(M_PI * (double)k / (2.0 * N));
        s[k] = (float)(4.0 * v * v);
    }
    PGB_CK(r, cudaMalloc(&r->dst_tw, sizeof(float2) * tw.size()));
    PGB_CK(r, cudaMalloc(&r->dst_s, sizeof(float) * s.size()));
    PGB_CK(r, cudaMalloc(&r->dst_t, sizeof(float) * (size_t)(N - 1) * N));
    PGB_CK(r, cudaMemcpy(r->dst_tw, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice));
    PGB_CK(r, cudaMemcpy(r->dst_s, s.data(), sizeof(float) * s.size(), cudaMemcpyHostToDevice));
    const int smem = (int)(sizeof(float2) * (M / 2 + 2 * M));
    if (smem > 48 * 1024) {
        PGB_CK(r, cudaFuncSetAttribute(k_dst_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        PGB_CK(r, cudaFuncSetAttribute(k_dst_columns, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        PGB_CK(r, cudaFuncSetAttribute(k_dst_back, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    }
    return 0;
}

void pgb_dst_free(pgb_run* r) {
    cudaFree(r->dst_tw);
    cudaFree(r->dst_s);
    cudaFree(r->dst_t);
    r->dst_tw = nullptr;
    r->dst_s = nullptr;
    r->dst_t = nullptr;
}

bool pgb_dst_ok(const pgb_run* r) { return r->dst_t != nullptr; }

/* u = the FP32 solution of L u = f with zero walls (f's walls not read) */
int pgb_dst_solve(pgb_run* r, const float* f, float* u) {
    if (!r->dst_t) return PGB_ERR_CUDA;
    DstArgs a;
    a.f = f; a.u = u; a.t = r->dst_t; a.tw = r->dst_tw; a.s = r->dst_s;
    a.n = r->nx; a.N = r->nx - 1;
    const int M = 2 * a.N;
    a.logM = 0;
    while ((1 << a.logM) < M) a.logM++;
    const double h = r->p.xlength / (double)a.N;
    a.scale = (float)(-(2.0 / a.N) * (2.0 / a.N) * h * h);
    const int th = dst_threads(M), blocks = a.N / 2;
    const size_t sm1 = sizeof(float2) * (M / 2 + M), sm2 = sizeof(float2) * (M / 2 + 2 * M);
    PGB_CK(r, pgb_launch_pdl(k_dst_rows, dim3(blocks), dim3(th), sm1, r->stream, a));
    PGB_CK(r, pgb_launch_pdl(k_dst_columns, dim3(blocks), dim3(th), sm2, r->stream, a));
    PGB_CK(r, pgb_launch_pdl(k_dst_back, dim3(blocks), dim3(th), sm1, r->stream, a));
    r->launches += 3;
    PGB_CK(r, cudaGetLastError());
    return 0;
}
