/*
 * Grid kernels: charge finalisation and rho, the Poisson right-hand side,
 * the full-multigrid solve and the electric field.
 *
 * Reference path: particle::collect_charge edge doubling
 * (particle.cpp:829-845), fields::grid_rho (fields.cpp:100-143),
 * fields::grid_potential (fields.cpp:169-220) with Mglin (mglin.cpp:21-196),
 * fields::grid_electric_field (fields.cpp:230-268).
 *
 * This file is compiled with --fmad=false: the FP64 multigrid performs the
 * reference's additions and multiplications one by one, in its order, so
 * that from the same right-hand side it returns the reference's potential
 * bit for bit.  Within one colour of the red-black sweep every update reads
 * only the other colour, so the order of updates inside a colour does not
 * change the result.
 *
 * Schedule (one call): restrict the right-hand side to every level, solve
 * the 3x3 grid, then for each finer level prolong and run two V(1,1)
 * cycles.  Levels with n <= PGB_MG_SMALL (65; PGB_MG_SMALL64 = 33 in FP64)
 * run inside one CTA with all their arrays in shared memory (one launch per
 * coarse sub-solve); finer levels use one launch per grid operation.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "pgb_internal.h"

/* ------------------------------------------------ charge, rho, rhs */
struct FinalizeArgs {
    const unsigned long long* acc[2];
    double* q[2];
    double* rho;
    double* f;            /* Poisson right-hand side, or null */
    int nx, ny;
    double qcdxdy[2];     /* qc/(DX*DY) per species */
    int mask;             /* species whose q is rebuilt from acc */
    double coef;          /* 1/EPSILON */
    double divdxdy;       /* 1/(DX*DY) */
    double phi0x, phi0y, phily;
    const double* phi_tab;   /* right wall: phi_tab[t - t_base] (fields.cpp:177) */
    const DevState* ds;
};

__device__ __forceinline__ double edge_factor(int i, int j, int nx, int ny) {
    bool ex = (i == 0 || i == nx - 1), ey = (j == 0 || j == ny - 1);
    /* columns doubled, rows doubled, corners doubled again (particle.cpp:830-845) */
    return (ex ? 2.0 : 1.0) * (ey ? 2.0 : 1.0) * ((ex && ey) ? 2.0 : 1.0);
}

/* RHS of fields::grid_potential (fields.cpp:184-204) for node (j, i) */
__device__ __forceinline__ double rhs_node(double rho, int i, int j, const FinalizeArgs& a, double phirx) {
    double f = -a.coef * rho;
    if (i == 1) f = f - a.phi0x * a.divdxdy;
    if (i == a.nx - 2) f = f - phirx * a.divdxdy;
    if (j == 1) f = f - a.phi0y * a.divdxdy;
    if (j == a.ny - 2) f = f - a.phily * a.divdxdy;
    return f;
}

__global__ void k_finalize(FinalizeArgs a) {
    pgb_pdl_entry();
    const int G = a.nx * a.ny;
    const double phirx = a.phi_tab[a.ds->tf - a.ds->t_base];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < G; k += gridDim.x * blockDim.x) {
        int j = k / a.nx, i = k - j * a.nx;
        double ef = edge_factor(i, j, a.nx, a.ny);
        for (int s = 0; s < 2; ++s)
            if (a.mask & (1 << s)) {
                double v = (double)(long long)a.acc[s][k] * (1.0 / PGB_FIX_SCALE);
                a.q[s][k] = (v * a.qcdxdy[s]) * ef;
            }
        double rho = a.q[1][k] + a.q[0][k];
        a.rho[k] = rho;
        if (a.f) a.f[k] = rhs_node(rho, i, j, a, phirx);
    }
}

__global__ void k_rhs(FinalizeArgs a) {
    pgb_pdl_entry();
    const int G = a.nx * a.ny;
    const double phirx = a.phi_tab[a.ds->tf - a.ds->t_base];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < G; k += gridDim.x * blockDim.x) {
        int j = k / a.nx, i = k - j * a.nx;
        a.f[k] = rhs_node(a.rho[k], i, j, a, phirx);
    }
}

/* ------------------------------------------------------ multigrid ops */
/* red-black Gauss-Seidel update of one point (mglin.cpp:116-127) */
template <class T>
__device__ __forceinline__ T gs_point(const T* u, const T* f, int n, int i, int j, T h2) {
    return (T)0.25 * (u[(i + 1) * n + j] + u[(i - 1) * n + j] + u[i * n + j + 1] + u[i * n + j - 1] - h2 * f[i * n + j]);
}
/* minus the residual at an interior point (mglin.cpp:133-141) */
template <class T>
__device__ __forceinline__ T resid_point(const T* u, const T* f, int n, int i, int j, T h2i) {
    return -h2i * (u[(i + 1) * n + j] + u[(i - 1) * n + j] + u[i * n + j + 1] + u[i * n + j - 1] - (T)4.0 * u[i * n + j]) +
           f[i * n + j];
}
/* half-weighting of the fine residual onto coarse interior point (ic,jc)
 * (mglin.cpp:151-160 applied to resid's output)                         */
template <class T>
__device__ __forceinline__ T restrict_resid_point(const T* u, const T* f, int nf, int ic, int jc, T h2i) {
    int i = 2 * ic, j = 2 * jc;
    T c = resid_point(u, f, nf, i, j, h2i);
    T n1 = resid_point(u, f, nf, i + 1, j, h2i), n2 = resid_point(u, f, nf, i - 1, j, h2i);
    T n3 = resid_point(u, f, nf, i, j + 1, h2i), n4 = resid_point(u, f, nf, i, j - 1, h2i);
    return (T)0.5 * c + (T)0.125 * (n1 + n2 + n3 + n4);
}
template <class T>
__device__ __forceinline__ T restrict_point(const T* uf, int nf, int ic, int jc) {
    int i = 2 * ic, j = 2 * jc;
    return (T)0.5 * uf[i * nf + j] + (T)0.125 * (uf[(i + 1) * nf + j] + uf[(i - 1) * nf + j] + uf[i * nf + j + 1] + uf[i * nf + j - 1]);
}
/* bilinear prolongation value at fine point (i,j) (mglin.cpp:70-82) */
template <class T>
__device__ __forceinline__ T prolong_point(const T* uc, int nc, int i, int j) {
    if ((j & 1) == 0) {
        if ((i & 1) == 0) return uc[(i >> 1) * nc + (j >> 1)];
        return (T)0.5 * (uc[((i + 1) >> 1) * nc + (j >> 1)] + uc[((i - 1) >> 1) * nc + (j >> 1)]);
    }
    T a, b;   /* values of the two even columns next to j, in row i */
    if ((i & 1) == 0) {
        a = uc[(i >> 1) * nc + ((j + 1) >> 1)];
        b = uc[(i >> 1) * nc + ((j - 1) >> 1)];
    } else {
        a = (T)0.5 * (uc[((i + 1) >> 1) * nc + ((j + 1) >> 1)] + uc[((i - 1) >> 1) * nc + ((j + 1) >> 1)]);
        b = (T)0.5 * (uc[((i + 1) >> 1) * nc + ((j - 1) >> 1)] + uc[((i - 1) >> 1) * nc + ((j - 1) >> 1)]);
    }
    return (T)0.5 * (a + b);
}

/* ------------------------------------------------ grid-wide launches */
/* One red-black Gauss-Seidel relaxation (both colours, mglin.cpp:116-127)
 * on a RT x RTX tile of interior points.  The tile and a two-point halo
 * of u are staged in shared memory; red points of the tile and of a
 * one-point ring are updated (the ring values are recomputed by the
 * neighbouring tiles too, from the same inputs, so they agree), then the
 * black points of the tile, which read only updated red values.  The
 * result equals the two separate colour sweeps bit for bit.
 * The sweep reads uin and writes the tile's interior to uout, a different
 * buffer: relaxing in place would let a block load a halo that the
 * neighbouring block has already overwritten, whenever the two blocks do
 * not run at the same time.  uout's walls are never written (they stay 0).
 * mode 0: relax uin
 * mode 1: uin + prolong(vc) first (addint, mglin.cpp:90-97), then relax
 * mode 2: prolong(vc) first (FMG interpolation, mglin.cpp:49), then relax;
 *         uin is not read
 * mode 3: relax from u = 0 (a correction's first smoothing); neither uin
 *         nor vc is read                                                  */
#define RT 8
#define RTX 32
template <class T, int MODE>
__global__ void __launch_bounds__(RT * RTX) k_relax_tile(const T* __restrict__ uin, T* __restrict__ uout, const T* f, int n,
                                                          T h2, const T* vc) {
    pgb_pdl_entry();
    __shared__ T su[RT + 4][RTX + 4];
    __shared__ T sf[RT + 2][RTX + 2];
    const int nc = n / 2 + 1;
    const int i0 = 1 + blockIdx.y * RT, j0 = 1 + blockIdx.x * RTX;   /* first interior point of the tile */
    const int tid = threadIdx.y * RTX + threadIdx.x;
    for (int k = tid; k < (RT + 4) * (RTX + 4); k += RT * RTX) {
        int li = k / (RTX + 4), lj = k - li * (RTX + 4);
        int i = i0 - 2 + li, j = j0 - 2 + lj;
        T v = (T)0;
        if (i >= 0 && j >= 0 && i < n && j < n) {
            if (MODE == 3) v = (T)0;
            else if (MODE == 2) v = prolong_point(vc, nc, i, j);
            else {
                v = uin[i * n + j];
                if (MODE == 1) v = v + prolong_point(vc, nc, i, j);
            }
        }
        su[li][lj] = v;
    }
    for (int k = tid; k < (RT + 2) * (RTX + 2); k += RT * RTX) {
        int li = k / (RTX + 2), lj = k - li * (RTX + 2);
        int i = i0 - 1 + li, j = j0 - 1 + lj;
        sf[li][lj] = (i >= 0 && j >= 0 && i < n && j < n) ? f[i * n + j] : (T)0;
    }
    __syncthreads();
    /* red: (i+j) even, on the tile and its one-point ring */
    for (int k = tid; k < (RT + 2) * (RTX + 2); k += RT * RTX) {
        int li = k / (RTX + 2), lj = k - li * (RTX + 2);
        int i = i0 - 1 + li, j = j0 - 1 + lj;
        if (i >= 1 && j >= 1 && i < n - 1 && j < n - 1 && ((i + j) & 1) == 0) {
            int a = li + 1, b = lj + 1;
            su[a][b] = (T)0.25 * (su[a + 1][b] + su[a - 1][b] + su[a][b + 1] + su[a][b - 1] - h2 * sf[li][lj]);
        }
    }
    __syncthreads();
    /* black: (i+j) odd, on the tile */
    {
        int li = threadIdx.y, lj = threadIdx.x;
        int i = i0 + li, j = j0 + lj;
        if (i < n - 1 && j < n - 1 && ((i + j) & 1) == 1) {
            int a = li + 2, b = lj + 2;
            su[a][b] = (T)0.25 * (su[a + 1][b] + su[a - 1][b] + su[a][b + 1] + su[a][b - 1] - h2 * sf[li + 1][lj + 1]);
        }
    }
    __syncthreads();
    /* write back the tile; the walls of every level stay 0 (mglin.cpp:103-110,
     * 143: the coarse solve, the residual and so every correction vanish
     * there), so they are never rewritten                                 */
    {
        int li = threadIdx.y, lj = threadIdx.x;
        int i = i0 + li, j = j0 + lj;
        if (i < n - 1 && j < n - 1) uout[i * n + j] = su[li + 2][lj + 2];
    }
}

/* minus the residual, half-weighted onto the coarse grid (mglin.cpp:133-169);
 * also zeroes the coarse correction vc that the next level starts from    */
template <class T>
__global__ void k_resid_restrict(T* rc, T* vc, const T* u, const T* f, int nf, T h2i) {
    pgb_pdl_entry();
    const int nc = (nf + 1) / 2;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc * nc; k += gridDim.x * blockDim.x) {
        int ic = k / nc, jc = k - ic * nc;
        T v = (T)0;
        if (ic > 0 && jc > 0 && ic < nc - 1 && jc < nc - 1) v = restrict_resid_point(u, f, nf, ic, jc, h2i);
        rc[k] = v;
        vc[k] = (T)0;
    }
}
template <class T>
__global__ void k_restrict(T* uc, const T* uf, int nc) {
    pgb_pdl_entry();
    const int nf = 2 * nc - 1;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nc * nc; k += gridDim.x * blockDim.x) {
        int ic = k / nc, jc = k - ic * nc;
        T v;
        if (ic > 0 && jc > 0 && ic < nc - 1 && jc < nc - 1) v = restrict_point(uf, nf, ic, jc);
        else v = uf[(2 * ic) * nf + 2 * jc];   /* injected boundary (mglin.cpp:161-168) */
        uc[k] = v;
    }
}
/* --------------------------------------- one-CTA solver for coarse levels */
/* Shared-memory image of levels 0..J (n_l = 2^(l+1)+1).  U/F: a level's
 * solution and right-hand side when it is the top of a V-cycle (every
 * level of a full multigrid), V/R: correction and restricted residual of
 * the levels below the top, so levels 0..J-1 only (J = 5, 65 nodes:
 * 2*5718 + 2*1493 values).                                               */
__host__ __device__ __forceinline__ int small_nodes_below(int l) {
    /* sum_{m<l} (2^(m+1)+1)^2 = 4(4^l-1)/3 + 4(2^l-1) + l */
    return (4 * ((1 << (2 * l)) - 1)) / 3 + 4 * ((1 << l) - 1) + l;
}
template <class T>
struct SmallMG {
    T* base;
    T length;
    int J;
    __device__ __forceinline__ int n(int l) const { return (1 << (l + 1)) + 1; }
    /* addresses are register arithmetic (a pointer table indexed by level
     * would live in local memory)                                        */
    __device__ __forceinline__ T* U(int l) const { return base + 2 * small_nodes_below(l); }
    __device__ __forceinline__ T* F(int l) const { return U(l) + n(l) * n(l); }
    __device__ __forceinline__ T* V(int l) const { return base + 2 * small_nodes_below(J + 1) + 2 * small_nodes_below(l); }
    __device__ __forceinline__ T* R(int l) const { return V(l) + n(l) * n(l); }
};

/* Loops of the one-CTA solver run over flat point indices so that every
 * lane has work (FP64 issue slots are scarce).  Rows are found without an
 * integer division: a relaxation colour has (n-1)/2 points per row, a
 * power of two; other grids use row = (int)((k + 0.5) / n) in FP32, exact
 * for k < 2^16 since k + 0.5 is never within FP32 rounding of a multiple
 * of n.                                                                  */
__device__ __forceinline__ int sm_row(int k, float inv_n) { return (int)(((float)k + 0.5f) * inv_n); }

/* Who works on a level.  Levels of 33 nodes and more use the whole CTA
 * and __syncthreads.  Levels of 17 nodes and fewer (at most 289 points)
 * use threads 0..255 and named barrier 1: with all 32 warps, every phase
 * of a small level would cost each scheduler the issue of eight warps'
 * loop code for a handful of points.  Every point is updated by the same
 * arithmetic whichever team updates it.                                  */
struct TeamCta {
    static __device__ __forceinline__ int size() { return blockDim.x; }
    static __device__ __forceinline__ void sync() { __syncthreads(); }
};
struct TeamSmall {   /* threads 0..255 only */
    static __device__ __forceinline__ int size() { return 256; }
    static __device__ __forceinline__ void sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
};

template <class T, class Tm>
__device__ __forceinline__ void sm_relax(T* u, const T* f, int n, T length) {
    T h = length / (T)(n - 1), h2 = h * h;
    const int m = n - 2, per_row = (n - 1) >> 1, sh = __ffs(per_row) - 1;
    for (int color = 0; color < 2; ++color) {
        for (int t = threadIdx.x; t < m * per_row; t += Tm::size()) {
            int r = t >> sh, c = t & (per_row - 1);
            int i = r + 1, j = 1 + ((i + 1 + color) & 1) + 2 * c;
            if (j <= n - 2) u[i * n + j] = gs_point(u, f, n, i, j, h2);
        }
        Tm::sync();
    }
}
/* the FMG interpolation u = P(uc) (mglin.cpp:49) followed by one
 * red-black sweep, as one sweep fewer: the red sweep reads only black
 * points and walls, so it interpolates the ones it reads (the same values,
 * so the same bits); the walls get their interpolated values; the black
 * sweep then overwrites the black points, whose interpolated values
 * nothing else would have read.                                          */
template <class T, class Tm>
__device__ __forceinline__ void sm_relax_from_coarse(T* u, const T* f, int n, T length, const T* uc, int nc) {
    T h = length / (T)(n - 1), h2 = h * h;
    const int m = n - 2, per_row = (n - 1) >> 1, sh = __ffs(per_row) - 1;
    for (int t = threadIdx.x; t < m * per_row; t += Tm::size()) {
        int r = t >> sh, c = t & (per_row - 1);
        int i = r + 1, j = 1 + ((i + 1) & 1) + 2 * c;
        if (j <= n - 2) {
            T a = prolong_point(uc, nc, i + 1, j), b = prolong_point(uc, nc, i - 1, j);
            T e = prolong_point(uc, nc, i, j + 1), w = prolong_point(uc, nc, i, j - 1);
            u[i * n + j] = (T)0.25 * (a + b + e + w - h2 * f[i * n + j]);
        }
    }
    for (int t = threadIdx.x; t < 4 * (n - 1); t += Tm::size()) {
        const int side = t / (n - 1), k = t - side * (n - 1);
        const int i = side == 0 ? 0 : side == 1 ? k : side == 2 ? n - 1 : n - 1 - k;
        const int j = side == 0 ? k : side == 1 ? n - 1 : side == 2 ? n - 1 - k : 0;
        u[i * n + j] = prolong_point(uc, nc, i, j);
    }
    Tm::sync();
    for (int t = threadIdx.x; t < m * per_row; t += Tm::size()) {
        int r = t >> sh, c = t & (per_row - 1);
        int i = r + 1, j = 1 + (i & 1) + 2 * c;
        if (j <= n - 2) u[i * n + j] = gs_point(u, f, n, i, j, h2);
    }
    Tm::sync();
}
template <class T, class Tm>
__device__ __forceinline__ void sm_coarsest(T* u, const T* f, T length) {
    if (threadIdx.x == 0) {
        T h = (T)0.5 * length;
        for (int k = 0; k < 9; ++k) u[k] = (T)0;
        u[4] = -h * h * f[4] / (T)4.0;   /* mglin.cpp:103-110 */
    }
    Tm::sync();
}
/* level l of a V-cycle whose top is j, on the way down: smooth, then the
 * restricted residual and a zero correction on level l-1               */
template <class T, class Tm>
__device__ __forceinline__ void sm_down(const SmallMG<T>& s, int j, int l, T* u, const T* f, const T* from = nullptr) {
    T* ul = (l == j) ? u : s.V(l);
    const T* fl = (l == j) ? f : s.R(l);
    const int nf = s.n(l), nc = s.n(l - 1);
    const T h = s.length / (T)(nf - 1), h2i = (T)1.0 / (h * h);
    if (from) sm_relax_from_coarse<T, Tm>(ul, fl, nf, s.length, from, nc);
    else sm_relax<T, Tm>(ul, fl, nf, s.length);
    const float inv = 1.0f / (float)nc;
    T* const rc = s.R(l - 1);
    T* const vc = s.V(l - 1);
    for (int k = threadIdx.x; k < nc * nc; k += Tm::size()) {
        int ic = sm_row(k, inv), jc = k - ic * nc;
        T v = (T)0;
        if (ic > 0 && jc > 0 && ic < nc - 1 && jc < nc - 1) v = restrict_resid_point(ul, fl, nf, ic, jc, h2i);
        rc[k] = v;
        vc[k] = (T)0;
    }
    Tm::sync();
}
/* level l on the way up: add the prolongated correction (addint,
 * mglin.cpp:90-97), then smooth.  The red sweep reads only black points
 * and walls, the black sweep only red points and walls, and neither reads
 * the point it updates; so the red sweep adds the correction to the values
 * it reads (the same sums as after a separate pass, so the same bits), the
 * red points' own corrected values would be overwritten unread, and the
 * black sweep then overwrites the black points.  The walls' correction is
 * +0 and leaves them as they are.  One pass and one barrier fewer.       */
template <class T, class Tm>
__device__ __forceinline__ void sm_up(const SmallMG<T>& s, int j, int l, T* u, const T* f) {
    T* ul = (l == j) ? u : s.V(l);
    const T* fl = (l == j) ? f : s.R(l);
    const int n = s.n(l), nc = s.n(l - 1);
    const T* vc = s.V(l - 1);
    T h = s.length / (T)(n - 1), h2 = h * h;
    const int m = n - 2, per_row = (n - 1) >> 1, sh = __ffs(per_row) - 1;
    for (int t = threadIdx.x; t < m * per_row; t += Tm::size()) {
        int r = t >> sh, c = t & (per_row - 1);
        int i = r + 1, jj = 1 + ((i + 1) & 1) + 2 * c;
        if (jj <= n - 2) {
            T a = ul[(i + 1) * n + jj] + prolong_point(vc, nc, i + 1, jj);
            T b = ul[(i - 1) * n + jj] + prolong_point(vc, nc, i - 1, jj);
            T e = ul[i * n + jj + 1] + prolong_point(vc, nc, i, jj + 1);
            T w = ul[i * n + jj - 1] + prolong_point(vc, nc, i, jj - 1);
            ul[i * n + jj] = (T)0.25 * (a + b + e + w - h2 * fl[i * n + jj]);
        }
    }
    Tm::sync();
    for (int t = threadIdx.x; t < m * per_row; t += Tm::size()) {
        int r = t >> sh, c = t & (per_row - 1);
        int i = r + 1, jj = 1 + (i & 1) + 2 * c;
        if (jj <= n - 2) ul[i * n + jj] = gs_point(ul, fl, n, i, jj, h2);
    }
    Tm::sync();
}
/* the part of a V-cycle (top j) from level l (at most 17 nodes) down to
 * the coarsest solve and back up to l; entered by threads 0..255 only   */
template <class T>
__device__ __forceinline__ void sm_vcycle_small(const SmallMG<T>& s, int j, int l, T* u, const T* f,
                                                const T* from = nullptr) {
    for (int m = l; m >= 1; --m) sm_down<T, TeamSmall>(s, j, m, u, f, m == j ? from : nullptr);
    if (j == 0) sm_coarsest<T, TeamSmall>(u, f, s.length);
    else sm_coarsest<T, TeamSmall>(s.V(0), s.R(0), s.length);
    for (int m = 1; m <= l; ++m) sm_up<T, TeamSmall>(s, j, m, u, f);
}
/* V-cycle at level j on (u, f) using V/R of the levels below; all threads.
 * from: the coarser level to interpolate u from first (FMG), or null.   */
template <class T>
__device__ __forceinline__ void sm_vcycle(const SmallMG<T> s, int j, T* u, const T* f, const T* from = nullptr) {
    int l = j;
    for (; l >= 1 && s.n(l) >= 33; --l) sm_down<T, TeamCta>(s, j, l, u, f, l == j ? from : nullptr);
    if (threadIdx.x < 256) sm_vcycle_small(s, j, l, u, f, l == j ? from : nullptr);
    __syncthreads();
    for (int m = l + 1; m <= j; ++m) sm_up<T, TeamCta>(s, j, m, u, f);
}

/* mode 0: full multigrid from level 0 to J on the rhs g_f[J] (the coarser
 *         right-hand sides are restricted here); writes u_J to g_u[J].
 * mode 1: one V-cycle at level J on (g_v[J], g_r[J]) in place.          */
template <class T>
__global__ void __launch_bounds__(1024, 1) k_mg_small(int J, int mode, T length, T** g_u, T** g_f, T** g_v, T** g_r) {
    pgb_pdl_entry();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmallMG<T> s;
    s.base = reinterpret_cast<T*>(smem_raw);
    s.length = length;
    s.J = J;
    if (mode == 0) {
        const T* gf = g_f[J];
        T* const fJ = s.F(J);
        for (int k = threadIdx.x; k < s.n(J) * s.n(J); k += blockDim.x) fJ[k] = gf[k];
        __syncthreads();
        /* right-hand sides of the coarser levels, as k_restrict computes them */
        for (int l = J - 1; l >= 0; --l) {
            const int nc = s.n(l), nf = s.n(l + 1);
            const float inv = 1.0f / (float)nc;
            for (int k = threadIdx.x; k < nc * nc; k += blockDim.x) {
                int ic = sm_row(k, inv), jc = k - ic * nc;
                s.F(l)[k] = (ic > 0 && jc > 0 && ic < nc - 1 && jc < nc - 1) ? restrict_point(s.F(l + 1), nf, ic, jc)
                                                                             : s.F(l + 1)[(2 * ic) * nf + 2 * jc];
            }
            __syncthreads();
        }
        /* the FMG levels of at most 17 nodes (l <= 3) by threads 0..255 */
        const int ls = J < 3 ? J : 3;
        if (threadIdx.x < 256) {
            sm_coarsest<T, TeamSmall>(s.U(0), s.F(0), length);
            for (int l = 1; l <= ls; ++l)
                for (int c = 0; c < 2; ++c) sm_vcycle_small(s, l, l, s.U(l), s.F(l), c == 0 ? s.U(l - 1) : nullptr);
        }
        __syncthreads();
        for (int l = ls + 1; l <= J; ++l)
            for (int c = 0; c < 2; ++c) sm_vcycle(s, l, s.U(l), s.F(l), c == 0 ? s.U(l - 1) : nullptr);
        T* const gu = g_u[J];
        const T* uJ = s.U(J);
        for (int k = threadIdx.x; k < s.n(J) * s.n(J); k += blockDim.x) gu[k] = uJ[k];
    } else {
        int n = s.n(J);
        T* const gv = g_v[J];
        const T* gr = g_r[J];
        T* const uJ = s.U(J);
        T* const fJ = s.F(J);
        for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
            uJ[k] = gv[k];
            fJ[k] = gr[k];
        }
        __syncthreads();
        sm_vcycle(s, J, uJ, fJ);
        for (int k = threadIdx.x; k < n * n; k += blockDim.x) gv[k] = uJ[k];
    }
}

static size_t small_smem_bytes(int J, size_t elem) {
    return (size_t)(2 * small_nodes_below(J + 1) + 2 * small_nodes_below(J)) * elem;
}

/* ------------------------------------------------------- E field */
/* fields::grid_electric_field (fields.cpp:230-268) in the stride-nx layout
 * of an (nx+1)*(ny+1) buffer; also writes the FP32 {Ex,Ey} copy read by
 * the gather.                                                           */
__device__ __forceinline__ double ex_interior(const double* phi, int nx, int ny, int j, int i, double twoDX) {
    if (j < 1 || j > ny - 2 || i < 1 || i > nx - 2) return 0.0;
    return (phi[j * nx + i - 1] - phi[j * nx + i + 1]) / twoDX;
}
__device__ __forceinline__ double ey_interior(const double* phi, int nx, int ny, int j, int i, double twoDX) {
    if (j < 1 || j > ny - 2 || i < 1 || i > nx - 2) return 0.0;
    return (phi[(j - 1) * nx + i] - phi[(j + 1) * nx + i]) / twoDX;
}
__global__ void k_efield(const double* phi, double* Ex, double* Ey, float2* exy, int nx, int ny, double twoDX,
                         DevState* ds, int advance) {
    pgb_pdl_entry();
    /* the last kernel of a field solve moves the field step counter on */
    if (advance && blockIdx.x == 0 && threadIdx.x == 0) ds->tf += 1;
    const int GE = (nx + 1) * (ny + 1);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < GE; k += gridDim.x * blockDim.x) {
        double ex = 0.0, ey = 0.0;
        if (k < nx * ny) {
            int j = k / nx, i = k - j * nx;
            if (i == 0) ex = 2.0 * ex_interior(phi, nx, ny, j, 1, twoDX) - ex_interior(phi, nx, ny, j, 2, twoDX);
            else if (i == nx - 1) ex = 2.0 * ex_interior(phi, nx, ny, j, nx - 2, twoDX) - ex_interior(phi, nx, ny, j, nx - 3, twoDX);
            else ex = ex_interior(phi, nx, ny, j, i, twoDX);
            if (j == 0) ey = 2.0 * ey_interior(phi, nx, ny, 1, i, twoDX) - ey_interior(phi, nx, ny, 2, i, twoDX);
            else if (j == ny - 1) ey = 2.0 * ey_interior(phi, nx, ny, ny - 2, i, twoDX) - ey_interior(phi, nx, ny, ny - 3, i, twoDX);
            else ey = ey_interior(phi, nx, ny, j, i, twoDX);
        }
        Ex[k] = ex;
        Ey[k] = ey;
        exy[k] = make_float2((float)ex, (float)ey);
    }
}

__global__ void k_walls(double* phi, int nx, int ny, double phi0x, const double* phi_tab, const DevState* ds,
                        double phi0y, double phily) {
    pgb_pdl_entry();
    const double phirx = phi_tab[ds->tf - ds->t_base];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nx * ny; k += gridDim.x * blockDim.x) {
        int j = k / nx, i = k - j * nx;
        /* fields.cpp:209-219: columns first, then rows overwrite the corners */
        if (j == 0) phi[k] = phi0y;
        else if (j == ny - 1) phi[k] = phily;
        else if (i == 0) phi[k] = phi0x;
        else if (i == nx - 1) phi[k] = phirx;
    }
}

/* ====================================================== host side */
static FinalizeArgs fin_args(pgb_run* r, int mask, bool rhs) {
    FinalizeArgs a;
    a.acc[0] = r->qacc[0]; a.acc[1] = r->qacc[1];
    a.q[0] = r->q[0]; a.q[1] = r->q[1];
    a.rho = r->rho; a.f = rhs ? r->mg_f[r->ng - 1] : nullptr;
    a.nx = r->nx; a.ny = r->ny;
    a.qcdxdy[0] = r->sp[0].qc / (r->dx * r->dy);
    a.qcdxdy[1] = r->sp[1].qc / (r->dx * r->dy);
    a.mask = mask;
    a.coef = 1.0 / 8.854e-12;
    a.divdxdy = 1.0 / (r->dx * r->dy);
    a.phi0x = r->p.phi_left; a.phi0y = r->p.phi_bottom; a.phily = r->p.phi_top;
    a.phi_tab = r->phi_tab; a.ds = r->ds;
    return a;
}

int pgb_launch_finalize(pgb_run* r, int mask, bool make_rhs) {
    FinalizeArgs a = fin_args(r, mask, make_rhs);
    int G = r->nx * r->ny;
    PGB_CK(r, pgb_launch_pdl(k_finalize, dim3((G + 255) / 256), dim3(256), 0, r->stream, a));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_rhs(pgb_run* r) {
    FinalizeArgs a = fin_args(r, 0, true);
    int G = r->nx * r->ny;
    PGB_CK(r, pgb_launch_pdl(k_rhs, dim3((G + 255) / 256), dim3(256), 0, r->stream, a));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

static int blocks_for(long long work) {
    long long b = (work + 255) / 256;
    if (b < 1) b = 1;
    if (b > 65535) b = 65535;
    return (int)b;
}

/* per-level device pointer tables for the small solver */
struct MgTables {
    double** u;
    double** f;
    double** v;
    double** r;
};

template <class T>
static int small_launch(pgb_run* r, T** tab, int J, int mode) {
    size_t smem = small_smem_bytes(J, sizeof(T));
    PGB_CK(r, pgb_launch_pdl(k_mg_small<T>, dim3(1), dim3(1024), smem, r->stream, J, mode, (T)r->p.xlength, tab, tab + PGB_MAX_LEVELS,
                                                tab + 2 * PGB_MAX_LEVELS, tab + 3 * PGB_MAX_LEVELS));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

/* level arrays of one precision */
template <class T>
struct Levels {
    T** u;
    T** f;
    T** v;
    T** rr;
    T** tab;   /* device copy: u, f, v, r tables */
    T** w;     /* pre-smoothing results */
};
static Levels<double> levels64(pgb_run* r) { return {r->mg_u, r->mg_f, r->mg_v, r->mg_r, r->mg_tab, r->mg_w}; }
static Levels<float> levels32(pgb_run* r) { return {r->mg32_u, r->mg32_f, r->mg32_v, r->mg32_r, r->mg32_tab, r->mg32_w}; }

template <class T, int MODE>
static int relax_launch(pgb_run* r, const T* uin, T* uout, const T* f, int n, T h2, const T* vc) {
    dim3 grid((n - 2 + RTX - 1) / RTX, (n - 2 + RT - 1) / RT), block(RTX, RT);
    PGB_CK(r, pgb_launch_pdl(k_relax_tile<T, MODE>, dim3(grid), dim3(block), 0, r->stream, uin, uout, f, n, h2, vc));
    r->launches++;
    return 0;
}

/* V-cycle at level j > small on (u, f) (mglin.cpp:176-196).  first_mode 2
 * replaces u by the prolongation of the coarser level before the
 * pre-smoothing (the FMG interpolation of mglin.cpp:49); first_mode 3
 * starts from u = 0 without reading it (a defect correction).  The
 * pre-smoothing goes from u to the level's spare buffer w, the residual is
 * taken there, and the post-smoothing goes from w back to u.  A level has
 * one V-cycle in flight at a time, so one spare buffer per level serves.  */
template <class T>
static int vcycle(pgb_run* r, const Levels<T>& L, int j, int jsmall, T* u, const T* f, int first_mode,
                  const T* coarse_u) {
    int nf = r->mg_n[j], nc = r->mg_n[j - 1];
    T h = (T)r->p.xlength / (T)(nf - 1), h2 = h * h, h2i = (T)1.0 / (h * h);
    T* w = L.w[j];
    int rc = first_mode == 2   ? relax_launch<T, 2>(r, nullptr, w, f, nf, h2, coarse_u)
             : first_mode == 3 ? relax_launch<T, 3>(r, nullptr, w, f, nf, h2, nullptr)
                               : relax_launch<T, 0>(r, u, w, f, nf, h2, nullptr);
    if (rc) return rc;
    PGB_CK(r, pgb_launch_pdl(k_resid_restrict<T>, dim3(blocks_for((long long)nc * nc)), dim3(256), 0, r->stream, L.rr[j - 1], L.v[j - 1], w, f, nf, h2i));
    r->launches++;
    if (j - 1 <= jsmall) {
        if (small_launch<T>(r, L.tab, j - 1, 1)) return PGB_ERR_CUDA;
    } else {
        if (vcycle<T>(r, L, j - 1, jsmall, L.v[j - 1], L.rr[j - 1], 0, nullptr)) return PGB_ERR_CUDA;
    }
    if ((rc = relax_launch<T, 1>(r, w, u, f, nf, h2, L.v[j - 1]))) return rc;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

/* top level of the one-CTA solver.  FP32 levels up to 65 nodes are faster
 * in one CTA than as separate launches; at 129 nodes one SM is slower than
 * the level's three launches (measured: 10 us more a V-cycle).  FP64 runs
 * at a small fraction of the FP32 rate, and one SM is too slow for more
 * than 33 nodes.                                                        */
static int small_top(pgb_run* r, size_t elem) {
    const int lim = elem == sizeof(float) ? PGB_MG_SMALL : PGB_MG_SMALL64;
    int jsmall = 0;
    while (jsmall + 1 < r->ng && r->mg_n[jsmall + 1] <= lim) jsmall++;
    return jsmall;
}

/* Mglin on the rhs in f[ng-1]; result in u[ng-1] */
template <class T>
static int fmg(pgb_run* r, const Levels<T>& L) {
    const int ng = r->ng;
    int jsmall = small_top(r, sizeof(T));
    /* the one-CTA solver restricts the levels below jsmall itself */
    for (int j = ng - 2; j >= jsmall; --j) {
        int nc = r->mg_n[j];
        PGB_CK(r, pgb_launch_pdl(k_restrict<T>, dim3(blocks_for((long long)nc * nc)), dim3(256), 0, r->stream, L.f[j], L.f[j + 1], nc));
        r->launches++;
    }
    if (small_launch<T>(r, L.tab, jsmall, 0)) return PGB_ERR_CUDA;
    for (int j = jsmall + 1; j < ng; ++j)
        for (int c = 0; c < 2; ++c)
            if (vcycle<T>(r, L, j, jsmall, L.u[j], L.f[j], c == 0 ? 2 : 0, L.u[j - 1])) return PGB_ERR_CUDA;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

/* One defect-correction update: u' = u + e in FP64 (u' = e on the first
 * pass, when u is null), written to a second buffer so that neighbours
 * read the old values, and the FP64 defect d = f - L u' of the interior
 * (zero on the walls) stored as FP32 for the next FP32 correction.  The
 * walls of u, e and so u' are 0.                                         */
__global__ void k_dc_update(const double* __restrict__ u, const float* __restrict__ e, double* __restrict__ uout,
                            const double* __restrict__ f, float* __restrict__ d, int n, double h2i) {
    pgb_pdl_entry();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n * n; k += gridDim.x * blockDim.x) {
        int i = k / n, j = k - i * n;
        auto U = [&](int q) { return u ? u[q] + (double)e[q] : (double)e[q]; };
        double c = U(k), v = 0.0;
        if (i > 0 && j > 0 && i < n - 1 && j < n - 1)
            v = f[k] - h2i * (U(k + n) + U(k - n) + U(k + 1) + U(k - 1) - 4.0 * c);
        uout[k] = c;
        d[k] = (float)v;
    }
}
/* the last correction: phi = u + e in FP64 (the walls are set after) */
__global__ void k_dc_final(double* __restrict__ phi, const double* __restrict__ u, const float* __restrict__ e,
                           int count) {
    pgb_pdl_entry();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x)
        phi[k] = u[k] + (double)e[k];
}
/* DST_DC: the FP32 right-hand side of the charge alone, -rho/EPSILON on
 * the interior (the walls' terms are in the wall solutions)             */
__global__ void k_rho32(float* __restrict__ f32, const double* __restrict__ rho, int n, double coef) {
    pgb_pdl_entry();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n * n; k += gridDim.x * blockDim.x) {
        int i = k / n, j = k - i * n;
        f32[k] = (i > 0 && j > 0 && i < n - 1 && j < n - 1) ? (float)(-coef * rho[k]) : 0.0f;
    }
}
/* DST_DC's first update: u = wc + phi_right(t) * wr + e (the walls' FP64
 * solutions and the FP32 solve of the charge term), and the FP64 defect
 * d = f - L u of the full right-hand side, as k_dc_update            */
__global__ void k_dc_first(const double* __restrict__ wc, const double* __restrict__ wr, const double* phi_tab,
                           const DevState* ds, const float* __restrict__ e, double* __restrict__ uout,
                           const double* __restrict__ f, float* __restrict__ d, int n, double h2i) {
    pgb_pdl_entry();
    const double phirx = phi_tab[ds->tf - ds->t_base];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n * n; k += gridDim.x * blockDim.x) {
        int i = k / n, j = k - i * n;
        auto U = [&](int q) { return (wc[q] + phirx * wr[q]) + (double)e[q]; };
        double c = U(k), v = 0.0;
        if (i > 0 && j > 0 && i < n - 1 && j < n - 1)
            v = f[k] - h2i * (U(k + n) + U(k - n) + U(k + 1) + U(k - 1) - 4.0 * c);
        uout[k] = c;
        d[k] = (float)v;
    }
}
/* the walls' terms of the right-hand side alone (rhs_node at rho = 0) */
__global__ void k_wall_rhs(FinalizeArgs a, double phirx) {
    pgb_pdl_entry();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < a.nx * a.ny; k += gridDim.x * blockDim.x) {
        int j = k / a.nx, i = k - j * a.nx;
        a.f[k] = rhs_node(0.0, i, j, a, phirx);
    }
}
__global__ void k_to32(float* d, const double* s, int count) {
    pgb_pdl_entry();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) d[k] = (float)s[k];
}
__global__ void k_to64(double* d, const float* s, int count) {
    pgb_pdl_entry();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) d[k] = (double)s[k];
}

/* FP64 defect correction around the FP32 sine-transform solve of L u = f64
 * (zero walls), `passes` solves in all; the result goes to out (FP64).
 * lift: the first approximation is the walls' solution wc + phi_right(t) wr
 * plus the FP32 solve of the charge term alone, which keeps the walls'
 * terms (-phi/(DX DY) next to a wall, a thousand times the charge term at
 * 1 V) out of the FP32 transform, whose rounding they would otherwise
 * spread over every mode; each pass then divides the error by about 1e6
 * instead of about 300.  Otherwise the first solve is of f64 itself.  */
static int dst_dc(pgb_run* r, const double* f64, double* out, int passes, bool lift) {
    const int top = r->ng - 1, n = r->nx, G = n * n, gb = blocks_for(G);
    const double h = r->p.xlength / (n - 1), h2i = 1.0 / (h * h);
    float* const f32 = r->mg32_f[top];   /* right-hand side, then each defect */
    float* const e32 = r->mg32_u[top];   /* each FP32 solve                   */
    if (lift) PGB_CK(r, pgb_launch_pdl(k_rho32, dim3(gb), dim3(256), 0, r->stream, f32, (const double*)r->rho, n,
                                       1.0 / 8.854e-12));
    else PGB_CK(r, pgb_launch_pdl(k_to32, dim3(gb), dim3(256), 0, r->stream, f32, f64, G));
    r->launches++;
    if (pgb_dst_solve(r, f32, e32)) return PGB_ERR_CUDA;
    if (passes <= 1 && !lift) {
        PGB_CK(r, pgb_launch_pdl(k_to64, dim3(gb), dim3(256), 0, r->stream, out, (const float*)e32, G));
        r->launches++;
        return 0;
    }
    double* ua = nullptr;   /* FP64 solution so far */
    double* ub = passes <= 1 ? out : r->dc_u;
    if (lift) {
        PGB_CK(r, pgb_launch_pdl(k_dc_first, dim3(gb), dim3(256), 0, r->stream, (const double*)r->dst_wc,
                                 (const double*)r->dst_wr, (const double*)r->phi_tab, (const DevState*)r->ds,
                                 (const float*)e32, ub, f64, f32, n, h2i));
        r->launches++;
        if (passes <= 1) return 0;
        ua = ub;
        ub = r->dc_u2;
        if (pgb_dst_solve(r, f32, e32)) return PGB_ERR_CUDA;
    }
    for (int it = lift ? 2 : 1; it < passes; ++it) {
        PGB_CK(r, pgb_launch_pdl(k_dc_update, dim3(gb), dim3(256), 0, r->stream, (const double*)ua, (const float*)e32,
                                 ub, f64, f32, n, h2i));
        r->launches++;
        ua = ub;
        ub = (ub == r->dc_u) ? r->dc_u2 : r->dc_u;
        if (pgb_dst_solve(r, f32, e32)) return PGB_ERR_CUDA;
    }
    PGB_CK(r, pgb_launch_pdl(k_dc_final, dim3(gb), dim3(256), 0, r->stream, out, (const double*)ua, (const float*)e32, G));
    r->launches++;
    return 0;
}

/* DST_DC's wall solutions: L u = (the walls' right-hand side terms), the
 * left, bottom and top walls at their potentials, then the right wall at
 * 1 V, each to FP64 rounding (eight passes; about 300x each without lift) */
static int dst_wall_solutions(pgb_run* r) {
    const size_t G = (size_t)r->nx * r->ny;
    PGB_CK(r, cudaMalloc(&r->dst_wc, G * sizeof(double)));
    PGB_CK(r, cudaMalloc(&r->dst_wr, G * sizeof(double)));
    PGB_CK(r, cudaDeviceSynchronize());   /* the setup's memsets ran on the legacy stream */
    double* const f64 = r->mg_w[r->ng - 1];   /* FP64 scratch of the top level */
    for (int w = 0; w < 2; ++w) {
        FinalizeArgs a = fin_args(r, 0, true);
        a.f = f64;
        if (w == 1) a.phi0x = a.phi0y = a.phily = 0.0;
        PGB_CK(r, pgb_launch_pdl(k_wall_rhs, dim3(blocks_for((long long)G)), dim3(256), 0, r->stream, a,
                                 w == 1 ? 1.0 : 0.0));
        if (dst_dc(r, f64, w == 0 ? r->dst_wc : r->dst_wr, 8, false)) return PGB_ERR_CUDA;
    }
    PGB_CK(r, cudaMemsetAsync(f64, 0, G * sizeof(double), r->stream));   /* the level's walls stay 0 */
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    return 0;
}

int pgb_mg_setup(pgb_run* r) {
    double* tabs[4 * PGB_MAX_LEVELS] = {};
    float* tabs32[4 * PGB_MAX_LEVELS] = {};
    for (int l = 0; l < r->ng; ++l) {
        size_t n2 = (size_t)r->mg_n[l] * r->mg_n[l];
        PGB_CK(r, cudaMalloc(&r->mg32_u[l], n2 * sizeof(float)));
        PGB_CK(r, cudaMalloc(&r->mg32_f[l], n2 * sizeof(float)));
        PGB_CK(r, cudaMalloc(&r->mg32_v[l], n2 * sizeof(float)));
        PGB_CK(r, cudaMalloc(&r->mg32_r[l], n2 * sizeof(float)));
        PGB_CK(r, cudaMalloc(&r->mg_w[l], n2 * sizeof(double)));
        PGB_CK(r, cudaMalloc(&r->mg32_w[l], n2 * sizeof(float)));
        tabs[l] = r->mg_u[l];
        tabs[PGB_MAX_LEVELS + l] = r->mg_f[l];
        tabs[2 * PGB_MAX_LEVELS + l] = r->mg_v[l];
        tabs[3 * PGB_MAX_LEVELS + l] = r->mg_r[l];
        tabs32[l] = r->mg32_u[l];
        tabs32[PGB_MAX_LEVELS + l] = r->mg32_f[l];
        tabs32[2 * PGB_MAX_LEVELS + l] = r->mg32_v[l];
        tabs32[3 * PGB_MAX_LEVELS + l] = r->mg32_r[l];
    }
    for (int l = 0; l < r->ng; ++l) {
        size_t n2 = (size_t)r->mg_n[l] * r->mg_n[l];
        PGB_CK(r, cudaMemset(r->mg_u[l], 0, n2 * sizeof(double)));
        PGB_CK(r, cudaMemset(r->mg_v[l], 0, n2 * sizeof(double)));
        PGB_CK(r, cudaMemset(r->mg32_u[l], 0, n2 * sizeof(float)));
        PGB_CK(r, cudaMemset(r->mg32_v[l], 0, n2 * sizeof(float)));
        PGB_CK(r, cudaMemset(r->mg_w[l], 0, n2 * sizeof(double)));   /* walls stay 0 */
        PGB_CK(r, cudaMemset(r->mg32_w[l], 0, n2 * sizeof(float)));
    }
    PGB_CK(r, cudaMalloc(&r->mg_tab, sizeof(tabs)));
    PGB_CK(r, cudaMemcpy(r->mg_tab, tabs, sizeof(tabs), cudaMemcpyHostToDevice));
    PGB_CK(r, cudaMalloc(&r->mg32_tab, sizeof(tabs32)));
    PGB_CK(r, cudaMemcpy(r->mg32_tab, tabs32, sizeof(tabs32), cudaMemcpyHostToDevice));
    size_t G = (size_t)r->nx * r->ny;
    PGB_CK(r, cudaMalloc(&r->dc_u, G * sizeof(double)));
    PGB_CK(r, cudaMalloc(&r->dc_u2, G * sizeof(double)));
    PGB_CK(r, cudaFuncSetAttribute(k_mg_small<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)small_smem_bytes(small_top(r, sizeof(double)), sizeof(double))));
    PGB_CK(r, cudaFuncSetAttribute(k_mg_small<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)small_smem_bytes(small_top(r, sizeof(float)), sizeof(float))));
    if (r->p.poisson_mode == PGB_POISSON_DST_DC) {
        if (pgb_dst_setup(r)) return PGB_ERR_CUDA;
        if (pgb_dst_ok(r) && dst_wall_solutions(r)) return PGB_ERR_CUDA;
    }
    return 0;
}

void pgb_mg_free(pgb_run* r) {
    for (int l = 0; l < r->ng; ++l) {
        cudaFree(r->mg32_u[l]); cudaFree(r->mg32_f[l]); cudaFree(r->mg32_v[l]); cudaFree(r->mg32_r[l]);
        cudaFree(r->mg_w[l]); cudaFree(r->mg32_w[l]);
    }
    cudaFree(r->mg32_tab);
    cudaFree(r->dc_u);
    cudaFree(r->dc_u2);
    cudaFree(r->dst_wc);
    cudaFree(r->dst_wr);
    pgb_dst_free(r);
}

/* fields::grid_potential after the right-hand side is in mg_f[ng-1]:
 *   FMG_REF  FP64 full multigrid with the reference's schedule (bitwise)
 *   FMG32    the same schedule in FP32
 *   FP32_DC  FP64 defect correction around FP32 multigrid: the FMG32 pass
 *            on the right-hand side, then dc_max_iters - 1 passes of
 *            (FP64 defect of the FP64 solution, one FP32 V-cycle on it
 *            from zero, FP64 addition of that correction).  The FP32 pass
 *            leaves an error of a few 1e-5 of phi; each V-cycle divides it
 *            by about ten, down to the FP64 discrete solution.
 *   DST_DC   the same FP64 defect correction around the FP32 sine-transform
 *            solve (pgb_dst.cu), which solves the discrete system exactly
 *            up to FP32 rounding (about 1e-6 of phi): a first solve, then
 *            dc_max_iters - 1 corrections, each dividing the error by
 *            about 1e6.                                                  */
int pgb_poisson_solve(pgb_run* r) {
    const int top = r->ng - 1, n = r->nx;
    const int G = n * n;
    const int gb = blocks_for(G);
    if (r->p.poisson_mode == PGB_POISSON_FMG_REF) {
        if (fmg<double>(r, levels64(r))) return PGB_ERR_CUDA;
        PGB_CK(r, cudaMemcpyAsync(r->phi, r->mg_u[top], sizeof(double) * G, cudaMemcpyDeviceToDevice, r->stream));
    } else if (r->p.poisson_mode == PGB_POISSON_DST_DC) {
        if (!pgb_dst_ok(r)) return PGB_ERR_CUDA;
        if (dst_dc(r, r->mg_f[top], r->phi, r->p.dc_max_iters > 1 ? r->p.dc_max_iters : 1, true)) return PGB_ERR_CUDA;
    } else {
        Levels<float> L = levels32(r);
        PGB_CK(r, pgb_launch_pdl(k_to32, dim3(gb), dim3(256), 0, r->stream, L.f[top], r->mg_f[top], G));
        r->launches++;
        if (fmg<float>(r, L)) return PGB_ERR_CUDA;
        const int passes = r->p.poisson_mode == PGB_POISSON_FP32_DC && r->p.dc_max_iters > 1 ? r->p.dc_max_iters : 1;
        if (passes == 1) {
            PGB_CK(r, pgb_launch_pdl(k_to64, dim3(gb), dim3(256), 0, r->stream, r->phi, L.u[top], G));
            r->launches++;
        } else {
            const double h = r->p.xlength / (n - 1), h2i = 1.0 / (h * h);
            const int jsmall = small_top(r, sizeof(float));
            /* a grid solved inside one CTA takes its V-cycle there, on the
             * level's correction and residual arrays (v, r)              */
            const bool one_cta = top <= jsmall;
            float* const dtop = one_cta ? L.rr[top] : L.f[top];
            float* const etop = one_cta ? L.v[top] : L.u[top];
            const float* e = L.u[top];   /* the FMG pass's result        */
            double* ua = nullptr;        /* FP64 solution so far (null: 0) */
            double* ub = r->dc_u;
            for (int it = 1; it < passes; ++it) {
                PGB_CK(r, pgb_launch_pdl(k_dc_update, dim3(gb), dim3(256), 0, r->stream, (const double*)ua, e, ub,
                                         (const double*)r->mg_f[top], dtop, n, h2i));
                r->launches++;
                ua = ub;
                ub = (ub == r->dc_u) ? r->dc_u2 : r->dc_u;
                if (one_cta) {
                    PGB_CK(r, cudaMemsetAsync(etop, 0, sizeof(float) * G, r->stream));
                    if (small_launch<float>(r, L.tab, top, 1)) return PGB_ERR_CUDA;
                } else if (vcycle<float>(r, L, top, jsmall, etop, dtop, 3, nullptr)) {
                    return PGB_ERR_CUDA;
                }
                e = etop;
            }
            PGB_CK(r, pgb_launch_pdl(k_dc_final, dim3(gb), dim3(256), 0, r->stream, r->phi, (const double*)ua, e, G));
            r->launches++;
        }
    }
    PGB_CK(r, pgb_launch_pdl(k_walls, dim3(blocks_for((long long)r->nx * r->ny)), dim3(256), 0, r->stream, r->phi, r->nx, r->ny, r->p.phi_left, r->phi_tab,
                                                                         r->ds, r->p.phi_bottom, r->p.phi_top));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}

int pgb_launch_efield(pgb_run* r, int advance) {
    int GE = (r->nx + 1) * (r->ny + 1);
    PGB_CK(r, pgb_launch_pdl(k_efield, dim3(blocks_for(GE)), dim3(256), 0, r->stream, r->phi, r->ex, r->ey, r->exy, r->nx, r->ny, 2.0 * r->dx, r->ds, advance));
    r->launches++;
    PGB_CK(r, cudaGetLastError());
    return 0;
}


