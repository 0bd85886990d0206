/*
 * Averaged diagnostics: the graphs class (graphs.cpp, pic.cl:151-251) with
 * its sums kept on the device.
 *
 * Every step of the window adds, after the field solve (pic.cpp:1189-1207):
 *   - rho, phi, Ex, Ey per node and each species' charge density divided
 *     by its macro charge (graphs::sum_fields, sum_density);
 *   - the mean vx of the particles in each cell of row ny/2 and the mean vy
 *     in each cell of column nx/2 (sum_av_velocities, pic.cl:154-186): the
 *     step's sums are fixed point (2^-10 m/s, int64 atomics) and counts,
 *     so they do not depend on the particle order; k_gr_vfinish turns them
 *     into the step's means;
 *   - the velocity histograms of sum_av_dist (pic.cl:191-251) as exact
 *     integer counts.  The reference gives the kernel `spread` as an 8-byte
 *     double read from its int member and the next one (graphs.cpp:865,
 *     graphs.h:281-282); kernel_spread() rebuilds that double, so the
 *     same cells are counted.
 * The reference's kernels add with plain `+=` from every work item, which
 * loses updates on a real device; the counts here are the serial ones.
 * Reading divides by NO_GRAPH_STEPS (graphs.cpp:1000-1155) on the host.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <string>
#include <vector>
#include "pgb_internal.h"
#include "pgb_physics.cuh"

#define GR_VFIX 1024.0   /* velocity sums: 2^10 per m/s */

/* per node: fields and both densities (graphs.cpp:412-453) */
__global__ void k_gr_fields(int nodes, const double* rho, const double* phi, const double* ex, const double* ey,
                            const double* q0, const double* q1, double qc0, double qc1, double* f0, double* f1,
                            double* f2, double* f3, double* g0, double* g1) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nodes; k += gridDim.x * blockDim.x) {
        f0[k] += rho[k];
        f1[k] += phi[k];
        f2[k] += ex[k];   /* EgridX[j*nx+i]: the stride-nx E layout */
        f3[k] += ey[k];
        g0[k] += q0[k] / qc0;
        g1[k] += q1[k] / qc1;
    }
}

struct GrParticleArgs {
    const float4* xv;
    const DevState* ds;
    int s, nx, ny, ps;
    double vt, dbb, spread;
    int half;
    double l1, l2, l3, l4;           /* DIST_LOCATIONX, 2X, Y, 2Y */
    long long *vsx, *vsy;
    unsigned int *cx, *cy;
    unsigned long long* d[4];        /* X1, Y1, X2, Y2 */
};

/* vbin = (int)((v / vt) * divide_bins_by), counted when |vbin| <= half
 * (pic.cl:218-221); a value outside the int range is not counted        */
__device__ __forceinline__ void gr_bin(unsigned long long* d, float v, const GrParticleArgs& a) {
    double b = ((double)v / a.vt) * a.dbb;
    if (!(b > -2147483649.0 && b < 2147483648.0)) return;
    int vbin = (int)b;
    if (abs(vbin) <= a.half) atomicAdd(&d[vbin + a.half], 1ull);
}

/* jp = (int)(x/DX) (pic.cl:164-165) is the position's cell field */
__global__ void __launch_bounds__(256) k_gr_particles(GrParticleArgs a) {
    const long long n = a.ds->n[a.s];
    const int xv = a.nx / 2, yv = a.ny / 2;   /* sum_av_velocities (pic.cl:161-162) */
    const int xd = a.ny / 2, yd = a.ny / 2;   /* sum_av_dist (pic.cl:202-203)      */
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float4 p = a.xv[i];
        if (is_dead(p.x)) continue;
        const int jp = pcell(p.x, a.ps), kp = pcell(p.y, a.ps);
        const bool xin = pos_gt0(p.x), yin = pos_gt0(p.y);
        if (kp != yv && kp != yd && jp != xv && jp != xd) continue;   /* off both slices */
        /* jp >= 0, kp >= 0: a position beyond the int range converts to
         * INT_MIN, which the reference would use as an index            */
        if (jp >= 0 && jp < a.nx && xin && kp == yv) {
            atomicAdd((unsigned long long*)&a.vsx[jp], (unsigned long long)__double2ll_rn((double)p.z * GR_VFIX));
            atomicAdd(&a.cx[jp], 1u);
        }
        if (jp == xv && kp >= 0 && kp < a.ny && yin) {
            atomicAdd((unsigned long long*)&a.vsy[kp], (unsigned long long)__double2ll_rn((double)p.w * GR_VFIX));
            atomicAdd(&a.cy[kp], 1u);
        }
        const double j = (double)jp, k = (double)kp;
        if (j >= a.l1 - a.spread && xin && j <= a.l1 + a.spread && jp < a.nx && kp == yd) gr_bin(a.d[0], p.z, a);
        if (j >= a.l2 - a.spread && xin && j <= a.l2 + a.spread && jp < a.nx && kp == yd) gr_bin(a.d[2], p.z, a);
        if (k >= a.l3 - a.spread && yin && k <= a.l3 + a.spread && kp < a.ny && jp == xd) gr_bin(a.d[1], p.w, a);
        if (k >= a.l4 - a.spread && yin && k <= a.l4 + a.spread && kp < a.ny && jp == xd) gr_bin(a.d[3], p.w, a);
    }
}

/* v_plot[j] += sum/count where count > 0 (graphs.cpp:679-688); clears the
 * step's sums for the next step                                          */
__global__ void k_gr_vfinish(int m, double* v, long long* vsum, unsigned int* cnt) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
        unsigned int c = cnt[j];
        if (c > 0) v[j] += ((double)vsum[j] / GR_VFIX) / (double)c;
        vsum[j] = 0;
        cnt[j] = 0;
    }
}

/* ============================================================ host side */
/* spread as sum_av_dist sees it: low word spread, high word dist_locationX */
static double kernel_spread(const pgb_graphs_params& g) {
    unsigned long long bits = ((unsigned long long)(unsigned int)g.dist_location_x << 32) | (unsigned int)g.spread;
    double d;
    memcpy(&d, &bits, sizeof d);
    return d;
}

static int gfail(pgb_run* r, int code, const std::string& msg) {
    if (r) r->err = msg;
    return code;
}

int pgb_launch_graphs(pgb_run* r) {
    auto& G = r->gr;
    const int nodes = r->nx * r->ny;
    const int gb = std::min((nodes + 255) / 256, r->sms * 4);
    k_gr_fields<<<gb, 256, 0, r->stream>>>(nodes, r->rho, r->phi, r->ex, r->ey, r->q[0], r->q[1], -PGB_CHARGE,
                                           PGB_CHARGE, G.f[0], G.f[1], G.f[2], G.f[3], G.q[0], G.q[1]);
    r->launches++;
    for (int s = 0; s < 2; ++s) {
        GrParticleArgs a;
        a.xv = r->sp[s].xv; a.ds = r->ds; a.s = s; a.nx = r->nx; a.ny = r->ny; a.ps = r->ps;
        a.vt = s == 0 ? r->p.vte : r->p.vti;   /* set_vt(VTE / VTI) (pic.cpp:543-552) */
        a.dbb = (double)G.g.divide_bins_by;
        a.spread = kernel_spread(G.g);
        a.half = (G.g.no_bins - 1) / 2;
        a.l1 = G.g.dist_location_x; a.l2 = G.g.dist_location2_x;
        a.l3 = G.g.dist_location_y; a.l4 = G.g.dist_location2_y;
        a.vsx = G.vsum[s][0]; a.vsy = G.vsum[s][1]; a.cx = G.vcnt[s][0]; a.cy = G.vcnt[s][1];
        for (int k = 0; k < 4; ++k) a.d[k] = G.d[s][k];
        k_gr_particles<<<r->sms * 8, 256, 0, r->stream>>>(a);
        k_gr_vfinish<<<(r->nx + 255) / 256, 256, 0, r->stream>>>(r->nx, G.v[s][0], G.vsum[s][0], G.vcnt[s][0]);
        k_gr_vfinish<<<(r->ny + 255) / 256, 256, 0, r->stream>>>(r->ny, G.v[s][1], G.vsum[s][1], G.vcnt[s][1]);
        r->launches += 3;
    }
    PGB_CK(r, cudaGetLastError());
    return 0;
}

extern "C" int pgb_graphs_params_default(const pgb_params* p, pgb_graphs_params* out) {
    if (!p || !out) return PGB_ERR_ARG;
    memset(out, 0, sizeof(*out));
    const int nx = p->x_no_of_cells, ny = p->y_no_of_cells;
    out->no_graph_steps = 1;
    out->no_bins = 30001;                                       /* parameters.h:288 */
    out->divide_bins_by = (out->no_bins - 1) / 100;             /* parameters.h:289 */
    out->spread = (int)(0.05 * (float)nx);                      /* parameters.h:302 */
    out->dist_location_x = (int)(0.9 * (float)nx);              /* parameters.h:293-298 */
    out->dist_location_y = (int)(0.5 * (float)ny);
    out->dist_location2_x = (int)(0.1 * (float)nx);
    out->dist_location2_y = (int)(0.5 * (float)ny);
    return 0;
}

extern "C" int pgb_graphs_enable(pgb_run* r, const pgb_graphs_params* g) {
    if (!r || !g) return gfail(r, PGB_ERR_ARG, "pgb_graphs_enable: bad argument");
    if (g->no_bins < 1 || (g->no_bins & 1) == 0 || g->no_graph_steps < 1 || g->divide_bins_by == 0)
        return gfail(r, PGB_ERR_ARG, "pgb_graphs_enable: no_bins must be odd and positive, no_graph_steps and "
                                     "divide_bins_by nonzero");
    /* queued steps may still add to an earlier window's buffer */
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    auto& G = r->gr;
    if (G.buf) { cudaFree(G.buf); G.buf = nullptr; G.on = false; }
    const size_t nodes = (size_t)r->nx * r->ny, nx = r->nx, ny = r->ny, nb = (size_t)g->no_bins;
    auto up = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const size_t sizes[] = {up(6 * nodes * 8), up(2 * (nx + ny) * 8), up(2 * (nx + ny) * 8), up(2 * (nx + ny) * 4),
                            up(8 * nb * 8)};
    size_t total = 0;
    for (size_t s : sizes) total += s;
    if (cudaMalloc(&G.buf, total) != cudaSuccess) {
        cudaGetLastError();
        G.buf = nullptr;
        return gfail(r, PGB_ERR_NOMEM, "pgb_graphs_enable: device allocation failed");
    }
    char* c = (char*)G.buf;
    double* f = (double*)c;
    for (int k = 0; k < 4; ++k) G.f[k] = f + k * nodes;
    G.q[0] = f + 4 * nodes; G.q[1] = f + 5 * nodes;
    c += sizes[0];
    double* v = (double*)c;
    long long* vs = (long long*)(c + sizes[1]);
    unsigned int* vc = (unsigned int*)(c + sizes[1] + sizes[2]);
    for (int s = 0; s < 2; ++s) {
        const size_t o = s * (nx + ny);
        G.v[s][0] = v + o; G.v[s][1] = v + o + nx;
        G.vsum[s][0] = vs + o; G.vsum[s][1] = vs + o + nx;
        G.vcnt[s][0] = vc + o; G.vcnt[s][1] = vc + o + nx;
    }
    c += sizes[1] + sizes[2] + sizes[3];
    unsigned long long* d = (unsigned long long*)c;
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 4; ++k) G.d[s][k] = d + (s * 4 + k) * nb;
    PGB_CK(r, cudaMemsetAsync(G.buf, 0, total, r->stream));
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    G.g = *g;
    G.on = true;
    return 0;
}

/* device sums -> host (waits for the run's queued steps) */
template <class T>
static int fetch(pgb_run* r, const T* src, size_t n, std::vector<T>& out) {
    out.resize(n);
    PGB_CK(r, cudaMemcpyAsync(out.data(), src, n * sizeof(T), cudaMemcpyDeviceToHost, r->stream));
    PGB_CK(r, cudaStreamSynchronize(r->stream));
    return 0;
}

/* the averaged graph `which` (graphs::average_*, graphs.cpp:1000-1155) */
static int graph_values(pgb_run* r, int which, int s, std::vector<double>& out) {
    auto& G = r->gr;
    const size_t nodes = (size_t)r->nx * r->ny;
    const double steps = (double)G.g.no_graph_steps;
    std::vector<unsigned long long> h;
    int rc = 0;
    switch (which) {
        case PGB_GRAPH_RHO: case PGB_GRAPH_PHI: case PGB_GRAPH_EX: case PGB_GRAPH_EY:
            rc = fetch(r, G.f[which], nodes, out);
            for (double& x : out) x /= steps;
            return rc;
        case PGB_GRAPH_DENSITY:
            rc = fetch(r, G.q[s], nodes, out);
            for (double& x : out) x /= steps;
            return rc;
        case PGB_GRAPH_VX: case PGB_GRAPH_VY:
            /* both species are scaled by VTE (graphs.cpp:1114-1121) */
            rc = fetch(r, G.v[s][which - PGB_GRAPH_VX], which == PGB_GRAPH_VX ? (size_t)r->nx : (size_t)r->ny, out);
            for (double& x : out) x = x / (r->p.vte * steps);
            return rc;
        case PGB_GRAPH_DIST_X1: case PGB_GRAPH_DIST_Y1: case PGB_GRAPH_DIST_X2: case PGB_GRAPH_DIST_Y2:
            if ((rc = fetch(r, (const unsigned long long*)G.d[s][which - PGB_GRAPH_DIST_X1], (size_t)G.g.no_bins, h)))
                return rc;
            out.resize(h.size());
            for (size_t k = 0; k < h.size(); ++k) out[k] = (double)h[k] / steps;
            return 0;
        default:
            return gfail(r, PGB_ERR_ARG, "pgb_graphs_get: unknown graph");
    }
}

/* running maximum from element `first` (graphs.cpp:1002-1028, 1093-1104) */
static double running_max(const std::vector<double>& a, size_t first) {
    double m = a[first];
    for (double v : a)
        if (m < v) m = v;
    return m;
}

extern "C" int pgb_graphs_get(pgb_run* r, int which, int species, double* out, int64_t n) {
    if (!r || !out || species < 0 || species > 1) return gfail(r, PGB_ERR_ARG, "pgb_graphs_get: bad argument");
    if (!r->gr.on) return gfail(r, PGB_ERR_STATE, "pgb_graphs_get: graphs are not enabled");
    std::vector<double> v;
    int rc;
    if (which == PGB_GRAPH_MAXIMA) {
        if (n < 5) return gfail(r, PGB_ERR_ARG, "pgb_graphs_get: buffer too small");
        const int src[5][2] = {{PGB_GRAPH_PHI, 0}, {PGB_GRAPH_EX, 0}, {PGB_GRAPH_EY, 0}, {PGB_GRAPH_DENSITY, 0},
                               {PGB_GRAPH_DENSITY, 1}};
        for (int k = 0; k < 5; ++k) {
            if ((rc = graph_values(r, src[k][0], src[k][1], v))) return rc;
            out[k] = running_max(v, k < 3 ? 0 : (size_t)r->nx + 1);   /* qMax starts at q_plot[1][1] */
        }
        return 0;
    }
    if ((rc = graph_values(r, which, species, v))) return rc;
    if (n < (int64_t)v.size()) return gfail(r, PGB_ERR_ARG, "pgb_graphs_get: buffer too small");
    memcpy(out, v.data(), v.size() * sizeof(double));
    return 0;
}

/* ------------------------------------------------ the reference's files */
static FILE* open_in(pgb_run* r, const std::string& dir, const std::string& name) {
    std::string path = dir.empty() ? name : dir + "/" + name;
    FILE* f = fopen(path.c_str(), "w");
    if (!f) r->err = "pgb_graphs_write: cannot write " + path;
    return f;
}

/* a [ny][nx] grid as rows of "%e " (graphs.cpp:1189-1299) */
static int write_grid(pgb_run* r, const std::string& dir, const char* name, const std::vector<double>& a) {
    FILE* f = open_in(r, dir, name);
    if (!f) return PGB_ERR_IO;
    for (int j = 0; j < r->ny; ++j) {
        for (int i = 0; i < r->nx; ++i) fprintf(f, "%e ", a[(size_t)j * r->nx + i]);
        fprintf(f, "\n");
    }
    fclose(f);
    return 0;
}

extern "C" int pgb_graphs_write(pgb_run* r, const char* dir_c) {
    if (!r || !dir_c) return gfail(r, PGB_ERR_ARG, "pgb_graphs_write: bad argument");
    if (!r->gr.on) return gfail(r, PGB_ERR_STATE, "pgb_graphs_write: graphs are not enabled");
    const std::string dir = dir_c;
    const int nx = r->nx;
    std::vector<double> f[4];
    int rc;
    for (int k = 0; k < 4; ++k)
        if ((rc = graph_values(r, k, 0, f[k]))) return rc;
    /* slices at y = ny/2 and x = nx/2 (graphs.cpp:1167-1187) */
    const int yp = r->ny / 2, xp = nx / 2;
    FILE* fx = open_in(r, dir, "rho_phi_EgridX.txt");
    if (!fx) return PGB_ERR_IO;
    FILE* fy = open_in(r, dir, "rho_phi_EgridY.txt");
    if (!fy) { fclose(fx); return PGB_ERR_IO; }
    for (int i = 0; i < nx; ++i) {
        const size_t kx = (size_t)yp * nx + i, ky = (size_t)i * nx + xp;
        fprintf(fx, "%e %e %e %e\n", (double)i, f[0][kx], f[1][kx], f[2][kx]);
        fprintf(fy, "%e %e %e %e\n", (double)i, f[0][ky], f[1][ky], f[3][ky]);
    }
    fclose(fx);
    fclose(fy);
    const char* grids[4] = {"rho2d.txt", "phi2d.txt", "egrid2dX.txt", "egrid2dY.txt"};
    for (int k = 0; k < 4; ++k)
        if ((rc = write_grid(r, dir, grids[k], f[k]))) return rc;
    const char* type[2] = {"e", "i1"};   /* ELECTRON_TYPE, ION_TYPE */
    const int half = (r->gr.g.no_bins - 1) / 2;
    const double dbb = (double)r->gr.g.divide_bins_by;
    for (int s = 0; s < 2; ++s) {
        std::vector<double> q, vx, vy;
        if ((rc = graph_values(r, PGB_GRAPH_DENSITY, s, q)) || (rc = graph_values(r, PGB_GRAPH_VX, s, vx)) ||
            (rc = graph_values(r, PGB_GRAPH_VY, s, vy)))
            return rc;
        if ((rc = write_grid(r, dir, ("density2d_" + std::string(type[s]) + ".txt").c_str(), q))) return rc;
        /* graphs.cpp:1303-1318: one row per x cell */
        FILE* fv = open_in(r, dir, "av_velocity_" + std::string(type[s]) + ".txt");
        if (!fv) return PGB_ERR_IO;
        for (int j = 0; j < nx; ++j) fprintf(fv, "%e %e %e \n", (double)j, vx[j], j < r->ny ? vy[j] : 0.0);
        fclose(fv);
        /* graphs.cpp:1320-1370 */
        const char* stems[2][2] = {{"first_v_distX_", "first_v_distY_"}, {"second_v_distX_", "second_v_distY_"}};
        const int which[2][2] = {{PGB_GRAPH_DIST_X1, PGB_GRAPH_DIST_Y1}, {PGB_GRAPH_DIST_X2, PGB_GRAPH_DIST_Y2}};
        for (int loc = 0; loc < 2; ++loc)
            for (int axis = 0; axis < 2; ++axis) {
                std::vector<double> d;
                if ((rc = graph_values(r, which[loc][axis], s, d))) return rc;
                FILE* fd = open_in(r, dir, std::string(stems[loc][axis]) + type[s] + ".txt");
                if (!fd) return PGB_ERR_IO;
                for (int j = 0; j < r->gr.g.no_bins; ++j) fprintf(fd, "%e %e \n", (double)(j - half) / dbb, d[j]);
                fclose(fd);
            }
    }
    return 0;
}
