/*
 * pgb_deposit_static: the charge deposit of one species without a run handle
 * and without allocating device memory.
 *
 * Callers that can't allocate:
 *   - a diagnostic or viewer hook that runs between steps on the
 *     simulation's own stream, with the particles already on the device.
 *     cudaMalloc and cudaFree synchronise the whole device, which would drain
 *     the step queue the caller keeps full;
 *   - a host that has reserved the device memory for particle capacity.
 *     There, a temporary grid-sized allocation can fail in the middle of a
 *     run.
 *
 * Output: the same grid as pgb_deposit + pgb_get_grid(PGB_GRID_Q_E/Q_I) for
 * the same particle records.  That is particle::collect_charge:
 *   - CIC weights (pic.cl:22-52);
 *   - the charge density qc/(DX*DY);
 *   - edge rows and columns doubled, corners doubled again
 *     (particle.cpp:663-858).
 * The per-node sums are int64 fixed point (2^19 per unit weight), so the
 * grid does not depend on the order of the records.
 *
 * Scratch: one int64 accumulator per node.  It lives in the file-scope
 * array g_static_acc below, of PGB_STATIC_DEPOSIT_MAX_NODES entries
 * (513 x 513 nodes, 2.1 MB), so no call allocates.  The rules that follow:
 *   - Every call shares the array and leaves its own sums in it.  Each call
 *     clears the nodes it uses before depositing.
 *   - Two calls whose kernels overlap on the GPU race on the array, for
 *     example calls on two streams without an event between them.  Calls on
 *     one stream are ordered and safe.
 *   - The first call on a device, with that device current, finds the
 *     array's address with cudaGetSymbolAddress and caches it.  This loads
 *     the module on that device if it is not loaded yet.  Make that first
 *     call before any stream capture begins.
 *   - The cached address belongs to the device's primary context.  After
 *     cudaDeviceReset on a device the module may load elsewhere, so the
 *     entry point must not be called on that device again in this process.
 */
#include <cuda_runtime.h>
#include <mutex>
#include <string>
#include "pgb_internal.h"
#include "pgb_physics.cuh"

#define PGB_STATIC_MAX_DEVICES 64

/* the shared accumulator: [ny][nx] int64 fixed point, nx*ny <= maximum */
static __device__ __align__(256) unsigned long long g_static_acc[PGB_STATIC_DEPOSIT_MAX_NODES];

namespace {

struct DeviceSetup {
    unsigned long long* acc = nullptr;   /* device address of g_static_acc */
    int sms = 0;
};

std::mutex g_setup_mu;
DeviceSetup g_setup[PGB_STATIC_MAX_DEVICES];

__global__ void k_static_clear(unsigned long long* acc, int nodes) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nodes; k += gridDim.x * blockDim.x) acc[k] = 0ull;
}

/* Each record is a particleVec {x, y, vx, vy, vz, w} (particleVec.h:26-35).
 * x and y become fixed-point positions exactly as pgb_load_species makes
 * them (pgb_pos_shift of the grid), so the deposit is bit-identical to the
 * run handle's.                                                          */
__global__ void __launch_bounds__(256) k_static_deposit(const double* aos6, long long n, int nx, int ny, double dx,
                                                        double dy, int ps, unsigned long long* acc) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double* r = aos6 + 6 * i;
        float xl = pos_from_m(r[0], dx, ps), yl = pos_from_m(r[1], dy, ps), w = (float)r[5];
        if (deposit_ok(xl, yl, nx, ny, ps)) deposit_cell(acc, nx, ps, xl, yl, w);
    }
}

/* q = (sum / PGB_FIX_SCALE * qc/(DX*DY)) * edge factor, the sum being in
 * units of 2^-19 of a unit weight (particle.cpp:829-845)                 */
__global__ void k_static_finish(const unsigned long long* acc, int nx, int ny, double qcdxdy, double* q) {
    const int nodes = nx * ny;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nodes; k += gridDim.x * blockDim.x) {
        int j = k / nx, i = k - j * nx;
        bool ex = (i == 0 || i == nx - 1), ey = (j == 0 || j == ny - 1);
        double ef = (ex ? 2.0 : 1.0) * (ey ? 2.0 : 1.0) * ((ex && ey) ? 2.0 : 1.0);
        double v = __dmul_rn((double)(long long)acc[k], 1.0 / PGB_FIX_SCALE);
        q[k] = __dmul_rn(__dmul_rn(v, qcdxdy), ef);
    }
}

int setup_error(const std::string& msg, cudaError_t e) {
    pgb_set_unbound_error(msg + ": " + cudaGetErrorString(e));
    return PGB_ERR_CUDA;
}

/* per-device set-up, once per device, with that device current */
int device_setup(DeviceSetup* out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return setup_error("pgb_deposit_static: cudaGetDevice", e);
    if (dev < 0 || dev >= PGB_STATIC_MAX_DEVICES) {
        pgb_set_unbound_error("pgb_deposit_static: device ordinal " + std::to_string(dev) + " is beyond " +
                              std::to_string(PGB_STATIC_MAX_DEVICES));
        return PGB_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& s = g_setup[dev];
    if (!s.acc) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_acc);
        if (e != cudaSuccess) return setup_error("pgb_deposit_static: cudaGetSymbolAddress", e);
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return setup_error("pgb_deposit_static: cudaDeviceGetAttribute", e);
        s.sms = sms > 0 ? sms : 1;
        s.acc = (unsigned long long*)p;
    }
    *out = s;
    return 0;
}

}  // namespace

extern "C" int pgb_deposit_static(const double* d_aos6, int64_t n, int32_t nx, int32_t ny, double dx, double dy,
                                  double qc, double* d_q, void* stream) {
    if (n < 0 || (n > 0 && !d_aos6) || !d_q || nx < 2 || ny < 2 || !(dx > 0.0) || !(dy > 0.0)) {
        pgb_set_unbound_error("pgb_deposit_static: bad argument");
        return PGB_ERR_ARG;
    }
    if ((int64_t)nx * ny > PGB_STATIC_DEPOSIT_MAX_NODES) {
        pgb_set_unbound_error("pgb_deposit_static: grid of " + std::to_string(nx) + " x " + std::to_string(ny) +
                              " nodes exceeds the static scratch maximum of " +
                              std::to_string(PGB_STATIC_DEPOSIT_MAX_NODES) + " nodes (513 x 513)");
        return PGB_ERR_CAPACITY;
    }
    DeviceSetup s;
    int rc = device_setup(&s);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int nodes = nx * ny;
    const int gblocks = (nodes + 255) / 256 < s.sms * 4 ? (nodes + 255) / 256 : s.sms * 4;
    k_static_clear<<<gblocks, 256, 0, st>>>(s.acc, nodes);
    if (n > 0) {
        long long want = (n + 255) / 256;
        int pblocks = want < (long long)s.sms * 8 ? (int)want : s.sms * 8;
        k_static_deposit<<<pblocks, 256, 0, st>>>(d_aos6, (long long)n, nx, ny, dx, dy, pgb_pos_shift(nx, ny), s.acc);
    }
    k_static_finish<<<gblocks, 256, 0, st>>>(s.acc, nx, ny, qc / (dx * dy), d_q);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return setup_error("pgb_deposit_static: kernel launch", e);
    return 0;
}
