/*
 * In-process stand-in for the OpenCL 1.2 runtime, used only to build the
 * reference code as a CPU oracle.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference offloads three particle loops to OpenCL (particle.cpp:663-1341
 * host side, pic.cl:22-149 device side) and two diagnostics loops (graphs.cpp,
 * pic.cl:151-251).  This container has no OpenCL driver, so this file
 * implements the handful of API calls the reference makes
 * (pic.cpp:592-885, particle.cpp, graphs.cpp, openCLutility.cpp:11-24) on
 * host memory and runs the reference's own pic.cl kernels, compiled as C++,
 * over the NDRange.
 *
 *  - Buffers are heap blocks; enqueue read/write are memcpy.
 *  - Kernel arguments are stored as raw bytes and unpacked per kernel name.
 *  - collectCharge and the two histogram kernels run serially in work-item
 *    order: their OpenCL versions add to shared cells with plain `+=`
 *    (pic.cl:46-49, 173-183, 221-248), which races on a real device; the
 *    serial order is the semantics the oracle fixes.
 *  - The gather and push kernels write only their own work-item's data, so
 *    they may run on several host threads (ORC_THREADS, default 1).
 */
#include <CL/cl.h>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <omp.h>

struct _cl_platform_id { int dummy; };
struct _cl_device_id { int dummy; };
struct _cl_context { int dummy; };
struct _cl_command_queue { int dummy; };
struct _cl_event { int dummy; };
struct _cl_program { int dummy; };
struct _cl_mem { std::vector<unsigned char> bytes; };
struct _cl_kernel {
    std::string name;
    std::vector<std::vector<unsigned char>> args;
};

namespace clk {
static thread_local size_t g_gid = 0;
static inline size_t get_global_id(int) { return g_gid; }
#define kernel
#define global
#include REF_PIC_CL
#undef kernel
#undef global
}  // namespace clk

static _cl_platform_id g_platform;
static _cl_device_id g_device;
static _cl_context g_context;
static _cl_command_queue g_queue;
static _cl_event g_event;
static _cl_program g_program;

static int orc_threads() {
    const char* s = std::getenv("ORC_THREADS");
    int t = s ? std::atoi(s) : 1;
    return t > 0 ? t : 1;
}

cl_int clGetPlatformIDs(cl_uint, cl_platform_id* platforms, cl_uint* num) {
    if (platforms) platforms[0] = &g_platform;
    if (num) *num = 1;
    return CL_SUCCESS;
}

cl_int clGetDeviceIDs(cl_platform_id, cl_device_type, cl_uint, cl_device_id* devices, cl_uint* num) {
    if (devices) devices[0] = &g_device;
    if (num) *num = 1;
    return CL_SUCCESS;
}

cl_context clCreateContext(const cl_context_properties*, cl_uint, const cl_device_id*,
                           void (*)(const char*, const void*, size_t, void*), void*, cl_int* err) {
    if (err) *err = CL_SUCCESS;
    return &g_context;
}

cl_command_queue clCreateCommandQueue(cl_context, cl_device_id, cl_command_queue_properties, cl_int* err) {
    if (err) *err = CL_SUCCESS;
    return &g_queue;
}

cl_program clCreateProgramWithSource(cl_context, cl_uint, const char**, const size_t*, cl_int* err) {
    if (err) *err = CL_SUCCESS;
    return &g_program;
}

cl_int clBuildProgram(cl_program, cl_uint, const cl_device_id*, const char*, void (*)(cl_program, void*), void*) {
    return CL_SUCCESS;
}

cl_int clGetProgramBuildInfo(cl_program, cl_device_id, cl_program_build_info, size_t, void* value, size_t* ret) {
    if (ret) *ret = 1;
    if (value) static_cast<char*>(value)[0] = 0;
    return CL_SUCCESS;
}

cl_kernel clCreateKernel(cl_program, const char* name, cl_int* err) {
    _cl_kernel* k = new _cl_kernel();
    k->name = name;
    k->args.resize(32);   /* sum_av_dist takes 17 (pic.cl:191-197) */
    if (err) *err = CL_SUCCESS;
    return k;
}

cl_mem clCreateBuffer(cl_context, cl_mem_flags, size_t size, void* host_ptr, cl_int* err) {
    _cl_mem* m = new _cl_mem();
    m->bytes.resize(size ? size : 1);
    if (host_ptr) std::memcpy(m->bytes.data(), host_ptr, size);
    if (err) *err = CL_SUCCESS;
    return m;
}

cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem buf, cl_bool, size_t off, size_t cb, const void* ptr,
                            cl_uint, const cl_event*, cl_event*) {
    if (!buf || off + cb > buf->bytes.size()) return CL_INVALID_VALUE;
    if (cb) std::memcpy(buf->bytes.data() + off, ptr, cb);
    return CL_SUCCESS;
}

cl_int clEnqueueReadBuffer(cl_command_queue, cl_mem buf, cl_bool, size_t off, size_t cb, void* ptr,
                           cl_uint, const cl_event*, cl_event*) {
    if (!buf || off + cb > buf->bytes.size()) return CL_INVALID_VALUE;
    if (cb) std::memcpy(ptr, buf->bytes.data() + off, cb);
    return CL_SUCCESS;
}

cl_int clSetKernelArg(cl_kernel k, cl_uint idx, size_t size, const void* value) {
    if (!k || idx >= k->args.size()) return CL_INVALID_ARG_INDEX;
    k->args[idx].assign(static_cast<const unsigned char*>(value),
                        static_cast<const unsigned char*>(value) + size);
    return CL_SUCCESS;
}


template <class T>
static T arg_val(const _cl_kernel* k, int i) {
    T v;
    std::memcpy(&v, k->args[i].data(), sizeof(T));
    return v;
}

template <class T>
static T* arg_buf(const _cl_kernel* k, int i) {
    cl_mem m = arg_val<cl_mem>(k, i);
    return reinterpret_cast<T*>(m->bytes.data());
}

cl_int clEnqueueNDRangeKernel(cl_command_queue, cl_kernel k, cl_uint, const size_t*, const size_t* gws,
                              const size_t*, cl_uint, const cl_event*, cl_event*) {
    const long n = static_cast<long>(gws[0]);
    if (k->name == "collectCharge") {
        auto* p = arg_buf<clk::particle>(k, 0);
        auto* q = arg_buf<double>(k, 1);
        double qc = arg_val<double>(k, 2), dx = arg_val<double>(k, 3), dy = arg_val<double>(k, 4);
        int nx = arg_val<int>(k, 5), ny = arg_val<int>(k, 6);
        for (long g = 0; g < n; ++g) {
            clk::g_gid = g;
            clk::collectCharge(p, q, qc, dx, dy, nx, ny);
        }
    } else if (k->name == "get_particle_electric_field") {
        auto* p = arg_buf<clk::particle>(k, 0);
        auto* exp_ = arg_buf<double>(k, 1);
        auto* eyp = arg_buf<double>(k, 2);
        auto* ex = arg_buf<double>(k, 3);
        auto* ey = arg_buf<double>(k, 4);
        double dx = arg_val<double>(k, 5), dy = arg_val<double>(k, 6);
        int nx = arg_val<int>(k, 7), ny = arg_val<int>(k, 8);
#pragma omp parallel for num_threads(orc_threads()) schedule(static)
        for (long g = 0; g < n; ++g) {
            clk::g_gid = g;
            clk::get_particle_electric_field(p, exp_, eyp, ex, ey, dx, dy, nx, ny);
        }
    } else if (k->name == "move_particles") {
        auto* p = arg_buf<clk::particle>(k, 0);
        auto* exp_ = arg_buf<double>(k, 1);
        auto* eyp = arg_buf<double>(k, 2);
        double dx = arg_val<double>(k, 3), dy = arg_val<double>(k, 4);
        int nx = arg_val<int>(k, 5), ny = arg_val<int>(k, 6);
        double c = arg_val<double>(k, 7), odt = arg_val<double>(k, 8), ca = arg_val<double>(k, 9);
        double sa = arg_val<double>(k, 10), dt = arg_val<double>(k, 11), co = arg_val<double>(k, 12);
        double so = arg_val<double>(k, 13), b = arg_val<double>(k, 14);
#pragma omp parallel for num_threads(orc_threads()) schedule(static)
        for (long g = 0; g < n; ++g) {
            clk::g_gid = g;
            clk::move_particles(p, exp_, eyp, dx, dy, nx, ny, c, odt, ca, sa, dt, co, so, b);
        }
    } else if (k->name == "sum_av_velocities") {
        auto* p = arg_buf<clk::particle>(k, 0);
        auto* cx = arg_buf<double>(k, 1);
        auto* cy = arg_buf<double>(k, 2);
        auto* vx = arg_buf<double>(k, 3);
        auto* vy = arg_buf<double>(k, 4);
        double dx = arg_val<double>(k, 5), dy = arg_val<double>(k, 6);
        int nx = arg_val<int>(k, 7), ny = arg_val<int>(k, 8);
        for (long g = 0; g < n; ++g) {
            clk::g_gid = g;
            clk::sum_av_velocities(p, cx, cy, vx, vy, dx, dy, nx, ny);
        }
    } else if (k->name == "sum_av_dist") {
        auto* p = arg_buf<clk::particle>(k, 0);
        auto* x1 = arg_buf<double>(k, 1);
        auto* x2 = arg_buf<double>(k, 2);
        auto* y1 = arg_buf<double>(k, 3);
        auto* y2 = arg_buf<double>(k, 4);
        double dx = arg_val<double>(k, 5), dy = arg_val<double>(k, 6);
        int nx = arg_val<int>(k, 7), ny = arg_val<int>(k, 8), nb = arg_val<int>(k, 9);
        double sp = arg_val<double>(k, 10), l1 = arg_val<double>(k, 11), l2 = arg_val<double>(k, 12);
        double l3 = arg_val<double>(k, 13), l4 = arg_val<double>(k, 14), vt = arg_val<double>(k, 15);
        double div = arg_val<double>(k, 16);
        for (long g = 0; g < n; ++g) {
            clk::g_gid = g;
            clk::sum_av_dist(p, x1, x2, y1, y2, dx, dy, nx, ny, nb, sp, l1, l2, l3, l4, vt, div);
        }
    } else {
        return CL_INVALID_KERNEL;
    }
    return CL_SUCCESS;
}

cl_int clFlush(cl_command_queue) { return CL_SUCCESS; }
cl_int clReleaseMemObject(cl_mem m) { delete m; return CL_SUCCESS; }
cl_int clReleaseKernel(cl_kernel k) { delete k; return CL_SUCCESS; }
cl_int clReleaseProgram(cl_program) { return CL_SUCCESS; }
cl_int clReleaseCommandQueue(cl_command_queue) { return CL_SUCCESS; }
cl_int clReleaseContext(cl_context) { return CL_SUCCESS; }
cl_int clEnqueueMarker(cl_command_queue, cl_event* ev) { if (ev) *ev = &g_event; return CL_SUCCESS; }
cl_int clWaitForEvents(cl_uint, const cl_event*) { return CL_SUCCESS; }
