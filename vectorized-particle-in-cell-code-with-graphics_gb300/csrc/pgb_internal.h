/*
 * Internal definitions shared by the libpicgb translation units.
 *
 * Device layout of one species (structure of arrays, slot order):
 *   xv  float4 {xs, ys, vx, vy}   xs, ys: x/DX, y/DY as signed 32-bit fixed
 *                                 point with ps fraction bits (the bit
 *                                 patterns sit in the float lanes; see the
 *                                 position helpers in pgb_physics.cuh);
 *                                 vx, vy in m/s
 *   vz  float                     m/s
 *   w   float                     macro-particle weight
 *   id  uint32                    stable identity: keys the random streams
 * A removed particle keeps its slot with the tombstone code in xs until the
 * next compaction, which keeps the surviving slots in order.  The cell index
 * (int)(x/DX) and the CIC weight x/DX - (int)(x/DX) are bit fields of the
 * fixed-point position; the reference computes the same quantities from
 * x/DX in FP64 (pic.cl:31-37).
 *
 * Counters that change on the device (slot counts, next id, statistics) live
 * in one DevState block so that a step never waits for the host.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "picgb.h"

#define PGB_TILE 1024          /* particles per tile of the push kernels   */
#define PGB_PUSH_THREADS 256
#define PGB_ITEMS (PGB_TILE / PGB_PUSH_THREADS)
#define PGB_FIX_SCALE 524288.0      /* deposit fixed point: 2^19 per unit weight */
#define PGB_FIX_SCALE_F 524288.0f
#define PGB_MG_SMALL 65        /* levels with n <= 65 are solved by one CTA  */
#define PGB_CX_TILE 2048       /* ions per charge-exchange tile sum            */
#define PGB_MG_SMALL64 33      /* the same for the FP64 multigrid            */
#define PGB_MAX_LEVELS 16
#define PGB_BIN 32             /* bin edge in cells (spatial sort)            */
#define PGB_HALO 8             /* deposit window halo around a bin, cells     */
#define PGB_WIN (PGB_BIN + 2 * PGB_HALO + 1)   /* window edge in nodes         */
#define PGB_PIECE_TILES 4      /* tiles of one bin per work piece             */
#define PGB_SORT_CHUNK 2048    /* slots per chunk of the bin sort passes      */
#define PGB_COPY_CHUNK (1 << 20)   /* particles per host-copy chunk of load/dump */
#define PGB_COPY_EVENTS 32

enum { ST_ABS_E = 0, ST_ABS_I, ST_PLOP, ST_REFL, ST_BACK, ST_SEE_EV, ST_SEE_EM, ST_ISEE_EM,
       ST_ELASTIC, ST_IONIZE, ST_CX, ST_INJ_E, ST_INJ_I, ST_RED_E, ST_RED_I, ST_COUNT };

enum { ERR_CAP_E = 1, ERR_CAP_I = 2, ERR_LIST = 4, ERR_RETRY = 8 };

/* device-resident run state (one allocation) */
struct DevState {
    long long n[2];          /* slots in use per species                     */
    long long dead[2];       /* tombstones among them                        */
    long long n_mcc;         /* electron slots present before this step's injection */
    unsigned int next_id[2];
    unsigned int pad0;
    long long list_n[4];     /* sizes of the dense event lists               */
    long long stats[ST_COUNT];
    int err;
    int pad1;
    long long t;             /* the reference's time_step of the particle phases being run */
    long long sorted_tiles[2];  /* tiles covered by bin pieces (0 = unsorted)   */
    int n_pieces[2];
    long long t_base;        /* step of phi_tab[0]                              */
    int sort_overflow;       /* the padded bin layout did not fit: the sort copies in place order */
    int pad2;
    long long tf;            /* time_step of the field solve being run (its right-wall
                                potential); trails t while a solve overlaps the next
                                step's collisions                                      */
    unsigned long long scat_n;   /* scattering events queued by the collision pass */
    long long n_cx;          /* ion slots whose charge exchange was tested before this
                                step's appends (the rest are tested after them)       */
};

/* dense event lists (ordered by slot) */
enum { LIST_OUT_E = 0, LIST_OUT_I = 1, LIST_ION_EV = 2, LIST_SPARE = 3 };

struct Species {
    float4* xv = nullptr;
    float* vz = nullptr;
    float* w = nullptr;
    unsigned int* id = nullptr;
    /* compaction targets */
    float4* xv2 = nullptr;
    float* vz2 = nullptr;
    float* w2 = nullptr;
    unsigned int* id2 = nullptr;
    long long cap = 0;
    double qc = 0, q_over_m = 0, mass = 0, vt = 0, dt = 0;
};

/* fraction bits of a fixed-point position for a grid of nx x ny nodes:
 * 2^-ps of a cell (20 bits at 513 nodes, at most 23 so that the fraction
 * is exact in FP32), with room for two grid lengths on either side of the
 * origin before a position saturates at +-2^30                            */
inline int pgb_pos_shift(int nx, int ny) {
    int cells = (nx > ny ? nx : ny) - 1, b = 0;
    while ((1 << b) < cells) ++b;
    int ps = 29 - b;
    return ps > 23 ? 23 : (ps < 8 ? 8 : ps);
}

struct PushConsts {
    int nx, ny;
    int ps;                /* fraction bits of the fixed-point positions    */
    float dtdx, dtdy;      /* dt/DX*2^ps, dt/DY*2^ps: position units per (m/s) */
    float coef;            /* 0.5*dt*q/m                                     */
    float ca, sa, co, so;  /* cos/sin of ANGLE and of omega*dt               */
    int bfield;            /* MAGNETIC_FIELD > 0                             */
    int steady;            /* STEADYSTATE wall classification               */
};

struct pgb_run {
    pgb_params p;
    std::string err;
    int dev = 0, sms = 0;
    cudaStream_t stream = nullptr;
    int nx = 0, ny = 0, dt_dti = 1;
    int ps = 20;                  /* pgb_pos_shift(nx, ny) */
    double dx = 0, dy = 0;
    int64_t time_step = 0;
    Species sp[2];
    DevState* ds = nullptr;       /* device */
    DevState* hs = nullptr;       /* pinned host mirror */
    /* grids */
    unsigned long long* qacc[2] = {nullptr, nullptr};   /* fixed-point deposit */
    double* q[2] = {nullptr, nullptr};
    double *rho = nullptr, *phi = nullptr, *rhs = nullptr;
    double *ex = nullptr, *ey = nullptr;
    float2* exy = nullptr;        /* FP32 {Ex,Ey} per node, stride nx, (nx+1)(ny+1) */
    /* multigrid */
    int ng = 0;
    int mg_n[PGB_MAX_LEVELS];
    double *mg_u[PGB_MAX_LEVELS], *mg_f[PGB_MAX_LEVELS], *mg_v[PGB_MAX_LEVELS], *mg_r[PGB_MAX_LEVELS];
    double** mg_tab = nullptr;                       /* device table of the level pointers */
    float** mg32_tab = nullptr;
    double *dc_u = nullptr, *dc_u2 = nullptr;       /* FP32_DC: FP64 solution, two buffers */
    /* DST_DC: sine-transform scratch ((N-1) rows of N floats), twiddles, s_k */
    float* dst_t = nullptr;
    float2* dst_tw = nullptr;
    float* dst_s = nullptr;
    /* DST_DC: FP64 solutions for the walls (zero charge): the left, bottom
     * and top walls at their potentials, and the right wall at 1 V       */
    double* dst_wc = nullptr;
    double* dst_wr = nullptr;
    float *mg32_u[PGB_MAX_LEVELS], *mg32_f[PGB_MAX_LEVELS], *mg32_v[PGB_MAX_LEVELS], *mg32_r[PGB_MAX_LEVELS];
    /* the pre-smoothing result of each level (the tiled smoother reads one
     * buffer and writes another: blocks never see a neighbour's update)  */
    double* mg_w[PGB_MAX_LEVELS] = {};
    float* mg32_w[PGB_MAX_LEVELS] = {};
    /* event lists: per tile 32 ballot words (slot order) and a count, then
     * the dense list in slot order                                       */
    int* tile_list[4] = {nullptr, nullptr, nullptr, nullptr};
    int* tile_cnt[4] = {nullptr, nullptr, nullptr, nullptr};
    int* list[4] = {nullptr, nullptr, nullptr, nullptr};
    long long list_cap = 0;   /* = max particle capacity                       */
    long long ntiles_cap = 0;
    int* aux_i = nullptr;     /* scratch ints (wall passes), list_cap entries  */
    int* inject_flag = nullptr;   /* NUMBER_TO_INJECT flags                     */
    int* aux_j = nullptr;
    /* collisions */
    float* neut[2] = {nullptr, nullptr};   /* [which]: 3 x N_neutral, FP32    */
    float vn_max[2] = {0.0f, 0.0f};        /* largest neutral speed per table */
    double* neut64[2] = {nullptr, nullptr};
    double* prob_cx = nullptr;             /* per-column CX accumulator       */
    double* phi_tab = nullptr;             /* right-wall potential per step   */
    double* phi_host = nullptr;            /* pinned: the table and the step number on their way */
    long long* t_host = nullptr;
    cudaEvent_t phi_ev;                    /* recorded after their upload     */
    bool phi_ev_ok = false;
    long long phi_tab_cap = 0;
    /* CUDA graphs of one step, keyed by (ion step, buffer orientation e, i) */
    cudaGraphExec_t graph[8] = {};
    int orient[2] = {0, 0};                /* which particle buffer is live   */
    long long graph_launches[8] = {};      /* kernels in each graph           */
    int use_graphs = 1;
    /* pipelined steps: graph A (collisions) and B (the other particle
     * phases) per key as above, graph F (field solve); F of step t runs on
     * the side stream while A of step t+1 runs on the run's stream        */
    cudaGraphExec_t graph_a[8] = {}, graph_b[8] = {}, graph_f = nullptr;
    long long graph_a_launches[8] = {}, graph_b_launches[8] = {}, graph_f_launches = 0;
    /* the captured templates of A, B and F, and per key one step graph
     * built from them: F of the previous step beside A, then B -- one
     * launch for a step that needs no host decision                      */
    cudaGraph_t tmpl_a[8] = {}, tmpl_b[8] = {}, tmpl_f = nullptr;
    cudaGraphExec_t graph_m[8] = {};
    int prio_hi = 0;                       /* the side stream's priority      */
    /* launch shapes (pgb_set_launch_config, pgb_autotune): they change no
     * result.  push grid = SMs x tune_push_per_sm; the collision kernels
     * beside a field solve leave it tune_field_sms SMs                   */
    int tune_push_per_sm = 8;
    int tune_field_sms = 32;
    bool fields_pending = false;           /* last step's field solve not yet issued */
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork, ev_join;
    bool side_ok = false;
    float* cx_p = nullptr;                 /* per-ion CX probability          */
    float* cx_tile_sum = nullptr;          /* [column][tile] (int64)          */
    long long cx_tiles_cap = 0;
    /* [column][tile / 64] bits of the tiles with a non-zero sum, and the
     * per-column totals; zero between passes (the walk clears them)     */
    unsigned long long* cx_mask = nullptr;
    long long* cx_total = nullptr;
    int cx_mask_words = 0;
    /* spatial sort */
    int* tile_bin[2] = {nullptr, nullptr};
    int4* pieces[2] = {nullptr, nullptr};
    int* sort_counts = nullptr;
    int* sort_offs = nullptr;
    int* sort_key_total = nullptr;
    long long* sort_key_start = nullptr;
    long long sort_chunks_cap = 0;
    /* population control (Kunhardt): group counts and digit histograms */
    void* kh = nullptr;
    /* averaged diagnostics (graphs class): sums on the device, one buffer */
    struct Graphs {
        bool on = false;
        pgb_graphs_params g{};
        double* f[4] = {};                /* rho, phi, Ex, Ey sums [ny][nx]          */
        double* q[2] = {};                /* density sums per species [ny][nx]       */
        double* v[2][2] = {};             /* per-cell mean vx [nx] / vy [ny] sums    */
        long long* vsum[2][2] = {};       /* this step's velocity sums, 2^10 per m/s */
        unsigned int* vcnt[2][2] = {};    /* this step's particle counts             */
        unsigned long long* d[2][4] = {}; /* histogram counts X1, Y1, X2, Y2         */
        void* buf = nullptr;
    } gr;
    /* headless viewer plots: the image and a 16-byte scratch (pgb_render) */
    void* rd_img = nullptr;
    long long rd_cap = 0;
    void* rd_scratch = nullptr;
    /* host staging */
    double* h_stage = nullptr;
    size_t h_stage_bytes = 0;
    double* d_stage = nullptr;     /* device staging for load/dump (AoS doubles) */
    size_t d_stage_bytes = 0;
    cudaStream_t copy_stream = nullptr;   /* host copies of load/dump, overlapped with their kernels */
    cudaEvent_t copy_ev[PGB_COPY_EVENTS];
    bool copy_ev_ok = false;
    /* instrumentation */
    long long launches = 0;        /* kernel launches issued                     */
    /* host-side fault injection for tests: PGB_FAULT_ALLOC=k at pgb_create
     * makes the handle's k-th particle-storage growth fail (PGB_ERR_NOMEM) */
    int fault_alloc = 0, alloc_events = 0;
    int prof_on = 0;
    pgb_profile prof;
    cudaEvent_t prof_ev[13];
    bool prof_ev_ok = false;
};

/* ------------------------------------------------------------ helpers */
bool pgb_cuda_ok(pgb_run* r, cudaError_t e, const char* what);
/* message for pgb_last_error(NULL), from entry points without a handle */
void pgb_set_unbound_error(const std::string& msg);
/* Programmatic dependent launch.  A kernel launched with pgb_launch_pdl may
 * be launched while the previous kernel on its stream finishes: as that
 * kernel's blocks exit, the next one's are scheduled.  Its first statement
 * is pgb_pdl_entry(), whose griddepcontrol.wait blocks until the previous
 * kernel has completed and its writes are visible.  No memory is touched
 * before it, so results are those of plain launches; what it saves is the
 * launch gap.  No kernel triggers its dependents early: blocks parked at
 * the wait would hold SM slots that other runs' streams need when many
 * runs share the GPU (pgb_step_batch), which cost those a third of their
 * throughput.  On a kernel launched without the attribute the wait does
 * nothing.                                                                */
#ifdef __CUDACC__
__device__ __forceinline__ void pgb_pdl_entry() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
template <typename... KArgs, typename... Args>
inline cudaError_t pgb_launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                  Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}
#endif

#define PGB_CK(r, call)                                  \
    do {                                                 \
        if (!pgb_cuda_ok((r), (call), #call)) return PGB_ERR_CUDA; \
    } while (0)

/* kernels launched from the host side (defined in the .cu files) */
struct CollConsts;
int pgb_launch_push(pgb_run* r, int s, bool deposit);
int pgb_launch_flag_outside(pgb_run* r, int s);
/* count_only: the list's length alone (ds->list_n), not the list */
int pgb_build_list(pgb_run* r, int which, int species_for_tiles, bool count_only = false);
int pgb_launch_deposit(pgb_run* r, int s);
int pgb_launch_finalize(pgb_run* r, int which_species_mask, bool make_rhs);
int pgb_launch_inject(pgb_run* r, int species_mask, bool push_e);
int pgb_launch_ionize_appends(pgb_run* r, int store_e, int store_i);
int pgb_launch_mcc(pgb_run* r, int leave_sms);
int pgb_launch_scatter(pgb_run* r, int leave_sms);
/* tail 0: the ions present (records their count); 1: those appended since;
 * 2: the same in one block, for a tail of a few thousand ions at most     */
int pgb_launch_cx(pgb_run* r, int tail, int leave_sms);
int pgb_launch_walls(pgb_run* r, int which);
int pgb_launch_load(pgb_run* r, int s, const double* d_aos, long long i0, long long i1);
int pgb_launch_dump_offsets(pgb_run* r, int s);
int pgb_launch_dump(pgb_run* r, int s, double* d_out, unsigned int* d_ids, long long cap, int t0, int t1);
int pgb_mg_setup(pgb_run* r);
void pgb_mg_free(pgb_run* r);
/* FP32 sine-transform Poisson solver (pgb_dst.cu) */
int pgb_dst_setup(pgb_run* r);
void pgb_dst_free(pgb_run* r);
bool pgb_dst_ok(const pgb_run* r);
int pgb_dst_solve(pgb_run* r, const float* f, float* u);
CollConsts pgb_coll_consts(pgb_run* r);
int pgb_launch_compact(pgb_run* r, int s);
int pgb_launch_sort(pgb_run* r, int s);
int pgb_sort_setup(pgb_run* r);
void pgb_bins(pgb_run* r, int* nbx, int* nby);
int pgb_launch_reduce(pgb_run* r, int s);
int pgb_launch_step_advance(pgb_run* r);
int pgb_launch_graphs(pgb_run* r);
int pgb_poisson_solve(pgb_run* r);
int pgb_launch_efield(pgb_run* r, int advance);
int pgb_launch_rhs(pgb_run* r);
int pgb_launch_cross_sections(int which, const double* d_e, long long n, double* d_out, cudaStream_t st);
