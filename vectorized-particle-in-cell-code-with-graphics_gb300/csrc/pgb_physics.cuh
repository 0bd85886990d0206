/*
 * Device physics shared by the particle, collision and wall kernels.
 *
 * Per-particle tests that run for every particle every step (in-domain
 * checks, energies, cross sections, collision probabilities) are FP32.
 * The events they select (scattering, ionization, charge exchange, wall
 * interactions, re-insertion) touch a small fraction of the particles and
 * are evaluated in FP64 with the reference's formulas and operation order.
 */
#pragma once
#include <math.h>
#include <stdint.h>
#include "pgb_internal.h"
#include "pgb_rng.h"

#define PGB_PI 3.141592654
#define PGB_CHARGE 1.602177e-19
#define PGB_AMU 1.66054e-27

/* (int)v with the x86-64 result for NaN and out-of-range values (INT_MIN),
 * which the reference relies on to treat NaN particles as outside the left
 * wall (boundary.cpp:595-599)                                              */
__device__ __forceinline__ int cellf(float v) {
    return (v >= -2147483648.0f && v < 2147483648.0f) ? __float2int_rz(v) : INT32_MIN;
}
__device__ __forceinline__ int celld(double v) {
    return (v > -2147483649.0 && v < 2147483648.0) ? (int)v : INT32_MIN;
}

/* ------------------------------------------------------------ positions
 * A particle position is a signed 32-bit fixed-point number of cells with
 * ps fraction bits (2^-ps of a cell: ps = 20 at 513 nodes, see
 * pgb_pos_shift), kept as a bit pattern in the x and y lanes of xv; no
 * floating-point operation ever touches those lanes.  The push adds the
 * rounded displacement exactly, so a position keeps 2^-ps of a cell
 * wherever it is (an FP32 cell coordinate keeps 2^-15 of a cell at 256-512
 * cells).  The cell index (int)(x/DX) and the CIC fraction are bit fields.
 * Two codes below the range: a removed particle (a tombstone) and a NaN
 * position (ionization products, a push with a NaN velocity), which keeps
 * the reference's x86 meaning: not pushed, not deposited, outside the
 * absorbing walls (its cell index is INT_MIN), never re-inserted by the
 * steady walls.  Positions saturate at +-2^30, far outside any grid.      */
#define PGB_POS_DEAD INT32_MIN
#define PGB_POS_NAN (INT32_MIN + 1)
#define PGB_POS_LIM (1 << 30)
__device__ __forceinline__ int pbits(float lane) { return __float_as_int(lane); }
__device__ __forceinline__ float plane(int x) { return __int_as_float(x); }
__device__ __forceinline__ float pos_dead() { return __int_as_float(PGB_POS_DEAD); }
__device__ __forceinline__ bool is_dead(float lane) { return __float_as_int(lane) == PGB_POS_DEAD; }
__device__ __forceinline__ bool pos_is_nan(float lane) { return __float_as_int(lane) == PGB_POS_NAN; }
/* (int)(x/DX): truncation toward zero (a negative x first gains 2^ps - 1,
 * then the arithmetic shift rounds down); INT_MIN for NaN (x86-64)       */
__device__ __forceinline__ int pcell(float lane, int ps) {
    const int x = __float_as_int(lane);
    const int c = (x + ((x >> 31) & ((1 << ps) - 1))) >> ps;
    return x <= PGB_POS_NAN ? INT32_MIN : c;
}
/* x > 0 and (int)(x/DX) < n, in one unsigned compare: 0 < x < n*2^ps
 * (false for the tombstone and NaN codes)                                */
__device__ __forceinline__ bool pos_open_in(float lane, int n, int ps) {
    /* in unsigned arithmetic: x - 1 wraps for the codes at INT_MIN */
    return (unsigned)__float_as_int(lane) - 1u < (unsigned)((n << ps) - 1);
}
/* 0 <= (int)(x/DX) < n (truncation toward zero): -2^ps < x < n*2^ps; false
 * for the tombstone and NaN codes, whose cell index is INT_MIN           */
__device__ __forceinline__ bool pos_trunc_in(float lane, int n, int ps) {
    return (unsigned)__float_as_int(lane) + (unsigned)((1 << ps) - 1) < (unsigned)((n << ps) + (1 << ps) - 1);
}
/* x > 0 and x < 0 (NaN is neither)                                        */
__device__ __forceinline__ bool pos_gt0(float lane) { return __float_as_int(lane) > 0; }
__device__ __forceinline__ bool pos_lt0(float lane) {
    const int x = __float_as_int(lane);
    return x < 0 && x != PGB_POS_NAN;
}
/* x/DX - (int)(x/DX) for x >= 0, exact: the ps fraction bits placed in the
 * mantissa of 1.0 (ps <= 23), minus 1                                     */
__device__ __forceinline__ float pfrac(float lane, int ps) {
    const unsigned m = ((unsigned)__float_as_int(lane) & ((1u << ps) - 1u)) << (23 - ps);
    return __int_as_float(0x3f800000 | (int)m) - 1.0f;
}
/* the position in cells (exact in FP64) and in metres                    */
__device__ __forceinline__ double pos_cells(float lane, int ps) {
    const int x = __float_as_int(lane);
    return x == PGB_POS_NAN ? __longlong_as_double(0x7ff8000000000000ll) : ldexp((double)x, -ps);
}
__device__ __forceinline__ double pos_m(float lane, int ps, double d) { return pos_cells(lane, ps) * d; }
/* FP32 cells, for plots and histograms                                   */
__device__ __forceinline__ float pos_cellsf(float lane, int ps) {
    const int x = __float_as_int(lane);
    return x == PGB_POS_NAN ? __int_as_float(0x7fffffff) : (float)x * __int_as_float((127 - ps) << 23);
}
/* a position from cells (c = x/DX), rounded to 2^-ps, saturated          */
__device__ __forceinline__ float pos_from_cells(double c, int ps) {
    if (c != c) return __int_as_float(PGB_POS_NAN);
    double v = ldexp(c, ps);
    v = fmin(fmax(v, -(double)PGB_POS_LIM), (double)PGB_POS_LIM);
    return __int_as_float(__double2int_rn(v));
}
__device__ __forceinline__ float pos_from_m(double x, double d, int ps) { return pos_from_cells(x / d, ps); }
/* x + d with d in units of 2^-ps of a cell (the push: d = dt*v/DX*2^ps),
 * in 32-bit integers: |x| <= 2^30 and |d| < 2^30 cannot overflow           */
__device__ __forceinline__ float pos_step(float lane, float d) {
    const float lim = 1073741760.0f;   /* the largest float below 2^30 */
    const int v = __float_as_int(lane) + __float2int_rn(fminf(fmaxf(d, -lim), lim));
    const int c = min(max(v, -PGB_POS_LIM), PGB_POS_LIM);
    return d != d ? __int_as_float(PGB_POS_NAN) : __int_as_float(c);
}

/* CIC deposit of one particle (pic.cl:36-49) as int64 fixed point:
 * round(a*w*2^19) per node (1e-6 of a unit weight, below the FP32
 * rounding of a); integer sums are exact and order-free, so the grid is
 * identical run to run.  Caller checks deposit_ok().                     */
__device__ __forceinline__ void deposit_cell(unsigned long long* qacc, int nx, int ps, float xl, float yl, float w) {
    int jp = pcell(xl, ps), kp = pcell(yl, ps);
    float wj = pfrac(xl, ps), wk = pfrac(yl, ps);
    float a4 = (1.0f - wj) * (1.0f - wk), a3 = wj * (1.0f - wk);
    float a2 = wk * (1.0f - wj), a1 = wj * wk;
    const float S = PGB_FIX_SCALE_F;
    long long c4 = __float2ll_rn(a4 * w * S), c3 = __float2ll_rn(a3 * w * S);
    long long c2 = __float2ll_rn(a2 * w * S), c1 = __float2ll_rn(a1 * w * S);
    unsigned long long* q = qacc + (long long)kp * nx + jp;
    atomicAdd(q, (unsigned long long)c4);
    atomicAdd(q + 1, (unsigned long long)c3);
    atomicAdd(q + nx, (unsigned long long)c2);
    atomicAdd(q + nx + 1, (unsigned long long)c1);
}

/* collect_charge's test: jp < nx-1 && x > 0 && kp < ny-1 && y > 0 (pic.cl:35) */
__device__ __forceinline__ bool deposit_ok(float xl, float yl, int nx, int ny, int ps) {
    return pos_open_in(xl, nx - 1, ps) && pos_open_in(yl, ny - 1, ps);
}

__device__ __forceinline__ void maybe_deposit(unsigned long long* qacc, int nx, int ny, int ps, float xl, float yl,
                                              float w) {
    if (deposit_ok(xl, yl, nx, ny, ps)) deposit_cell(qacc, nx, ps, xl, yl, w);
}

/* ---------------------------------------------------------- wall classes */
/* e_boundary / ion_boundary: outside iff jp<0 || jp>=nx || kp<0 || kp>=ny
 * (boundary.cpp:595-599, 774-778)                                         */
__device__ __forceinline__ bool outside_absorbing(float xl, float yl, int nx, int ny, int ps) {
    return !(pos_trunc_in(xl, nx, ps) && pos_trunc_in(yl, ny, ps));
}
/* steady walls: x < 0 or (int)(x/DX) >= nx, same for y (boundary.cpp:906-1013);
 * as unsigned, a negative x is above n*2^ps; NaN is neither               */
__device__ __forceinline__ bool outside_steady(float xl, float yl, int nx, int ny, int ps) {
    const int x = __float_as_int(xl), y = __float_as_int(yl);
    return (x != PGB_POS_NAN && (unsigned)x >= (unsigned)(nx << ps)) ||
           (y != PGB_POS_NAN && (unsigned)y >= (unsigned)(ny << ps));
}

/* ------------------------------------------------------- cross sections */
/* FP32 forms of e_collisions.cpp:205-308 and ion_collisions.cpp:170-199;
 * values the reference leaves uninitialised on branch edges are 0        */
__device__ __forceinline__ float p6(float e, float a6, float a5, float a4, float a3, float a2, float a1, float a0) {
    return ((((((a6 * e + a5) * e + a4) * e + a3) * e + a2) * e + a1) * e + a0);
}
__device__ __forceinline__ float sig_ar_el(float e) {
    if (e < 0.35f) return p6(e, 28019.0f, -32798.0f, 15048.0f, -34312.0f, 4084.0f, -249.0f, 7.576f);
    if (e < 15.0f && e > 0.35f) return ((-0.013f * e + 0.232f) * e + 1.066f) * e + 0.085f;
    if (e > 15.0f) return 126.2f * __powf(e, -0.69f);
    return 0.0f;
}
__device__ __forceinline__ float sig_ar_ion(float e) {
    if (e < 15.755f) return 0.0f;
    if (e < 100.0f && e > 15.755f) return (((-3.0e-7f * e + 8.0e-5f) * e - 0.008f) * e + 0.416f) * e - 4.758f;
    if (e > 100.0f) return 130.0f * __powf(e, -0.74f);
    return 0.0f;
}
__device__ __forceinline__ float sig_h_el(float e) {
    if (e < 1.0e-2f) return (3.834f * e - 20.82f) * e + 40.98f;
    if (e >= 1.0e-2f && e < 20.0f) return -6.15f * logf(e) + 20.91f;
    if (e >= 20.0f) return 102.2f * __powf(e, -1.19f);
    return 0.0f;
}
__device__ __forceinline__ float sig_h_ion(float e) {
    const float I = 13.6f;
    if (!(e >= I)) return 0.0f;
    float IE = e / I, C = 1.0f - 1.0f / IE;
    float poly = ((((2.2986f * C - 2.8115f) * C + 1.4003f) * C - 0.034539f) * C - 0.032226f) * C;
    return (1.0f / (I * e)) * (0.18450f * logf(IE) + poly);
}
__device__ __forceinline__ float sig_ar_cx(float e) {
    if (e > 4.0f) return (2.0f + 5.5f / sqrtf(e)) * 10.0f;
    return (-2.95f * sqrtf(e) + 10.65f) * 10.0f;
}
/* ion_collisions.cpp:185-199: the energy is divided by 1000 and by AMU, so
 * the scaled energy is ~1e22 and the fit's denominator overflows float to
 * +inf for any physical energy; the FP64 value (~1e-72) gives the same zero
 * probability once it enters 1-exp(-x) and the fixed-point accumulator.   */
__device__ __forceinline__ float sig_h_cx(float e) {
    /* from ee = 1e10 on, ee^5.4 overflows FP32: den is +inf and the result
     * is exactly 0, so the powers and the logarithm are skipped.  A product
     * within 1e-6 of ee decides the common case without the two divisions */
    if (e * (1.0f / (1000.0f * 1.66054e-27f)) >= 2.0e10f) return 0.0f;
    float ee = e / 1000.0f / 1.66054e-27f;
    if (!(ee >= 1.0e-4f)) return 0.0f;
    if (ee >= 1.0e10f) return 0.0f;
    float den = 1.0f + 0.038371f * ee + 3.8068e-6f * __powf(ee, 3.5f) + 1.1832e-10f * __powf(ee, 5.4f);
    return (3.2345f * logf((235.88f / ee) + 2.3713f)) / den;
}

struct CollConsts {
    int species;              /* PGB_ARGON / PGB_HYDROGEN */
    int el_const, ion_const, cx_const;
    float el_value, ion_value, cx_value;
    float e_energy_coef;      /* (0.5/CHARGE)*ME  */
    float i_energy_coef;      /* (0.5/CHARGE)*MI  */
    float e_pcoef;            /* DT*1e-20*NEUTRAL_DENSITY  */
    float i_pcoef;            /* DTI*1e-20*NEUTRAL_DENSITY */
    double me, mi, dt, dti, threshold, reduced_mass;
    /* electron speed below which e_collisions::ionization certainly gives
     * a negative excess energy, hence NaN velocities (see mcc_ionize)  */
    float ion_vcap;
    /* an upper bound of sigma_el over every energy: 50.5 for the H fit
     * (largest 49.23 at 0.01 eV), 25.5 for the Ar fit (largest 24.81 near
     * 13.9 eV; its low-energy polynomial goes negative), the value itself
     * for a constant cross-section                                        */
    float el_max;
    /* (e_pcoef * el_max * 1.000001 * (1 + 1e-5))^2, rounded up: the
     * collision kernel's square-root-free form of that bound            */
    float el_bound2;
    /* the lowest energy (eV) at which sigma_ion can be non-zero: 13.6 and
     * 15.755 below which the H and Ar fits return 0; for a constant
     * cross-section -inf if it is positive (any speed ionizes), else +inf */
    float ion_emin;
    int n_neutral;
    uint64_t seed;
};

__device__ __forceinline__ float sigma_el(const CollConsts& c, float e) {
    if (c.el_const) return c.el_value;
    return c.species == PGB_ARGON ? sig_ar_el(e) : sig_h_el(e);
}
__device__ __forceinline__ float sigma_ion(const CollConsts& c, float e) {
    if (c.ion_const) return c.ion_value;
    return c.species == PGB_ARGON ? sig_ar_ion(e) : sig_h_ion(e);
}
__device__ __forceinline__ float sigma_cx(const CollConsts& c, float e) {
    if (c.cx_const) return c.cx_value;
    return c.species == PGB_ARGON ? sig_ar_cx(e) : sig_h_cx(e);
}

/* ------------------------------------------------ electron collisions */
/* collisions::scattered_velocity (collisions.cpp:107-171) in FP32.  The
 * scattering angle cosChi = 2(1-(1+E)^R)/E + 1 (cosChi = sqrt(1-R) below
 * 0.01 eV) enters as t = 1 - cosChi and s = 1 + cosChi, sinChi = sqrt(t s):
 *   t = 2 expm1(R log1p(E)) / E,    s = -2 (1+E) expm1(-(1-R) log1p(E)) / E
 *   (below 0.01 eV: t = R / (1 + sqrt(1-R)),  s = 1 + sqrt(1-R)),
 * the same values without the cancellations FP32 would suffer in
 * 1-(1+E)^R, 1-sqrt(1-R) and 1-cosChi^2 near forward (R -> 0) and backward
 * (R -> 1) scattering; 1-R is exact in FP32 for these draws.  The scattered
 * velocity then keeps 2e-6 of the speed.  Events are rare (a few per cent
 * of the particles per step), and FP64 here would run at 1/64 rate on a
 * divergent warp.                                                         */
__device__ __forceinline__ void scatter_f32(pgb_stream* st, const float* neut, int nn, float energy, float cf,
                                            float& vx, float& vy, float& vz) {
    const float two_pi = (float)(2.0 * PGB_PI);
    float R = pgb_u01f(pgb_stream_u32(st));
    float t, s;   /* 1 - cosChi, 1 + cosChi */
    if (energy < 1.0e-2f) {
        const float c = sqrtf(1.0f - R);
        t = R / (1.0f + c);
        s = 1.0f + c;
    } else {
        const float l = log1pf(energy);
        t = 2.0f * expm1f(R * l) / energy;
        s = -2.0f * (1.0f + energy) * expm1f(-(1.0f - R) * l) / energy;
    }
    float sinChi = sqrtf(fmaxf(t * s, 0.0f));
    float sinPhi, cosPhi;
    sincosf(two_pi * R, &sinPhi, &cosPhi);
    int index = (int)(pgb_stream_u32(st) % (uint32_t)(nn - 1));
    float nvx = neut[index], nvy = neut[nn + index], nvz = neut[2 * nn + index];
    float ux = vx - nvx, uy = vy - nvy, uz = vz - nvz;
    float uperp = sqrtf(uy * uy + uz * uz);
    float u = sqrtf(ux * ux + uperp * uperp);
    float uyp, uzp;
    if (uperp < 1.0f) { uyp = 1.0f; uzp = 1.0f; }
    else { uyp = uy / uperp; uzp = uz / uperp; }
    vz -= cf * (uz * t - (ux * uzp * cosPhi - u * uyp * sinPhi) * sinChi);
    vy -= cf * (uy * t - (ux * uyp * cosPhi + u * uzp * sinPhi) * sinChi);
    vx -= cf * (ux * t + uperp * cosPhi * sinChi);
}

/* e_collisions::ionization (e_collisions.cpp:319-443).  The excess energy
 * mixes J and eV (line 377) and is negative, so every output is NaN as in
 * the reference.  Returns the parent's new velocity and the new electron
 * and ion states (positions in metres).                                   */
struct IonizeOut {
    float evx, evy, evz;              /* parent electron after               */
    double nx_, ny_;                  /* new electron position               */
    float nvx, nvy, nvz;
    double ix, iy;                    /* new ion position                    */
    float ivx, ivy, ivz;
};
__device__ inline IonizeOut ionize_f32(pgb_stream* st, const float* neut, int nn, const CollConsts& c,
                                       double xe, double ye, float vxe, float vye, float vze) {
    const float me = (float)c.me, mi = (float)c.mi;
    float reduced_mass = (float)(c.reduced_mass * c.me);
    float R = pgb_u01f(pgb_stream_u32(st));
    float Rxe = 1.0f - 2.0f * pgb_u01f(pgb_stream_u32(st));
    float Rye = 1.0f - 2.0f * pgb_u01f(pgb_stream_u32(st));
    float Rze = 1.0f - 2.0f * pgb_u01f(pgb_stream_u32(st));
    float R2xe = 1.0f - 2.0f * pgb_u01f(pgb_stream_u32(st));
    float R2ye = 1.0f - 2.0f * pgb_u01f(pgb_stream_u32(st));
    float R2ze = 1.0f - 2.0f * pgb_u01f(pgb_stream_u32(st));
    int index = (int)(pgb_stream_u32(st) % (uint32_t)(nn - 1));
    float nvx = neut[index], nvy = neut[nn + index], nvz = neut[2 * nn + index];
    float mr = me / (mi + me), nr = mi / (mi + me);
    float Wx = nr * nvx + mr * vxe, Wy = nr * nvy + mr * vye, Wz = nr * nvz + mr * vze;
    float ve = sqrtf(vxe * vxe + vye * vye + vze * vze);
    float vn = sqrtf(nvx * nvx + nvy * nvy + nvz * nvz);
    float excess = (reduced_mass / 2.0f) * (ve - vn) * (ve - vn) - (float)c.threshold;
    float ve_after = sqrtf(2.0f * R * excess / me);
    float v2e_after = sqrtf(2.0f * (1.0f - R) * excess / me);
    float a0 = ve_after * Rxe, a1 = ve_after * Rye, a2 = ve_after * Rze;
    float b0 = v2e_after * R2xe, b1 = v2e_after * R2ye, b2 = v2e_after * R2ze;
    IonizeOut o;
    o.ivx = Wx - (me / mi) * (a0 + b0);
    o.ivy = Wy - (me / mi) * (a1 + b1);
    o.ivz = Wz - (me / mi) * (a2 + b2);
    o.ix = xe + (double)o.ivx * c.dti;
    o.iy = ye + (double)o.ivy * c.dti;
    o.evx = a0 + Wx; o.evy = a1 + Wy; o.evz = a2 + Wz;
    o.nvx = b0 + Wx; o.nvy = b1 + Wy; o.nvz = b2 + Wz;
    o.nx_ = xe + (double)o.nvx * c.dt;
    o.ny_ = ye + (double)o.nvy * c.dt;
    return o;
}

/* particle::get_particle_velocity (particle.cpp:452-464) in FP32 */
__device__ inline float maxwell_f32(pgb_stream* st, float vt) {
    float v = 0.0f;
    for (int k = 0; k < 64; ++k) {
        float R1 = pgb_u01f(pgb_stream_u32(st));
        float R2 = pgb_u01f(pgb_stream_u32(st));
        v = vt * cosf((float)(2.0 * PGB_PI) * R2) * sqrtf(fabsf(logf(R1)));
        if (!(fabsf(v) > vt * 10000.0f)) break;
    }
    return v;
}

/* particle::get_particle_velocity / boundary::get_particle_velocity
 * (particle.cpp:452-464, boundary.cpp:833-845), FP64                     */
__device__ inline double maxwell_fp64(pgb_stream* st, double vt) {
    double v = 0.0;
    for (int k = 0; k < 64; ++k) {
        double R1 = pgb_u01d(pgb_stream_u32(st));
        double R2 = pgb_u01d(pgb_stream_u32(st));
        v = vt * cos(2.0 * PGB_PI * R2) * sqrt(fabs(log(R1)));
        if (!(fabs(v) > vt * 10000)) break;
    }
    return v;
}
