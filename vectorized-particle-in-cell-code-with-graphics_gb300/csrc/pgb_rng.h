/*
 * Counter-based random numbers for the PIC step (host and device).
 *
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11): a 10-round bijection of a 128-bit counter under a
 * 64-bit key.  Every random draw of the simulation is a pure function of
 *   key     = run seed
 *   counter = {particle id, time step, stream*4 + species, draw block}
 * so results do not depend on thread count, launch shape or particle order.
 * The reference draws from the C library's rand() in loop order
 * (collisions.cpp:74-135, e_collisions.cpp:340-356, boundary.cpp:379-860,
 * particle.cpp:458-501); this replaces that source only.
 *
 * A uniform is formed from the top 23 bits as ((r >> 9) + 0.5) * 2^-23, which
 * lies strictly inside (0, 1) and is exactly representable in float and
 * double, so host (double) and device (float) code see the same value.
 */
#ifndef PGB_RNG_H
#define PGB_RNG_H
#include <stdint.h>

#if defined(__CUDACC__)
#define PGB_HD __host__ __device__ __forceinline__
#else
#define PGB_HD static inline
#endif

#define PGB_PHILOX_M0 0xD2511F53u
#define PGB_PHILOX_M1 0xCD9E8D57u
#define PGB_PHILOX_W0 0x9E3779B9u
#define PGB_PHILOX_W1 0xBB67AE85u

/* random streams: one per kind of decision, so that the draws of different
 * physics never overlap for the same particle and step                    */
enum {
    PGB_STREAM_NEUTRAL_E = 1,   /* e-neutral velocity table entry i           */
    PGB_STREAM_NEUTRAL_I = 2,   /* ion-neutral velocity table entry i         */
    PGB_STREAM_EMCC      = 3,   /* elastic test + scattering                  */
    PGB_STREAM_IONIZE    = 4,   /* ionization energy split and directions     */
    PGB_STREAM_CX        = 5,   /* charge-exchange neutral pick               */
    PGB_STREAM_EWALL     = 6,   /* electron wall: yield tests, reflect, backscatter */
    PGB_STREAM_SEE       = 7,   /* one secondary electron (id of the secondary) */
    PGB_STREAM_IWALL     = 8,   /* ion wall: ion-impact SEE                   */
    PGB_STREAM_PLOP      = 9,   /* steady-state pair re-insertion             */
    PGB_STREAM_INJECT    = 10,  /* injected particle                          */
    PGB_STREAM_REDUCE    = 11   /* Kunhardt reduction priority                */
};

typedef struct pgb_u32x4 { uint32_t v[4]; } pgb_u32x4;

PGB_HD uint32_t pgb_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    return (uint32_t)p;
}

PGB_HD pgb_u32x4 pgb_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                   uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += PGB_PHILOX_W0; k1 += PGB_PHILOX_W1; }
        uint32_t hi0, hi1;
        uint32_t lo0 = pgb_mulhilo32(PGB_PHILOX_M0, c0, &hi0);
        uint32_t lo1 = pgb_mulhilo32(PGB_PHILOX_M1, c2, &hi1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    pgb_u32x4 out;
    out.v[0] = c0; out.v[1] = c1; out.v[2] = c2; out.v[3] = c3;
    return out;
}

/* A sequential reader over one (id, step, stream, species) stream. */
typedef struct pgb_stream {
    uint32_t id, step, sel, block;
    uint32_t k0, k1;
    uint32_t buf[4];
    int pos;
} pgb_stream;

PGB_HD void pgb_stream_init(pgb_stream* s, uint64_t seed, uint32_t id, uint32_t step,
                            uint32_t stream, uint32_t species) {
    s->id = id; s->step = step; s->sel = stream * 4u + species; s->block = 0;
    s->k0 = (uint32_t)seed; s->k1 = (uint32_t)(seed >> 32);
    s->pos = 4;
}

PGB_HD uint32_t pgb_stream_u32(pgb_stream* s) {
    if (s->pos == 4) {
        pgb_u32x4 r = pgb_philox4x32_10(s->id, s->step, s->sel, s->block, s->k0, s->k1);
        s->buf[0] = r.v[0]; s->buf[1] = r.v[1]; s->buf[2] = r.v[2]; s->buf[3] = r.v[3];
        s->block += 1u;
        s->pos = 0;
    }
    return s->buf[s->pos++];
}

/* uniform in (0,1), identical in float and double */
PGB_HD float pgb_u01f(uint32_t r) { return ((float)(r >> 9) + 0.5f) * (1.0f / 8388608.0f); }
PGB_HD double pgb_u01d(uint32_t r) { return ((double)(r >> 9) + 0.5) * (1.0 / 8388608.0); }

#endif /* PGB_RNG_H */
