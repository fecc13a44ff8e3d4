/*
 * pbd_oracle.c -- CPU restatement of the reference PBD step.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the oracle, never the product: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference arm load it.  The shipped library never links it.
 *
 * It restates niklasandersson/PBD-Simulation-Framework-CUDA's Fluid::compute()
 * (src/app/simulation/Fluid.cu:14-97) kernel by kernel, in the reference's order and with
 * the reference's explicit neighbour list (N x maxNeighboursPerParticle).  One source is
 * built twice:
 *   ORC_REAL=float  -- FP32 transliteration of the reference kernels (the "reference CPU
 *                      build": also the timed CPU baseline, OpenMP over particles);
 *   ORC_REAL=double -- FP64 oracle with the same semantics.
 * Build with -ffp-contract=off: the only fused multiply-adds are the explicit FMA() calls
 * below, placed where nvcc contracts the reference's expressions in applyForces and in the
 * neighbour-cell offsets (a*b+c forms), so that the FP32 build reproduces the reference's
 * predicted positions and Morton keys bit for bit.
 *
 * Semantics where the reference races (documented, switchable nowhere -- the GPU library
 * implements the same definition):
 *  - solveCollisions (kernel/Collision.h:171-242) adds with float atomics while other
 *    threads read: here every contact reads the positions as they were when the kernel
 *    started (Jacobi snapshot) and the adds of particle i are applied in list order.
 *  - computeViscosity (kernel/Density.h:280-310) writes velocities in place: here it reads a
 *    snapshot (Jacobi).
 *  - computeCellInfo (kernel/SortReorder.h:160-188): the write cellEndings[N-1] = N is
 *    applied after the boundary writes (the order of a sequential run of the kernel).
 *  - findContacts/findNeighbours disabled: the list part is empty (the reference would
 *    reuse a list whose indices refer to an earlier order).
 * The restatement is pinned to the reference's own kernel code run on the CPU
 * (oracle/refexec, fixtures in tests/golden): bit-exact front of a frame and neighbour lists,
 * FP tolerance after whole frames.
 * The sort is a stable LSD counting sort over all 32 key bits: CUB's
 * DeviceRadixSort::SortPairs (kernel/SortReorder.h:39-47) is a stable LSD radix sort, so
 * any stable sort by the uint32 key gives the same permutation.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/pbd.h"

#ifndef ORC_REAL
#define ORC_REAL double
#endif
typedef ORC_REAL real;
#define ORC_IS_F32 (sizeof(real) == 4)

/* The reference defines M_PI as a double literal (kernel/Globals.h:122). */
#define REF_PI 3.14159265359

static inline real SQRT(real a) { return ORC_IS_F32 ? (real)sqrtf((float)a) : (real)sqrt((double)a); }
static inline real FMA(real a, real b, real c) {
    return ORC_IS_F32 ? (real)fmaf((float)a, (float)b, (float)c) : (real)fma((double)a, (double)b, (double)c);
}
static inline real FMIN(real a, real b) { return ORC_IS_F32 ? (real)fminf((float)a, (float)b) : (real)fmin(a, b); }
static inline real FMAX(real a, real b) { return ORC_IS_F32 ? (real)fmaxf((float)a, (float)b) : (real)fmax(a, b); }

typedef struct { real x, y, z, w; } r4;

static inline r4 mk4(real x, real y, real z, real w) { r4 r = {x, y, z, w}; return r; }
static inline r4 add4(r4 a, r4 b) { return mk4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
static inline r4 sub4(r4 a, r4 b) { return mk4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
static inline r4 scl4(real s, r4 a) { return mk4(s * a.x, s * a.y, s * a.z, s * a.w); }
static inline real dot4(r4 a, r4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline real dot3(r4 a, r4 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline real len3(r4 a) { return SQRT(dot3(a, a)); }

/* Integer power by repeated multiplication: the reference's pow(float, int) calls
 * (kernel/Density.h:36-37,138). */
static inline real powi_r(real x, int n) {
    int m = n < 0 ? -n : n;
    real r = (real)1;
    for (int k = 0; k < m; ++k) r *= x;
    return n < 0 ? (real)1 / r : r;
}

typedef struct orc_sim {
    pbd_params prm;
    uint32_t cap, N;
    uint32_t M;                 /* list cap */
    uint32_t G;                 /* max grid */
    r4 *x, *p, *v, *col, *fext, *delta, *omega;
    r4 *xc, *pc, *vc, *colc;    /* copies for the gather re-order */
    real *lambda;
    real *w, *wc;               /* inverse masses (unified solids; 1 = the reference) */
    int mass_used;
    uint32_t *ids, *idsc;
    uint32_t *keys_in, *keys_out, *vals_in, *vals_out, *tmpk, *tmpv;
    uint32_t *cell_start, *cell_end;
    uint32_t *nbr, *nbr_count, *contact_count;
    uint8_t* csolved;           /* collisionType 1: constraint solved in this stabilization pass (N x M) */
    uint64_t* cbest;            /* collisionType 1: each particle's chosen constraint (priority << 32 | c) */
    /* derived parameters (kernel/Initialize.h:42-69) */
    real diameter, h_spiky, h_poly, q_scorr;
} orc_sim;

/* ---------------------------------------------------------------- Hash.h:10-34 ----- */
uint32_t orc_expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

/* mortonCode: clamp each coordinate to [0, 1023], truncate, interleave x<<2 | y<<1 | z. */
static inline uint32_t morton_r(real x, real y, real z) {
    x = FMIN(FMAX(x, (real)0), (real)1023);
    y = FMIN(FMAX(y, (real)0), (real)1023);
    z = FMIN(FMAX(z, (real)0), (real)1023);
    return (orc_expand_bits((uint32_t)x) << 2) + (orc_expand_bits((uint32_t)y) << 1) +
           orc_expand_bits((uint32_t)z);
}
uint32_t orc_morton_f32(float x, float y, float z) {
    x = fminf(fmaxf(x, 0.f), 1023.f); y = fminf(fmaxf(y, 0.f), 1023.f); z = fminf(fmaxf(z, 0.f), 1023.f);
    return (orc_expand_bits((uint32_t)x) << 2) + (orc_expand_bits((uint32_t)y) << 1) + orc_expand_bits((uint32_t)z);
}

/* --------------------------------------------------- Density.h:14-42 kernel shapes -- */
/* poly6Viscosity: 315 (h^2-d^2)^6 / (0.001 + 64 pi h^9) for 0.001 < d < h - 0.001.
 * In the reference the denominator is double (64.0f * M_PI) and so is the division. */
static inline real poly6(const orc_sim* s, real distance) {
    const real h = s->h_poly;
    if (distance > (real)0.001f && distance < h - (real)0.001f) {
        real t = h * h - distance * distance;
        real t3 = t * t * t;
        if (ORC_IS_F32) {
            float h9 = (float)powi_r(h, 9);
            double den = (double)0.001f + 64.0 * REF_PI * (double)h9;
            return (real)((double)((float)(315.0f * (float)t3 * (float)t3)) / den);
        }
        return (real)(315.0 * t3 * t3 / (0.001 + 64.0 * REF_PI * pow(h, 9)));
    }
    return (real)0;
}

/* spiky: 15 (h-d)^2/(pi h^6) * normalize(r), r = pi - pj (float4; normalize over all
 * four lanes, distance over xyz), for d > 1e-4 and h - d > 1e-4. */
static inline r4 spiky(const orc_sim* s, r4 pi, r4 pj) {
    const real h = s->h_spiky;
    r4 r = sub4(pi, pj);
    real distance = len3(r);
    if (distance > (real)0.0001f && (h - distance) > (real)0.0001f) {
        real num = powi_r(h - distance, 2);
        real den = ORC_IS_F32 ? (real)(float)(REF_PI * (double)(float)powi_r(h, 6)) : (real)(REF_PI * pow(h, 6));
        real inv = (real)1 / SQRT(dot4(r, r));
        return scl4((real)15 * (num / den), scl4(inv, r));
    }
    return mk4(0, 0, 0, 0);
}

/* ------------------------------------------------------------ derived parameters -- */
static void derive(orc_sim* s) {
    const pbd_params* P = &s->prm;
    s->diameter = (real)2 * (real)P->particle_radius;                         /* Initialize.h:43 */
    s->h_spiky = ORC_IS_F32 ? (real)(2.0f * P->particle_radius * P->kernel_width_spiky)
                            : s->diameter * (real)P->kernel_width_spiky;      /* Initialize.h:45 */
    s->q_scorr = ORC_IS_F32 ? (real)((float)s->h_spiky * P->q_scorr)
                            : s->h_spiky * (real)P->q_scorr;                  /* Initialize.h:49 */
    s->h_poly = (real)P->kernel_width_poly;                                   /* Initialize.h:53 */
    s->M = P->max_neighbours_per_particle;
    s->G = P->max_grid;
}

/* ----------------------------------------------------------------- lifecycle -------- */
static void* zalloc(size_t n) { void* p = calloc(n ? n : 1, 1); return p; }

void orc_destroy(orc_sim* s);

orc_sim* orc_create(const pbd_params* prm, uint32_t capacity) {
    orc_sim* s = (orc_sim*)zalloc(sizeof(orc_sim));
    if (!s) return NULL;
    s->prm = *prm;
    s->cap = capacity;
    derive(s);
    size_t c = capacity;
    s->x = zalloc(c * sizeof(r4)); s->p = zalloc(c * sizeof(r4)); s->v = zalloc(c * sizeof(r4));
    s->col = zalloc(c * sizeof(r4)); s->fext = zalloc(c * sizeof(r4)); s->delta = zalloc(c * sizeof(r4));
    s->omega = zalloc(c * sizeof(r4));
    s->xc = zalloc(c * sizeof(r4)); s->pc = zalloc(c * sizeof(r4)); s->vc = zalloc(c * sizeof(r4));
    s->colc = zalloc(c * sizeof(r4));
    s->lambda = zalloc(c * sizeof(real));
    s->w = zalloc(c * sizeof(real)); s->wc = zalloc(c * sizeof(real));
    for (size_t k = 0; k < c; ++k) s->w[k] = 1;
    s->ids = zalloc(c * 4); s->idsc = zalloc(c * 4);
    s->keys_in = zalloc(c * 4); s->keys_out = zalloc(c * 4); s->vals_in = zalloc(c * 4);
    s->vals_out = zalloc(c * 4); s->tmpk = zalloc(c * 4); s->tmpv = zalloc(c * 4);
    s->cell_start = zalloc((size_t)s->G * 4); s->cell_end = zalloc((size_t)s->G * 4);
    s->nbr = zalloc(c * (size_t)s->M * 4);
    s->nbr_count = zalloc(c * 4); s->contact_count = zalloc(c * 4);
    if (!s->x || !s->nbr || !s->cell_start || !s->cell_end) { orc_destroy(s); return NULL; }
    for (uint32_t i = 0; i < capacity; ++i) s->vals_in[i] = i;   /* initializeParticleIds, SortReorder.h:199-210 */
    for (uint32_t g = 0; g < s->G; ++g) { s->cell_start[g] = UINT32_MAX; s->cell_end[g] = 0; }
    return s;
}

void orc_destroy(orc_sim* s) {
    if (!s) return;
    void* bufs[] = {s->x, s->p, s->v, s->col, s->fext, s->delta, s->omega, s->xc, s->pc, s->vc, s->colc,
                    s->lambda, s->w, s->wc, s->ids, s->idsc, s->keys_in, s->keys_out, s->vals_in, s->vals_out,
                    s->tmpk, s->tmpv, s->cell_start, s->cell_end, s->nbr, s->nbr_count, s->contact_count,
                    s->csolved, s->cbest};
    for (size_t k = 0; k < sizeof(bufs) / sizeof(bufs[0]); ++k) free(bufs[k]);
    free(s);
}

int orc_set_params(orc_sim* s, const pbd_params* prm) {
    if (prm->max_neighbours_per_particle != s->prm.max_neighbours_per_particle || prm->max_grid != s->prm.max_grid)
        return PBD_ERR_UNSUPPORTED;   /* list and grid sizes are fixed at creation */
    s->prm = *prm;
    derive(s);
    return PBD_OK;
}

uint32_t orc_num_particles(const orc_sim* s) { return s->N; }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* --------------------------------------------- Communication.h:22-67, 626-660 ------ */
int orc_add_particles_mass(orc_sim* s, uint32_t n, const float* pos4, const float* vel4, const float* col4,
                           const float* inv_mass);
int orc_add_particles(orc_sim* s, uint32_t n, const float* pos4, const float* vel4, const float* col4) {
    return orc_add_particles_mass(s, n, pos4, vel4, col4, NULL);
}

/* Unified solids: inverse mass per particle (1 for everything added without it). */
int orc_add_particles_mass(orc_sim* s, uint32_t n, const float* pos4, const float* vel4, const float* col4,
                           const float* inv_mass) {
    if ((uint64_t)s->N + n > s->cap) return PBD_ERR_CAPACITY;   /* :645 (silent there) */
    if (inv_mass) s->mass_used = 1;
    for (uint32_t k = 0; k < n; ++k) s->w[s->N + k] = inv_mass ? (real)inv_mass[k] : (real)1;
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t i = s->N + k;
        s->x[i] = mk4(pos4[4 * k], pos4[4 * k + 1], pos4[4 * k + 2], pos4[4 * k + 3]);
        s->v[i] = mk4(vel4[4 * k], vel4[4 * k + 1], vel4[4 * k + 2], vel4[4 * k + 3]);
        if (col4) s->col[i] = mk4(col4[4 * k], col4[4 * k + 1], col4[4 * k + 2], col4[4 * k + 3]);
        s->ids[i] = i;
    }
    s->N += n;
    return PBD_OK;
}

int orc_add_particle(orc_sim* s, const float pos[3], const float dir[3]) {
    if ((uint64_t)s->N + 1 > s->cap) return PBD_ERR_CAPACITY;
    uint32_t i = s->N;
    s->x[i] = mk4(pos[0], pos[1], pos[2], 0);
    s->v[i] = mk4(50.0f * dir[0], 50.0f * dir[1], 50.0f * dir[2], 0);   /* :27 */
    s->col[i] = mk4(1, 0, 0, 1);
    s->ids[i] = i;
    s->w[i] = 1;
    s->N += 1;
    return PBD_OK;
}

void orc_clear(orc_sim* s) { s->N = 0; }

/* The external force of the current particles, in their current order (test hook: lets a frame
 * start from another implementation's state, whose f_ext the previous frame's vorticity left,
 * Forces.h:82, Fluid.cu:21-29). */
void orc_set_fext(orc_sim* s, const float* f4) {
    for (uint32_t i = 0; i < s->N; ++i) s->fext[i] = mk4(f4[4 * i], f4[4 * i + 1], f4[4 * i + 2], f4[4 * i + 3]);
}

/* ------------------------------------------------------------ Forces.h:19-101 ------- */
static void apply_forces(orc_sim* s) {
    const pbd_params* P = &s->prm;
    const real dt = (real)P->delta_t, g = (real)P->gravity;
    const real vd = (real)P->enclosure_velocity_damping, pd = (real)P->enclosure_position_damping;
    const real bmin[3] = {P->bounds_min[0], P->bounds_min[1], P->bounds_min[2]};
    const real bmax[3] = {P->bounds_max[0], P->bounds_max[1], P->bounds_max[2]};
    const real eps = (real)0.001f;
    const int N = (int)s->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        r4 v = s->v[i];
        if (s->w[i] != 0) {                           /* solids (inverse mass 0) take no forces */
            v.y = FMA(g, dt, v.y);                    /* velocity.y += inverseMass*gravity*deltaT */
            r4 f = s->fext[i];
            v.x = FMA(f.x, dt, v.x); v.y = FMA(f.y, dt, v.y);
            v.z = FMA(f.z, dt, v.z); v.w = FMA(f.w, dt, v.w);  /* velocity += externalForces*deltaT */
        }
        r4 x = s->x[i];
        r4 p = mk4(FMA(v.x, dt, x.x), FMA(v.y, dt, x.y), FMA(v.z, dt, x.z), FMA(v.w, dt, x.w));
        int upd = 0;
        real* pc[3] = {&p.x, &p.y, &p.z};
        real* vc[3] = {&v.x, &v.y, &v.z};
        for (int a = 0; a < 3; ++a) {                 /* confineToBox, Forces.h:26-54 */
            if (*pc[a] < bmin[a]) { *vc[a] = vd * *vc[a]; *pc[a] = bmin[a] + eps; upd = 1; }
            else if (*pc[a] > bmax[a]) { *vc[a] = vd * *vc[a]; *pc[a] = bmax[a] - eps; upd = 1; }
        }
        if (upd) {                                     /* Forces.h:56-58 */
            x.x = FMA(pd, p.x - x.x, x.x); x.y = FMA(pd, p.y - x.y, x.y);
            x.z = FMA(pd, p.z - x.z, x.z); x.w = FMA(pd, p.w - x.w, x.w);
            s->x[i] = x;
        }
        s->v[i] = v;
        p.w = (real)1;                                 /* Forces.h:94 */
        s->p[i] = p;
    }
}

/* ------------------------------------------------------ SortReorder.h:13-188 -------- */
static void initialize_cell_ids(orc_sim* s) {
    const int N = (int)s->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) s->keys_in[i] = morton_r(s->p[i].x, s->p[i].y, s->p[i].z);
}

/* Stable LSD counting sort of (key, value) over 32 bits, 8 bits per pass. */
static void sort_ids(orc_sim* s) {
    const uint32_t N = s->N;
    uint32_t *ka = s->tmpk, *va = s->tmpv, *kb = s->keys_out, *vb = s->vals_out;
    memcpy(ka, s->keys_in, N * 4u);
    memcpy(va, s->vals_in, N * 4u);   /* SortPairs never writes its inputs: vals_in stays identity */
    for (int pass = 0; pass < 4; ++pass) {
        uint32_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        int sh = 8 * pass;
        for (uint32_t i = 0; i < N; ++i) cnt[((ka[i] >> sh) & 255u) + 1]++;
        for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
        for (uint32_t i = 0; i < N; ++i) {
            uint32_t d = (ka[i] >> sh) & 255u;
            uint32_t o = cnt[d]++;
            kb[o] = ka[i]; vb[o] = va[i];
        }
        uint32_t* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    /* after 4 passes the result is back in tmpk/tmpv */
    memcpy(s->keys_out, ka, N * 4u);
    memcpy(s->vals_out, va, N * 4u);
}

static void reorder(orc_sim* s) {          /* copy (:53-75) + reorder (:86-115) */
    const int N = (int)s->N;
    memcpy(s->xc, s->x, N * sizeof(r4)); memcpy(s->pc, s->p, N * sizeof(r4));
    memcpy(s->vc, s->v, N * sizeof(r4)); memcpy(s->colc, s->col, N * sizeof(r4));
    memcpy(s->idsc, s->ids, N * 4u);
    memcpy(s->wc, s->w, N * sizeof(real));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        uint32_t o = s->vals_out[i];
        s->x[i] = s->xc[o]; s->p[i] = s->pc[o]; s->v[i] = s->vc[o]; s->col[i] = s->colc[o];
        s->ids[i] = s->idsc[o];
        s->w[i] = s->wc[o];
    }
}

static void reset_cell_info(orc_sim* s) {   /* :135-149 */
    for (uint32_t g = 0; g < s->G; ++g) { s->cell_start[g] = UINT32_MAX; s->cell_end[g] = s->N; }
}

static void compute_cell_info(orc_sim* s) { /* :160-188 */
    const uint32_t N = s->N;
    const uint32_t* k = s->keys_out;
    /* Keys >= maxGrid would index past the reference's tables (undefined there); they are
     * left out of the tables here. */
    for (uint32_t i = 0; i < N; ++i) {
        uint32_t c = k[i];
        if (i == 0) {
            if (c < s->G) s->cell_start[c] = 0;
        } else {
            uint32_t pc = k[i - 1];
            if (pc != c) {
                if (c < s->G) s->cell_start[c] = i;
                if (pc < s->G) s->cell_end[pc] = i;
            }
        }
    }
    if ((s->prm.flags & PBD_FLAG_CELL_END_QUIRK) && N >= 2 && N - 1 < s->G)
        s->cell_end[N - 1] = N;              /* :183-184, applied last */
}

/* ---------------------------------------------------------- Collision.h:11-160 ------ */
static inline uint32_t offset_hash(const orc_sim* s, r4 p, int a, int b, int c) {
    const real d = s->diameter;
    return morton_r(FMA((real)a, d, p.x), FMA((real)b, d, p.y), FMA((real)c, d, p.z));
}

static void find_neighbours_all(orc_sim* s) {
    const uint32_t N = s->N, M = s->M, G = s->G;
    const int K = (int)s->prm.kernel_width_neighbours;
    const int do_contacts = (s->prm.active & PBD_ACTIVE_FIND_CONTACTS) != 0;
    const int do_shells = (s->prm.active & PBD_ACTIVE_FIND_NEIGHBOURS) != 0;
    const int iN = (int)N;
#pragma omp parallel for schedule(dynamic, 256)
    for (int ii = 0; ii < iN; ++ii) {
        const uint32_t i = (uint32_t)ii;
        uint32_t* list = s->nbr + (size_t)i * M;
        uint32_t cnt = 0;
        const r4 p1 = s->p[i];
        int full = (M == 0);
        if (do_contacts && !full) {               /* findContacts, :43-71 */
            for (int a = -1; a <= 1 && !full; ++a)
                for (int b = -1; b <= 1 && !full; ++b)
                    for (int c = -1; c <= 1 && !full; ++c) {
                        uint32_t h = offset_hash(s, p1, a, b, c);
                        if (h >= G) continue;
                        uint32_t st = s->cell_start[h];
                        if (st >= N) continue;
                        uint32_t en = s->cell_end[h];
                        for (uint32_t j = st; j < en; ++j) {
                            if (j != i && j < N) {
                                list[cnt++] = j;
                                if (cnt == M) { full = 1; break; }
                            }
                        }
                    }
        }
        s->contact_count[i] = cnt;
        if (do_shells && !full) {                 /* findNeighbours, :126-155 */
            for (int sh = 2; sh <= K && !full; ++sh)
                for (int a = -sh; a <= sh && !full; ++a)
                    for (int b = -sh; b <= sh && !full; ++b)
                        for (int c = -sh; c <= sh && !full; ++c) {
                            if (abs(a) != sh && abs(b) != sh && abs(c) != sh) continue;
                            uint32_t h = offset_hash(s, p1, a, b, c);
                            if (h >= G) continue;
                            uint32_t st = s->cell_start[h];
                            uint32_t en = s->cell_end[h];
                            if (st == UINT32_MAX) continue;
                            for (uint32_t j = st; j < en; ++j) {
                                if (j != i && j < N) {
                                    list[cnt++] = j;
                                    if (cnt == M) { full = 1; break; }
                                }
                            }
                        }
        }
        s->nbr_count[i] = cnt;
        if (do_shells && (s->prm.flags & PBD_FLAG_COLORS)) {   /* :118-120 */
            real f = (real)((float)cnt / (float)M);
            s->col[i] = mk4(f, f, f, 1);
        }
    }
}

/* ----------------------------------------------------------- Density.h:48-168 ------- */
static void compute_lambda(orc_sim* s) {
    const int N = (int)s->N;
    const real rho0 = (real)s->prm.rest_density, eps = (real)s->prm.lambda_epsilon;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const uint32_t* list = s->nbr + (size_t)i * s->M;
        const r4 pi = s->p[i];
        real A = 0, B = 0;
        r4 C = mk4(0, 0, 0, 0);
        for (uint32_t k = 0; k < s->nbr_count[i]; ++k) {
            const r4 pj = s->p[list[k]];
            A += poly6(s, len3(sub4(pi, pj)));
            r4 g = spiky(s, pi, pj);
            B += dot4(g, g);
            C = add4(C, g);
        }
        real a = (A / rho0) - (real)1;
        real b = B / rho0;
        real c = dot4(C, C) / rho0;
        s->lambda[i] = -a / (b + c + eps);
    }
}

static void compute_delta_positions(orc_sim* s) {
    const int N = (int)s->N;
    const real rho0 = (real)s->prm.rest_density, k = (real)s->prm.k_scorr;
    const int n = s->prm.n_scorr;
    /* poly6Viscosity(make_float4(q,0,0,0), make_float4(0,0,0,0)): distance = length((q,0,0)) */
    const real Wq = poly6(s, SQRT(s->q_scorr * s->q_scorr + (real)0 + (real)0));
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const uint32_t* list = s->nbr + (size_t)i * s->M;
        const r4 pi = s->p[i];
        const real li = s->lambda[i];
        r4 acc = mk4(0, 0, 0, 0);
        for (uint32_t kk = 0; kk < s->nbr_count[i]; ++kk) {
            const uint32_t j = list[kk];
            const r4 pj = s->p[j];
            const real sc = -k * powi_r(poly6(s, len3(sub4(pi, pj))) / Wq, n);
            acc = add4(acc, scl4(li + s->lambda[j] + sc, spiky(s, pi, pj)));
        }
        s->delta[i] = mk4(acc.x / rho0, acc.y / rho0, acc.z / rho0, acc.w / rho0);
    }
}

static void apply_delta_positions(orc_sim* s) {
    const int N = (int)s->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) s->p[i] = sub4(s->p[i], s->mass_used ? scl4(s->w[i], s->delta[i]) : s->delta[i]);
}

/* --------------------------------------------------- Collision.h:171-242 (Jacobi) --- */
static void solve_collisions(orc_sim* s) {
    const int N = (int)s->N;
    const real d = s->diameter, st = (real)s->prm.stiffness;
    memcpy(s->pc, s->p, (size_t)N * sizeof(r4));     /* snapshot */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const uint32_t* list = s->nbr + (size_t)i * s->M;
        const r4 p1 = s->pc[i];
        r4 pa = s->p[i], xa = s->x[i];
        for (uint32_t kk = 0; kk < s->contact_count[i]; ++kk) {
            const r4 p2 = s->pc[list[kk]];
            r4 dir = sub4(p2, p1);
            real len = len3(dir);
            real overlap = d - len;
            real share = (real)0.5;   /* inverseMass1 / (inverseMass1 + inverseMass2), Collision.h:223-225 */
            if (s->mass_used) {
                const real wi = s->w[i], wj = s->w[list[kk]];
                share = (wi + wj) > 0 ? wi / (wi + wj) : 0;
                if (share == 0) continue;
            }
            if (overlap > 0) {
                if (len <= (real)0.00001f) continue;
                real nx = dir.x / len, ny = dir.y / len, nz = dir.z / len;
                /* -1.0 * inverseMass * overlap is evaluated in double (Collision.h:227) */
                real sc = ORC_IS_F32 ? (real)(float)(-1.0 * (double)share * (double)overlap) : -share * overlap;
                real one_m = (real)1 - st;
                real ax = sc * nx * one_m, ay = sc * ny * one_m, az = sc * nz * one_m;
                pa.x += ax; xa.x += ax;
                pa.y += ay; xa.y += ay;
                pa.z += az; xa.z += az;
            }
        }
        s->p[i] = pa;
        s->x[i] = xa;
    }
}

/* ------------------------------------- Collision.h:288-436 (collisionType 1), batched ---
 * The reference claims contacts with a __syncthreads inside divergent code and lets blocks race
 * on the claims (undefined across blocks).  Restated deterministically as locally dominant
 * matching: the constraints are the frame's list entries c = i * M + k (partner list[k];
 * Fluid.cu:37-47 fills the same array).  In each of maxCollisionBatches batches, a constraint
 * not yet solved in this stabilization pass competes when its particles overlap at the batch's
 * start (diameter - |p_j - p_i| > 0, |p_j - p_i| > 1e-5, a movable particle); its priority is
 * lowbias32(c + 1) (C. Wellons' published 32-bit integer mix) above c itself; every particle takes
 * its highest-priority competing constraint, and a constraint both of whose particles took it is
 * solved -- a batch is a matching, so its projections are independent.  Solving follows
 * setupCollisionConstraintBatchesCheck: d = p2 - p1 (w = 0), half = (diameter - |d|) / 2,
 * p1 and x1 move by -n half (1 - stiffness), p2 and x2 by +n half (1 - stiffness), and both p*
 * are written back with w = 0.  Unified solids split the overlap by inverse mass (w1 / (w1 + w2);
 * 1/2 with unit masses, the same bits as half). */
static inline uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

static int contact_geometry(const orc_sim* s, uint32_t i, uint32_t j, r4* n, real* h1, real* h2) {
    r4 p1 = s->p[i], p2 = s->p[j];
    p1.w = 0; p2.w = 0;
    const r4 dir = sub4(p2, p1);
    const real len = len3(dir);
    real s1 = (real)0.5, s2 = (real)0.5;
    if (s->mass_used) {
        const real w1 = s->w[i], w2 = s->w[j];
        if (!(w1 + w2 > 0)) return 0;
        s1 = w1 / (w1 + w2);
        s2 = w2 / (w1 + w2);
    }
    const real overlap = s->diameter - len;
    if (!(overlap * (real)0.5 > 0) || len <= (real)0.00001f) return 0;
    *n = mk4(dir.x / len, dir.y / len, dir.z / len, dir.w / len);
    *h1 = overlap * s1;
    *h2 = overlap * s2;
    return 1;
}

static int solve_collisions_batched(orc_sim* s) {
    const uint32_t N = s->N, M = s->M;
    const real one_m = (real)1 - (real)s->prm.stiffness;
    if (!s->csolved) {
        s->csolved = (uint8_t*)zalloc((size_t)s->cap * M);
        s->cbest = (uint64_t*)zalloc((size_t)s->cap * sizeof(uint64_t));
        if (!s->csolved || !s->cbest) return PBD_ERR_ALLOC;
    }
    memset(s->csolved, 0, (size_t)N * M);
    uint64_t* best = s->cbest;
    for (uint32_t b = 0; b < s->prm.max_collision_batches; ++b) {
        memset(best, 0, (size_t)N * sizeof(uint64_t));
        for (uint32_t i = 0; i < N; ++i) {
            const uint32_t* list = s->nbr + (size_t)i * M;
            for (uint32_t k = 0; k < s->nbr_count[i]; ++k) {
                const uint32_t c = i * M + k;
                if (s->csolved[c]) continue;
                r4 n; real h1, h2;
                const uint32_t j = list[k];
                if (!contact_geometry(s, i, j, &n, &h1, &h2)) continue;
                const uint64_t key = ((uint64_t)lowbias32(c + 1u) << 32) | c;   /* never 0: lowbias32 fixes only 0 */
                if (key > best[i]) best[i] = key;
                if (key > best[j]) best[j] = key;
            }
        }
        for (uint32_t i = 0; i < N; ++i) {
            const uint64_t key = best[i];
            if (!key) continue;
            const uint32_t c = (uint32_t)key;
            if (c / M != i) continue;
            const uint32_t j = s->nbr[c];
            if (best[j] != key) continue;
            s->csolved[c] = 1;
            r4 n; real h1, h2;
            if (!contact_geometry(s, i, j, &n, &h1, &h2)) continue;
            const r4 a1 = mk4(-n.x * h1 * one_m, -n.y * h1 * one_m, -n.z * h1 * one_m, -n.w * h1 * one_m);
            const r4 a2 = mk4(n.x * h2 * one_m, n.y * h2 * one_m, n.z * h2 * one_m, n.w * h2 * one_m);
            r4 p1 = s->p[i], p2 = s->p[j];
            p1.w = 0; p2.w = 0;
            s->p[i] = add4(p1, a1);
            s->p[j] = add4(p2, a2);
            s->x[i] = add4(s->x[i], a1);
            s->x[j] = add4(s->x[j], a2);
        }
    }
    return PBD_OK;
}

/* ---------------------------------------------------------------- Update.h:11-32 ---- */
static void update_positions(orc_sim* s) {
    const int N = (int)s->N;
    const real dt = (real)s->prm.delta_t;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        r4 d = sub4(s->p[i], s->x[i]);
        s->v[i] = mk4(d.x / dt, d.y / dt, d.z / dt, d.w / dt);
        s->x[i] = s->p[i];
    }
}

/* -------------------------------------------------------- Density.h:179-310 --------- */
static void compute_omega(orc_sim* s) {
    const int N = (int)s->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const uint32_t* list = s->nbr + (size_t)i * s->M;
        const r4 pi = s->p[i], vi = s->v[i];
        real ox = 0, oy = 0, oz = 0;
        for (uint32_t kk = 0; kk < s->nbr_count[i]; ++kk) {
            const uint32_t j = list[kk];
            r4 vij = sub4(s->v[j], vi);
            r4 g = spiky(s, pi, s->p[j]);
            ox += vij.y * g.z - vij.z * g.y;
            oy += vij.z * g.x - vij.x * g.z;
            oz += vij.x * g.y - vij.y * g.x;
        }
        s->omega[i] = mk4(ox, oy, oz, 0);
    }
}

static void compute_vorticity(orc_sim* s) {
    const int N = (int)s->N;
    const real e = (real)s->prm.e_vorticity;
    const real EPS = (real)0.00000001f;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const uint32_t* list = s->nbr + (size_t)i * s->M;
        const r4 pi = s->p[i];
        const r4 oi = s->omega[i];
        real gx = 0, gy = 0, gz = 0;
        for (uint32_t kk = 0; kk < s->nbr_count[i]; ++kk) {
            const uint32_t j = list[kk];
            const r4 oj = s->omega[j];
            r4 dw = sub4(oj, oi);
            real ol = len3(dw);
            r4 pj = s->p[j];
            real px = pj.x - pi.x + EPS, py = pj.y - pi.y + EPS, pz = pj.z - pi.z + EPS;
            gx += ol / px; gy += ol / py; gz += ol / pz;
        }
        real gl = SQRT(gx * gx + gy * gy + gz * gz);
        real inv = (real)1 / (gl + EPS);
        real Nx = inv * (gx + EPS), Ny = inv * (gy + EPS), Nz = inv * (gz + EPS);
        real cx = Ny * oi.z - Nz * oi.y, cy = Nz * oi.x - Nx * oi.z, cz = Nx * oi.y - Ny * oi.x;
        s->fext[i] = mk4(e * cx, e * cy, e * cz, 0);
    }
}

static void compute_viscosity(orc_sim* s) {
    const int N = (int)s->N;
    const real c = (real)s->prm.c_viscosity;
    memcpy(s->vc, s->v, (size_t)N * sizeof(r4));     /* snapshot (Jacobi) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const uint32_t* list = s->nbr + (size_t)i * s->M;
        const r4 pi = s->p[i], vi = s->vc[i];
        r4 sum = mk4(0, 0, 0, 0);
        for (uint32_t kk = 0; kk < s->nbr_count[i]; ++kk) {
            const uint32_t j = list[kk];
            r4 vij = sub4(s->vc[j], vi);
            sum = add4(sum, scl4(poly6(s, len3(sub4(pi, s->p[j]))), vij));
        }
        s->v[i] = add4(vi, scl4(s->mass_used ? s->w[i] * c : c, sum));
    }
}

/* ------------------------------------------------------------ Fluid.cu:14-97 -------- */
#define ORC_PHASE_ALL 0
#define ORC_PHASE_FRONT 1      /* stop after computeCellInfo (Fluid.cu:33) */
#define ORC_PHASE_LISTS 2      /* stop after findNeighbours (Fluid.cu:47) */

int orc_step_phase(orc_sim* s, int phase) {
    const pbd_params* P = &s->prm;
    if (s->N == 0) return PBD_OK;                         /* Fluid.cu:19 */
    if (P->collision_type > 1) return PBD_ERR_UNSUPPORTED;
    if (P->active & PBD_ACTIVE_APPLY_FORCES) apply_forces(s);
    initialize_cell_ids(s);
    sort_ids(s);
    reorder(s);
    reset_cell_info(s);
    compute_cell_info(s);
    if (phase == ORC_PHASE_FRONT) return PBD_OK;
    find_neighbours_all(s);
    if (phase == ORC_PHASE_LISTS) return PBD_OK;
    for (uint32_t it = 0; it < P->solver_iterations; ++it) {
        if (P->active & PBD_ACTIVE_COMPUTE_LAMBDA) compute_lambda(s);
        if (P->active & PBD_ACTIVE_COMPUTE_DELTA_POSITIONS) compute_delta_positions(s);
        for (uint32_t k = 0; k < P->stabilization_iterations; ++k) {
            if (P->collision_type == 0) {
                solve_collisions(s);
            } else {
                const int rc = solve_collisions_batched(s);
                if (rc) return rc;
            }
        }
        if (P->active & PBD_ACTIVE_APPLY_DELTA_POSITIONS) apply_delta_positions(s);
    }
    if (P->active & PBD_ACTIVE_UPDATE_POSITIONS) update_positions(s);
    if (P->active & PBD_ACTIVE_COMPUTE_OMEGAS) compute_omega(s);
    if (P->active & PBD_ACTIVE_COMPUTE_VORTICITY) compute_vorticity(s);
    if (P->active & PBD_ACTIVE_COMPUTE_VISCOSITY) compute_viscosity(s);
    return PBD_OK;
}

int orc_step(orc_sim* s, int nsteps) {
    for (int k = 0; k < nsteps; ++k) {
        int rc = orc_step_phase(s, ORC_PHASE_ALL);
        if (rc) return rc;
    }
    return PBD_OK;
}

/* ------------------------------------------------------------------ read-out -------- */
static void out4(const r4* a, double* o, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) { o[4 * i] = a[i].x; o[4 * i + 1] = a[i].y; o[4 * i + 2] = a[i].z; o[4 * i + 3] = a[i].w; }
}

void orc_get_state(const orc_sim* s, double* x4, double* v4, double* p4, uint32_t* ids) {
    if (x4) out4(s->x, x4, s->N);
    if (v4) out4(s->v, v4, s->N);
    if (p4) out4(s->p, p4, s->N);
    if (ids) memcpy(ids, s->ids, s->N * 4u);
}

void orc_get_debug(const orc_sim* s, uint32_t* keys, uint32_t* perm, uint32_t* cell_start,
                   uint32_t* cell_end, uint32_t ncells, double* lambda, double* fext4, double* omega4,
                   double* col4) {
    const uint32_t N = s->N;
    if (keys) memcpy(keys, s->keys_out, N * 4u);
    if (perm) memcpy(perm, s->vals_out, N * 4u);
    if (ncells > s->G) ncells = s->G;
    if (cell_start) memcpy(cell_start, s->cell_start, (size_t)ncells * 4);
    if (cell_end) memcpy(cell_end, s->cell_end, (size_t)ncells * 4);
    if (lambda) for (uint32_t i = 0; i < N; ++i) lambda[i] = s->lambda[i];
    if (fext4) out4(s->fext, fext4, N);
    if (omega4) out4(s->omega, omega4, N);
    if (col4) out4(s->col, col4, N);
}

void orc_get_neighbours(const orc_sim* s, uint32_t max_entries, uint32_t* list, uint32_t* count,
                        uint32_t* contacts) {
    const uint32_t N = s->N;
    for (uint32_t i = 0; i < N; ++i) {
        uint32_t c = s->nbr_count[i];
        if (count) count[i] = c;
        if (contacts) contacts[i] = s->contact_count[i];
        if (list) {
            uint32_t m = c < max_entries ? c : max_entries;
            memcpy(list + (size_t)i * max_entries, s->nbr + (size_t)i * s->M, m * 4u);
        }
    }
}

/* Density-constraint error |rho_i/rho0 - 1| (Density.h:84) over the current state. */
void orc_density_error(orc_sim* s, double* out) {
    const int N = (int)s->N;
    const real rho0 = (real)s->prm.rest_density;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
        const uint32_t* list = s->nbr + (size_t)i * s->M;
        real A = 0;
        for (uint32_t k = 0; k < s->nbr_count[i]; ++k) A += poly6(s, len3(sub4(s->p[i], s->p[list[k]])));
        out[i] = (double)(A / rho0 - (real)1);
    }
}

int orc_real_size(void) { return (int)sizeof(real); }

/* ---------------------------------- particle sprites (particleSpriteGeom.vert/.geom/.frag) ---
 * Float arithmetic with every operation correctly rounded and in a fixed order (this file is
 * built with -ffp-contract=off), so the CUDA renderer, written with the same operations in the
 * same order, gives the same bits.  pow(x, 1/6) is a 32-step bisection on [0, 1] and pow(s, 10)
 * repeated squaring -- the renderer's own definitions, not GLSL's pow. */
static float spr_root6(float x) {
    if (!(x > 0.0f)) return 0.0f;
    if (x >= 1.0f) return 1.0f;
    float lo = 0.0f, hi = 1.0f;
    for (int k = 0; k < 32; ++k) {
        const float m = (lo + hi) * 0.5f;
        const float m2 = m * m;
        const float m6 = (m2 * m2) * m2;
        if (m6 < x) lo = m; else hi = m;
    }
    return lo;
}

/* column-major 4x4 times (x, y, z, w): ((m0 x + m4 y) + m8 z) + m12 w per row */
static void spr_mat4(const float* m, float x, float y, float z, float w, float* o) {
    for (int r = 0; r < 4; ++r) o[r] = ((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * w;
}

static void spr_normalize3(float* v) {
    const float l = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    v[0] = v[0] / l; v[1] = v[1] / l; v[2] = v[2] / l;
}

static uint32_t spr_unorm8(float c) {
    c = c < 0.0f ? 0.0f : (c > 1.0f ? 1.0f : c);
    return (uint32_t)floorf(c * 255.0f + 0.5f);
}

void orc_render_sprites(const float* pos4, const float* col4, uint32_t n, const pbd_camera* cam, uint8_t* rgba,
                        float* depth) {
    const uint32_t W = cam->width, H = cam->height;
    uint64_t* key = (uint64_t*)malloc((size_t)W * H * sizeof(uint64_t));
    if (!key) return;
    uint32_t clear = spr_unorm8(cam->clear_rgba[0]) | (spr_unorm8(cam->clear_rgba[1]) << 8) |
                     (spr_unorm8(cam->clear_rgba[2]) << 16) | (spr_unorm8(cam->clear_rgba[3]) << 24);
    float one = 1.0f;
    uint32_t one_bits;
    memcpy(&one_bits, &one, 4);
    for (size_t q = 0; q < (size_t)W * H; ++q) key[q] = ((uint64_t)one_bits << 32) | clear;
    const float* V = cam->view;
    const float r = cam->sphere_radius;
    float vd[3] = {-cam->view_direction[0], -cam->view_direction[1], -cam->view_direction[2]};
    spr_normalize3(vd);
    for (uint32_t i = 0; i < n; ++i) {
        const float px = pos4[4 * i], py = pos4[4 * i + 1], pz = pos4[4 * i + 2];
        const float t = spr_root6(col4 ? col4[4 * i] : 0.0f);
        const float c[3] = {0.95f * (1.0f - t) + 0.0f * t, 0.97f * (1.0f - t) + 0.0f * t, 0.97f * (1.0f - t) + 1.0f * t};
        float L[3] = {cam->light_position[0] - px, cam->light_position[1] - py, cam->light_position[2] - pz};
        spr_normalize3(L);
        float vp[4];
        spr_mat4(V, px, py, pz, 1.0f, vp);
        float lo[4], hi[4];
        spr_mat4(cam->projection, vp[0] - r, vp[1] - r, vp[2], vp[3], lo);
        spr_mat4(cam->projection, vp[0] + r, vp[1] + r, vp[2], vp[3], hi);
        if (!(lo[3] > 0.0f)) continue;                              /* behind the eye */
        const float zn = lo[2] / lo[3];
        if (zn < -1.0f || zn > 1.0f) continue;                     /* outside the near / far planes */
        const float x0 = (lo[0] / lo[3] * 0.5f + 0.5f) * (float)W, y0 = (lo[1] / lo[3] * 0.5f + 0.5f) * (float)H;
        const float x1 = (hi[0] / hi[3] * 0.5f + 0.5f) * (float)W, y1 = (hi[1] / hi[3] * 0.5f + 0.5f) * (float)H;
        if (!(x1 > x0) || !(y1 > y0)) continue;
        long ix0 = (long)ceilf(x0 - 0.5f), ix1 = (long)ceilf(x1 - 0.5f);
        long iy0 = (long)ceilf(y0 - 0.5f), iy1 = (long)ceilf(y1 - 0.5f);
        if (ix0 < 0) ix0 = 0;
        if (iy0 < 0) iy0 = 0;
        if (ix1 > (long)W) ix1 = (long)W;
        if (iy1 > (long)H) iy1 = (long)H;
        const float sx = 2.0f / (x1 - x0), sy = 2.0f / (y1 - y0);
        for (long iy = iy0; iy < iy1; ++iy) {
            const float v = ((float)iy + 0.5f - y0) * sy - 1.0f;
            for (long ix = ix0; ix < ix1; ++ix) {
                const float u = ((float)ix + 0.5f - x0) * sx - 1.0f;
                const float mag = u * u + v * v;
                if (mag > 1.0f) continue;
                const float nz = sqrtf(1.0f - mag);
                /* inverse of the view rotation = its transpose: N_world[k] = sum_r V[4k + r] N[r] */
                float N[3];
                for (int k = 0; k < 3; ++k) N[k] = (V[4 * k] * u + V[4 * k + 1] * v) + V[4 * k + 2] * nz;
                spr_normalize3(N);
                const float ln = (L[0] * N[0] + L[1] * N[1]) + L[2] * N[2];
                float R[3];
                for (int k = 0; k < 3; ++k) R[k] = -L[k] + (2.0f * ln) * N[k];
                float rv = (R[0] * vd[0] + R[1] * vd[1]) + R[2] * vd[2];
                rv = rv < 0.0f ? 0.0f : (rv > 1.0f ? 1.0f : rv);
                const float s2 = rv * rv, s4 = s2 * s2, s8 = s4 * s4, s10 = s8 * s2;
                const float diff = ln > 0.0f ? ln : 0.0f;
                uint32_t col = 0;
                for (int k = 0; k < 3; ++k) {
                    const float f = (0.3f * c[k] + (0.7f * diff) * c[k]) + (0.2f * s10) * 1.0f;
                    col |= spr_unorm8(f) << (8 * k);
                }
                col |= 255u << 24;
                float dp[4];
                spr_mat4(cam->projection, vp[0], vp[1], vp[2] + r * nz, vp[3], dp);
                float dz = 0.5f * (dp[2] / dp[3]) + 0.5f;
                if (dz < 0.0f) dz = 0.0f;
                if (!(dz < 1.0f)) continue;                        /* GL_LESS against the cleared 1 */
                uint32_t db;
                memcpy(&db, &dz, 4);
                const uint64_t k64 = ((uint64_t)db << 32) | col;
                const size_t q = (size_t)iy * W + (size_t)ix;
                if (k64 < key[q]) key[q] = k64;
            }
        }
    }
    for (uint32_t y = 0; y < H; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            const uint64_t k64 = key[(size_t)y * W + x];
            const size_t o = (size_t)(H - 1 - y) * W + x;             /* rows top-down */
            if (rgba) { const uint32_t c = (uint32_t)k64; memcpy(rgba + 4 * o, &c, 4); }
            if (depth) { const uint32_t db = (uint32_t)(k64 >> 32); memcpy(depth + o, &db, 4); }
        }
    free(key);
}
