/*
 * oracle_gi.c -- CPU oracle of SVO ray traversal and of plain GI.
 *
 * TEST INFRASTRUCTURE.  Neither exists in the reference as a runnable pass:
 * its GPU traversal (svo_functions.inc:1-329) only feeds a debug view and
 * shading.frag:285-316 does direct light only; secondary rays exist only in a
 * disabled CPU probe (tgvk_raytracer.c:1390-1434).  This file therefore
 * DEFINES the semantics the CUDA path must reproduce, using only exactly
 * rounded binary32 operations (+ - * / sqrt floor) so that both sides give
 * the same bits:
 *
 *  - traversal: a hierarchical DDA over the one-bit voxel set (the same set
 *    tg_svo_create builds): occupancy levels of cells of 2^g voxels for
 *    g = L-1, ..., 9, 7, 5 (every other level of the block pyramid), then
 *    g = 3 and 2 (8^3 and 4^3 cells inside a 32^3 block), then single
 *    voxels; descend into occupied cells, step out of empty ones through the
 *    nearest face, ascend when the step leaves the parent; one loop
 *    iteration is one step.  The hit is the first set voxel along the ray,
 *    its distance is the entry distance, its normal the face crossed.
 *  - primary hits come from the visibility buffer, decoded as shading.frag
 *    does (:116-135), with the hit point and face normal of shading.frag:
 *    177-228 in cluster space and rotated to world space.
 *  - bounce lighting: Lambertian albedo from the material LUT, a directional
 *    sun with an SVO shadow ray, a constant sky, cosine-weighted secondary
 *    directions from a randomised R2 point set per (pixel, bounce) (see
 *    sample_cosine), random numbers from Philox4x32-10 (Salmon et al. 2011)
 *    keyed by the seed and counted by (pixel, bounce, frame, tag).
 */
#include "oracle_common.h"

#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* SVO in the oracle: dense block table over the non-empty blocks.     */
/* ------------------------------------------------------------------ */

typedef struct
{
    float     mn[3];
    uint32_t  L, B, NL;          /* side 2^L, blocks per axis, traversal levels */
    uint32_t* table;             /* B^3, 0 = empty, else block + 1 */
    uint32_t* words;             /* n * 1024 */
    uint16_t* mats;              /* n * 32768 or NULL */
    uint32_t* occ;               /* pyramid bits, level 0 = blocks */
    uint64_t  occ_off[16];
    uint32_t* sub;               /* n * 32: 8^3 cells of 4^3 voxels (words 0-15), 4^3 cells of 8^3 (16-17) */
    uint32_t  lg[16];            /* traversal level li covers cells of 2^lg[li] voxels */
} osvo;

/* Traversal levels for side 2^L: 1, 4, 8, 32, 128, 512, ... and 2^(L-1) on top. */
uint32_t oracle_svo_levels(uint32_t L, uint32_t* lg)
{
    uint32_t n = 0;
    lg[n++] = 0; lg[n++] = 2; lg[n++] = 3; lg[n++] = 5;
    for (uint32_t g = 7; g < L - 1; g += 2) lg[n++] = g;
    if (lg[n - 1] != L - 1) lg[n++] = L - 1;
    return n;
}

/* sub-block occupancy of one 4 KiB block (bit 1024z + 32y + x) */
void oracle_svo_sub_masks(const uint32_t* w, uint32_t out[32])
{
    memset(out, 0, 32 * 4);
    for (uint32_t z = 0; z < 32; z++)
        for (uint32_t y = 0; y < 32; y++)
        {
            const uint32_t row = w[z * 32 + y];
            for (uint32_t x = 0; x < 32; x++)
                if ((row >> x) & 1u)
                {
                    const uint32_t i4 = ((z >> 2) * 8 + (y >> 2)) * 8 + (x >> 2);
                    const uint32_t i8 = ((z >> 3) * 4 + (y >> 3)) * 4 + (x >> 3);
                    out[i4 >> 5] |= 1u << (i4 & 31u);
                    out[16 + (i8 >> 5)] |= 1u << (i8 & 31u);
                }
        }
}

void* oracle_svo_open(const int32_t* block_xyz, const uint32_t* words, const uint16_t* mats, uint32_t n,
                      const float mn[3], uint32_t L)
{
    osvo* s = (osvo*)calloc(1, sizeof(osvo));
    memcpy(s->mn, mn, sizeof(s->mn));
    s->L = L;
    s->B = 1u << (L - 5);
    s->NL = oracle_svo_levels(L, s->lg);
    const uint64_t nt = (uint64_t)s->B * s->B * s->B;
    s->table = (uint32_t*)calloc(nt, 4);
    s->words = (uint32_t*)malloc((size_t)(n ? n : 1) * 4096);
    memcpy(s->words, words, (size_t)n * 4096);
    if (mats)
    {
        s->mats = (uint16_t*)malloc((size_t)(n ? n : 1) * 65536);
        memcpy(s->mats, mats, (size_t)n * 65536);
    }
    uint64_t off = 0;
    for (uint32_t k = 0; k + 1 <= s->NL - 1 + 1 && k < 16; k++)
    {
        const uint64_t m = (uint64_t)(s->B >> k);
        if (m == 0) break;
        s->occ_off[k] = off;
        off += (m * m * m + 31) / 32;
    }
    s->occ = (uint32_t*)calloc(off + 1, 4);
    s->sub = (uint32_t*)calloc((size_t)(n ? n : 1) * 32, 4);
    for (uint32_t i = 0; i < n; i++)
    {
        oracle_svo_sub_masks(&s->words[(size_t)i * 1024], &s->sub[(size_t)i * 32]);
        const uint32_t bx = (uint32_t)((float)block_xyz[3 * i] - mn[0]) / 32u;
        const uint32_t by = (uint32_t)((float)block_xyz[3 * i + 1] - mn[1]) / 32u;
        const uint32_t bz = (uint32_t)((float)block_xyz[3 * i + 2] - mn[2]) / 32u;
        s->table[((uint64_t)bz * s->B + by) * s->B + bx] = i + 1;
        for (uint32_t k = 0; (s->B >> k) >= 1 && k < 16; k++)
        {
            const uint64_t m = s->B >> k;
            const uint64_t idx = ((uint64_t)(bz >> k) * m + (by >> k)) * m + (bx >> k);
            s->occ[s->occ_off[k] + idx / 32] |= 1u << (idx % 32);
            if (m == 1) break;
        }
    }
    return s;
}

void oracle_svo_close(void* h)
{
    osvo* s = (osvo*)h;
    if (!s) return;
    free(s->table); free(s->words); free(s->mats); free(s->occ); free(s->sub); free(s);
}

static inline float level_size(const osvo* s, uint32_t li) { return (float)(1u << s->lg[li]); }
static inline int32_t level_cells(const osvo* s, uint32_t li) { return (int32_t)(1u << (s->L - s->lg[li])); }

static int occupied(const osvo* s, uint32_t li, const int32_t c[3])
{
    const uint32_t g = s->lg[li];
    if (g < 5)
    {
        const uint32_t sh = 5u - g;
        const uint32_t bx = (uint32_t)c[0] >> sh, by = (uint32_t)c[1] >> sh, bz = (uint32_t)c[2] >> sh;
        const uint32_t tv = s->table[((uint64_t)bz * s->B + by) * s->B + bx];
        if (!tv) return 0;
        const uint32_t m = 32u >> g, mk = m - 1u;
        const uint32_t v = (((uint32_t)c[2] & mk) * m + ((uint32_t)c[1] & mk)) * m + ((uint32_t)c[0] & mk);
        const uint32_t* w = g == 0 ? &s->words[(uint64_t)(tv - 1) * 1024u]
                          : &s->sub[(uint64_t)(tv - 1) * 32u + (g == 3 ? 16u : 0u)];
        return (w[v / 32u] >> (v % 32u)) & 1u;
    }
    const uint32_t k = g - 5u;
    const uint64_t m = s->B >> k;
    const uint64_t idx = ((uint64_t)c[2] * m + (uint64_t)c[1]) * m + (uint64_t)c[0];
    return (s->occ[s->occ_off[k] + idx / 32] >> (idx % 32)) & 1u;
}

static uint16_t material_at(const osvo* s, const int32_t c[3])
{
    if (!s->mats) return 0;
    const uint32_t bx = (uint32_t)c[0] >> 5, by = (uint32_t)c[1] >> 5, bz = (uint32_t)c[2] >> 5;
    const uint32_t tv = s->table[((uint64_t)bz * s->B + by) * s->B + bx];
    if (!tv) return 0;
    const uint32_t v = ((uint32_t)c[2] & 31u) * 1024u + ((uint32_t)c[1] & 31u) * 32u + ((uint32_t)c[0] & 31u);
    return s->mats[(uint64_t)(tv - 1) * 32768u + v];
}

/* cell index of coordinate p at a level: floor(p / size), a point exactly on
 * a cell face belongs to the cell the ray moves into, clamped to [lo, hi] */
static inline int32_t cell_at(float p, float inv_size, int32_t step, int32_t lo, int32_t hi)
{
    const float x = p * inv_size;
    float f = floorf(x);
    if (step < 0 && x == f) f = f - 1.0f;
    int32_t c = (int32_t)f;
    if (f < (float)lo) c = lo;
    if (f > (float)hi) c = hi;
    return c;
}

/*
 * Traverses one ray (world origin o, direction d).  Returns 1 on hit (t =
 * entry distance in units of |d|, c = grid voxel, *axis = face axis crossed
 * or -1 when the origin is inside the voxel), 0 on a miss, -1 when the step
 * budget ran out (treated as a miss by callers).  *steps = steps used.
 */
int oracle_trace(const void* h, const float o[3], const float d[3], uint32_t max_steps, float* out_t,
                 int32_t out_c[3], int32_t* out_axis, uint32_t* out_steps)
{
    const osvo* s = (const osvo*)h;
    const float E = (float)(1u << s->L);
    float og[3], inv[3];
    int32_t st[3];
    for (int a = 0; a < 3; a++)
    {
        og[a] = o[a] - s->mn[a];
        st[a] = d[a] > 0.0f ? 1 : d[a] < 0.0f ? -1 : 0;
        inv[a] = st[a] ? 1.0f / d[a] : 0.0f;
    }
    *out_steps = 0;
    if (!st[0] && !st[1] && !st[2]) return 0;
    /* slab test against the SVO cube [0, E]^3 */
    float t0 = OR_F32_MIN, t1 = OR_F32_MAX;
    int32_t entry_axis = -1;
    for (int a = 0; a < 3; a++)
    {
        if (!st[a])
        {
            if (og[a] < 0.0f || og[a] >= E) return 0;
            continue;
        }
        const float ta = (0.0f - og[a]) * inv[a];
        const float tb = (E - og[a]) * inv[a];
        const float tn = ta < tb ? ta : tb;
        const float tf = ta < tb ? tb : ta;
        if (tn > t0) { t0 = tn; entry_axis = a; }
        if (tf < t1) t1 = tf;
    }
    float t = t0 > 0.0f ? t0 : 0.0f;
    if (!(t < t1)) return 0;
    int32_t last_axis = t0 > 0.0f ? entry_axis : -1;

    uint32_t li = s->NL - 1;
    int32_t c[3];
    {
        const float isz = 1.0f / level_size(s, li);
        const int32_t hi = level_cells(s, li) - 1;
        for (int a = 0; a < 3; a++) c[a] = cell_at(og[a] + t * d[a], isz, st[a], 0, hi);
    }
    uint32_t steps = 0;
    while (steps < max_steps)
    {
        steps++;
        if (occupied(s, li, c))
        {
            if (li == 0)
            {
                *out_t = t;
                out_c[0] = c[0]; out_c[1] = c[1]; out_c[2] = c[2];
                *out_axis = last_axis;
                *out_steps = steps;
                return 1;
            }
            const uint32_t shift = s->lg[li] - s->lg[li - 1];
            li--;
            const float isz = 1.0f / level_size(s, li);
            for (int a = 0; a < 3; a++)
            {
                const int32_t lo = c[a] << shift, hi = lo + (1 << shift) - 1;
                c[a] = cell_at(og[a] + t * d[a], isz, st[a], lo, hi);
            }
            continue;
        }
        const float size = level_size(s, li);
        float tn[3];
        for (int a = 0; a < 3; a++)
            tn[a] = st[a] > 0 ? ((float)(c[a] + 1) * size - og[a]) * inv[a]
                  : st[a] < 0 ? ((float)c[a] * size - og[a]) * inv[a] : OR_F32_MAX;
        int32_t am = 0;
        if (tn[1] < tn[am]) am = 1;
        if (tn[2] < tn[am]) am = 2;
        if (tn[am] > t) t = tn[am];
        last_axis = am;
        int32_t prev = c[am];
        c[am] += st[am];
        if (c[am] < 0 || c[am] >= level_cells(s, li)) { *out_steps = steps; return 0; }
        int32_t cur = c[am];
        /* the step left the parent cell: ascend to the level whose parent it stayed in */
        while (li < s->NL - 1)
        {
            const uint32_t shift = s->lg[li + 1] - s->lg[li];
            if ((prev >> shift) == (cur >> shift)) break;
            prev >>= shift; cur >>= shift;
            c[0] >>= shift; c[1] >>= shift; c[2] >>= shift;
            li++;
        }
    }
    *out_steps = steps;
    return -1;
}

/* batch form for tests: out_t = FLT max on miss */
void oracle_trace_batch(const void* h, uint32_t n, const float* o, const float* d, uint32_t max_steps, float* out_t,
                        int32_t* out_voxel, int32_t* out_axis, uint32_t* out_steps)
{
    const osvo* s = (const osvo*)h;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; i++)
    {
        float t;
        int32_t c[3], ax;
        uint32_t stp;
        const int r = oracle_trace(h, &o[3 * i], &d[3 * i], max_steps, &t, c, &ax, &stp);
        out_steps[i] = stp;
        if (r == 1)
        {
            out_t[i] = t;
            for (int a = 0; a < 3; a++) out_voxel[3 * i + a] = c[a] + (int32_t)s->mn[a];
            out_axis[i] = ax;
        }
        else
        {
            out_t[i] = OR_F32_MAX;
            out_voxel[3 * i] = out_voxel[3 * i + 1] = out_voxel[3 * i + 2] = 0;
            out_axis[i] = r == -1 ? -2 : -1;
        }
    }
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10                                                       */
/* ------------------------------------------------------------------ */

static inline void philox(uint32_t ctr[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; r++)
    {
        const uint64_t p0 = (uint64_t)0xD2511F53u * ctr[0];
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * ctr[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ ctr[1] ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ ctr[3] ^ k1;
        ctr[1] = (uint32_t)p1;
        ctr[3] = (uint32_t)p0;
        ctr[0] = n0;
        ctr[2] = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

void oracle_philox(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4])
{
    uint32_t c[4] = { in[0], in[1], in[2], in[3] };
    philox(c, k0, k1);
    memcpy(out, c, sizeof(c));
}

static inline float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

/* ------------------------------------------------------------------ */
/* GI                                                                  */
/* ------------------------------------------------------------------ */

typedef struct
{
    uint32_t spp, bounces, max_steps, frame;
    uint64_t seed;
    float    sun_dir[3];      /* unit vector toward the sun */
    float    sun_radiance[3];
    float    sky_radiance[3];
    float    offset;          /* ray origin offset along the normal, voxels */
} ogi_params;

#define OR_INV_PI 0.318309886f

/*
 * sin and cos on [-pi/4, pi/4] from their Taylor series (degree 7 and 8),
 * Horner form in binary32; only + and * so every platform rounds alike.
 */
static inline float sin_q(float x)
{
    const float x2 = x * x;
    return x * (1.0f + x2 * (-0.16666667f + x2 * (0.0083333333f + x2 * -0.00019841270f)));
}
static inline float cos_q(float x)
{
    const float x2 = x * x;
    return 1.0f + x2 * (-0.5f + x2 * (0.041666668f + x2 * (-0.0013888889f + x2 * 0.000024801587f)));
}

/*
 * Cosine-weighted direction about unit n for sample `sample` of a pixel (or
 * training point) `key`: randomised quasi-Monte Carlo.  The 2D point is the
 * R2 sequence (Roberts 2018, plastic-number additive recurrence, in 32-bit
 * fixed point) at index `sample`, rotated (Cranley-Patterson) by Philox
 * counter (key, bounce, frame, tag); it is mapped to the unit disk by the
 * concentric map of Shirley and Chiu (1997), lifted to the hemisphere
 * (Malley) and expressed in the orthonormal basis of Duff et al. (2017).
 */
static void sample_cosine(const float n[3], uint32_t key, uint32_t sample, uint32_t bounce, const ogi_params* p,
                          float out[3])
{
    const float sign = n[2] >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sign + n[2]);
    const float b = n[0] * n[1] * a;
    const float t1[3] = { 1.0f + sign * n[0] * n[0] * a, sign * b, -sign * n[0] };
    const float t2[3] = { b, sign + n[1] * n[1] * a, -n[1] };
    uint32_t c[4] = { key, bounce, p->frame, 0x52325351u };
    philox(c, (uint32_t)p->seed, (uint32_t)(p->seed >> 32));
    const uint32_t qx = sample * 3242174889u + c[0];
    const uint32_t qy = sample * 2447445413u + c[1];
    const float u = 2.0f * u01(qx) - 1.0f;
    const float v = 2.0f * u01(qy) - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (fabsf(u) > fabsf(v))
    {
        const float phi = 0.78539819f * (v / u);
        dx = u * cos_q(phi);
        dy = u * sin_q(phi);
    }
    else if (v != 0.0f)
    {
        const float phi = 0.78539819f * (u / v);
        dx = v * sin_q(phi);
        dy = v * cos_q(phi);
    }
    const float r2 = dx * dx + dy * dy;
    const float z = r2 < 1.0f ? sqrtf(1.0f - r2) : 0.0f;
    for (int i = 0; i < 3; i++) out[i] = dx * t1[i] + dy * t2[i] + z * n[i];
}

/* test hook: the sampler above for n directions of one key */
void oracle_sample_cosine(const float n[3], uint32_t key, uint32_t first_sample, uint32_t count, uint32_t bounce,
                          const void* params, float* out)
{
    for (uint32_t k = 0; k < count; k++) sample_cosine(n, key, first_sample + k, bounce, (const ogi_params*)params, &out[3 * k]);
}

static void svo_albedo(const osvo* s, const int32_t c[3], const tgx_material* luts, float out[3])
{
    const uint16_t code = material_at(s, c);
    if (!code || !luts) { out[0] = out[1] = out[2] = 0.5f; return; }
    const tgx_material* m = &luts[code - 1u];
    out[0] = m->albedo[0]; out[1] = m->albedo[1]; out[2] = m->albedo[2];
}

/* sun light arriving at a surface point (origin already offset) with normal n and albedo a */
static void direct_sun(const osvo* s, const float o2[3], const float n[3], const float a[3], const ogi_params* p,
                       float out[3])
{
    out[0] = out[1] = out[2] = 0.0f;
    const float ndl = n[0] * p->sun_dir[0] + n[1] * p->sun_dir[1] + n[2] * p->sun_dir[2];
    if (!(ndl > 0.0f)) return;
    float t; int32_t c[3], ax; uint32_t stp;
    if (oracle_trace(s, o2, p->sun_dir, p->max_steps, &t, c, &ax, &stp) == 1) return;
    for (int i = 0; i < 3; i++) out[i] = a[i] * OR_INV_PI * p->sun_radiance[i] * ndl;
}

/*
 * Radiance arriving at o2 along w: a path of up to p->bounces bounces,
 * accumulated forward with its throughput T (v += T * D at every hit, T *= albedo
 * before the next bounce, v += T * sky when the path escapes).
 */
static void incoming(const osvo* s, const float o2[3], const float w[3], uint32_t pixel, uint32_t sample,
                     const tgx_material* luts, const ogi_params* p, float out[3])
{
    float v[3] = { 0.0f, 0.0f, 0.0f }, T[3] = { 1.0f, 1.0f, 1.0f };
    float o[3] = { o2[0], o2[1], o2[2] }, d[3] = { w[0], w[1], w[2] };
    for (uint32_t b = 0; b < p->bounces; b++)
    {
        float t; int32_t c[3], ax; uint32_t stp;
        if (oracle_trace(s, o, d, p->max_steps, &t, c, &ax, &stp) != 1)
        {
            for (int i = 0; i < 3; i++) v[i] = v[i] + T[i] * p->sky_radiance[i];
            break;
        }
        float n2[3] = { 0.0f, 0.0f, 0.0f };
        if (ax >= 0) n2[ax] = d[ax] > 0.0f ? -1.0f : 1.0f;
        else
        {
            int m = 0;
            if (fabsf(d[1]) > fabsf(d[m])) m = 1;
            if (fabsf(d[2]) > fabsf(d[m])) m = 2;
            n2[m] = d[m] > 0.0f ? -1.0f : 1.0f;
        }
        float a2[3], o3[3], D[3];
        svo_albedo(s, c, luts, a2);
        for (int i = 0; i < 3; i++) o3[i] = (o[i] + t * d[i]) + n2[i] * p->offset;
        direct_sun(s, o3, n2, a2, p, D);
        for (int i = 0; i < 3; i++) v[i] = v[i] + T[i] * D[i];
        if (b + 1 < p->bounces)
        {
            for (int i = 0; i < 3; i++) T[i] = T[i] * a2[i];
            sample_cosine(n2, pixel, sample, b + 1, p, d);
            o[0] = o3[0]; o[1] = o3[1]; o[2] = o3[2];
        }
    }
    out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
}

/* Primary surface of a visibility word (shading.frag:116-228): cluster-space
 * ray, voxel box hit and dominant-axis face normal rotated to world space. */
typedef struct
{
    float    depth;
    uint32_t ptr, voxel, ci, oi, mat_byte;
    int      box_hit;
    float    nw[3], dws[3], dn[3], te, albedo[3];
} surface;

static int decode_surface(const tgx_object* objects, const uint32_t* cluster_pointers, const uint32_t* c2o,
                          const uint8_t* material, const tgx_material* luts, const tgx_view* cam, uint64_t word,
                          uint32_t px, uint32_t py, surface* sf)
{
    const float fx = ((float)px + 0.5f) / (float)cam->width;
    const float fy = 1.0f - ((float)py + 0.5f) / (float)cam->height;
    sf->depth = (float)(word >> 40) / 16777215.0f;
    if (!(sf->depth < 1.0f)) return 0;
    const uint32_t ptr = (uint32_t)(word >> 9) & 2147483647u;
    const uint32_t voxel = (uint32_t)word & 511u;
    const uint32_t ci = cluster_pointers[ptr];
    const uint32_t oi = c2o[ci];
    sf->ptr = ptr; sf->voxel = voxel; sf->ci = ci; sf->oi = oi;
    const tgx_object* od = &objects[oi];
    /* shading.frag:147-181: the same ws2ms, origin and direction as the visibility pass */
    const uint32_t nx = od->n_cluster_pointers_per_dim[0], ny = od->n_cluster_pointers_per_dim[1];
    const uint32_t rel = ptr - od->first_cluster_pointer;
    const float offx = (float)((rel % nx) * 8u), offy = (float)(((rel / nx) % ny) * 8u), offz = (float)((rel / (nx * ny)) * 8u);
    const float half = 8.0f * 0.5f;
    float m0[16], m1[16], m2[16], m3[16], ws2ms[16];
    or_m4_translate(-od->translation[0], -od->translation[1], -od->translation[2], m0);
    or_m4_inverse(od->rotation, m1);
    or_m4_translate(half * (float)od->n_cluster_pointers_per_dim[0], half * (float)od->n_cluster_pointers_per_dim[1],
                    half * (float)od->n_cluster_pointers_per_dim[2], m2);
    or_m4_translate(-offx, -offy, -offz, m3);
    or_m4_mul(m3, m2, ws2ms);
    or_m4_mul(ws2ms, m1, ws2ms);
    or_m4_mul(ws2ms, m0, ws2ms);
    const float ow[4] = { cam->camera[0], cam->camera[1], cam->camera[2], 1.0f };
    float o4[4];
    or_m4_mulv4(ws2ms, ow, o4);
    float dws[4];
    for (int i = 0; i < 3; i++)
    {
        const float a = cam->ray_bl[i] * (1.0f - fy) + cam->ray_tl[i] * fy;
        const float b = cam->ray_br[i] * (1.0f - fy) + cam->ray_tr[i] * fy;
        dws[i] = a * (1.0f - fx) + b * fx;
        sf->dws[i] = dws[i];
    }
    dws[3] = 0.0f;
    float d4[4];
    or_m4_mulv4(ws2ms, dws, d4);
    const float mag = sqrtf(d4[0] * d4[0] + d4[1] * d4[1] + d4[2] * d4[2]);
    const float dm[3] = { d4[0] / mag, d4[1] / mag, d4[2] / mag };
    const float vmin[3] = { (float)(voxel % 8u), (float)((voxel / 8u) % 8u), (float)(voxel / 64u) };
    const float vmax[3] = { vmin[0] + 1.0f, vmin[1] + 1.0f, vmin[2] + 1.0f };
    float enter, exit_;
    sf->nw[0] = sf->nw[1] = sf->nw[2] = 0.0f;
    sf->box_hit = or_ray_aabb(o4, dm, vmin, vmax, &enter, &exit_);
    if (sf->box_hit)
    {
        /* shading.frag:195-228 */
        float hm[3], nm[3];
        for (int i = 0; i < 3; i++) hm[i] = enter > 0.0f ? o4[i] + enter * dm[i] : o4[i];
        for (int i = 0; i < 3; i++) nm[i] = hm[i] - (vmin[i] + 0.5f);
#define SGN(v) ((v) > 0.0f ? 1.0f : (v) < 0.0f ? -1.0f : 0.0f)
        if (fabsf(nm[0]) > fabsf(nm[1]))
        {
            nm[1] = 0.0f;
            if (fabsf(nm[0]) > fabsf(nm[2])) { nm[0] = SGN(nm[0]); nm[2] = 0.0f; }
            else { nm[2] = SGN(nm[2]); nm[0] = 0.0f; }
        }
        else
        {
            nm[0] = 0.0f;
            if (fabsf(nm[1]) > fabsf(nm[2])) { nm[1] = SGN(nm[1]); nm[2] = 0.0f; }
            else { nm[2] = SGN(nm[2]); nm[1] = 0.0f; }
        }
#undef SGN
        const float n4[4] = { nm[0], nm[1], nm[2], 0.0f };
        float r4[4];
        or_m4_mulv4(od->rotation, n4, r4);
        const float rl = sqrtf(r4[0] * r4[0] + r4[1] * r4[1] + r4[2] * r4[2]);
        if (rl > 0.0f) { sf->nw[0] = r4[0] / rl; sf->nw[1] = r4[1] / rl; sf->nw[2] = r4[2] / rl; }
    }
    const float dl = sqrtf(dws[0] * dws[0] + dws[1] * dws[1] + dws[2] * dws[2]);
    for (int i = 0; i < 3; i++) sf->dn[i] = dws[i] / dl;
    sf->te = sf->box_hit && enter > 0.0f ? enter : 0.0f;
    sf->albedo[0] = sf->albedo[1] = sf->albedo[2] = 0.5f;
    sf->mat_byte = material ? material[(uint64_t)ci * 512u + voxel] : 0u;
    if (material && luts)
    {
        const tgx_material* m = &luts[od->lut_idx * 256u + sf->mat_byte];
        sf->albedo[0] = m->albedo[0]; sf->albedo[1] = m->albedo[1]; sf->albedo[2] = m->albedo[2];
    }
    return 1;
}

/*
 * One pixel of plain GI.  The primary hit comes from the visibility word (as
 * shading.frag:116-228 decodes it); world hit point = camera + enter * the
 * normalised pixel ray.  Writes RGB.
 */
void oracle_gi_pixel(const void* svo, const tgx_object* objects, const uint32_t* cluster_pointers,
                     const uint32_t* c2o, const uint8_t* material, const tgx_material* luts, const tgx_view* cam,
                     const ogi_params* p, uint64_t word, uint32_t px, uint32_t py, float out[3])
{
    const osvo* s = (const osvo*)svo;
    surface sf;
    if (!decode_surface(objects, cluster_pointers, c2o, material, luts, cam, word, px, py, &sf))
    {
        out[0] = p->sky_radiance[0]; out[1] = p->sky_radiance[1]; out[2] = p->sky_radiance[2];
        return;
    }
    /* no voxel-box hit in cluster space: face the camera */
    float nw[3] = { sf.nw[0], sf.nw[1], sf.nw[2] };
    if (nw[0] == 0.0f && nw[1] == 0.0f && nw[2] == 0.0f) { nw[0] = -sf.dn[0]; nw[1] = -sf.dn[1]; nw[2] = -sf.dn[2]; }
    const float* a = sf.albedo;
    float o2[3];
    for (int i = 0; i < 3; i++) o2[i] = (cam->camera[i] + sf.te * sf.dn[i]) + nw[i] * p->offset;
    float L[3];
    direct_sun(s, o2, nw, a, p, L);
    const uint32_t pixel = py * cam->width + px;
    float acc[3] = { 0.0f, 0.0f, 0.0f };
    for (uint32_t smp = 0; smp < p->spp; smp++)
    {
        float w[3], li[3];
        sample_cosine(nw, pixel, smp, 0, p, w);
        incoming(s, o2, w, pixel, smp, luts, p, li);
        for (int i = 0; i < 3; i++) acc[i] = acc[i] + li[i];
    }
    const float inv_spp = 1.0f / (float)(p->spp ? p->spp : 1);
    for (int i = 0; i < 3; i++) out[i] = L[i] + a[i] * (acc[i] * inv_spp);
}

/* ------------------------------------------------------------------ */
/* shading pass (shading.frag:53-110, 285-336)                          */
/* ------------------------------------------------------------------ */

#define OR_PI 3.14159265358979323846f

static inline float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void normalize3(const float* v, float* out)
{
    const float l = sqrtf(dot3(v, v));
    out[0] = v[0] / l; out[1] = v[1] / l; out[2] = v[2] / l;
}
/* GLSL max(x, y) = x < y ? y : x, min(x, y) = y < x ? y : x */
static inline float gl_max(float x, float y) { return x < y ? y : x; }
static inline float gl_min(float x, float y) { return y < x ? y : x; }
static inline float clamp01(float x) { return gl_min(gl_max(x, 0.0f), 1.0f); }

static float ggx_distribution(float c_ndh, float roughness)
{
    const float a = roughness * roughness;
    const float a2 = a * a;
    float den = c_ndh * c_ndh * (a2 - 1.0f) + 1.0f;
    den = OR_PI * den * den;
    return a2 / den;
}
static float schlick_ggx(float n_dot_v, float roughness)
{
    const float r = roughness + 1.0f;
    const float k = (r * r) / 8.0f;
    return n_dot_v / (n_dot_v * (1.0f - k) + k);
}
/* pow(1 - u, 5) as (t t)(t t) t */
static float fresnel_schlick(float u, float roughness)
{
    const float fl = 1.0f - roughness;
    const float t = 1.0f - u;
    const float t2 = t * t;
    return fl + (1.0f - fl) * ((t2 * t2) * t);
}
static void tg_shade(const float* n, const float* v, const float* l, const float* diffuse_albedo,
                     const float* specular_albedo, float metallic, float roughness, float radiance, float* out)
{
    const float hv[3] = { v[0] + l[0], v[1] + l[1], v[2] + l[2] };
    float h[3];
    normalize3(hv, h);
    const float c_hdn = clamp01(dot3(h, n));
    const float c_ldn = clamp01(dot3(n, l));
    const float c_ndv = clamp01(dot3(n, v));
    const float d = ggx_distribution(c_hdn, roughness);
    const float f = fresnel_schlick(c_ndv, roughness);
    const float g = schlick_ggx(c_ldn, roughness) * schlick_ggx(c_ndv, roughness);
    const float dfg = d * f * g;
    const float den = 4.0f * c_ndv * c_ldn;
    const float q = dfg / gl_max(den, 0.001f);
    const float kd = (1.0f - f) * (1.0f - metallic);
    for (int i = 0; i < 3; i++)
    {
        const float spec = specular_albedo[i] * q;
        const float diff = (kd * diffuse_albedo[i]) / OR_PI;
        out[i] = ((diff + spec) * radiance) * c_ldn;
    }
}
/* MurmurHash3 finaliser (util.inc:47-56) */
static inline uint32_t hash_u32(uint32_t v)
{
    v ^= v >> 16; v *= 0x85ebca6bu; v ^= v >> 13; v *= 0xc2b2ae35u; v ^= v >> 16;
    return v;
}
static void hash_color(uint32_t v, float* out)
{
    const uint32_t h0 = hash_u32(v), h1 = hash_u32(h0), h2 = hash_u32(h1);
    out[0] = (float)h0 / 4294967295.0f; out[1] = (float)h1 / 4294967295.0f; out[2] = (float)h2 / 4294967295.0f;
}

/* one frame of the shading pass; out = W*H*4 floats (RGBA) */
void oracle_shade_render(const tgx_object* objects, const uint32_t* cluster_pointers, const uint32_t* c2o,
                         const uint8_t* material, const tgx_material* luts, const tgx_view* cam, const uint64_t* visbuf,
                         uint32_t mode, float* out)
{
    for (uint32_t py = 0; py < cam->height; py++)
        for (uint32_t px = 0; px < cam->width; px++)
        {
            const uint64_t pixel = (uint64_t)py * cam->width + px;
            float* o = &out[4 * pixel];
            surface sf;
            o[3] = 1.0f;
            if (!decode_surface(objects, cluster_pointers, c2o, material, luts, cam, visbuf[pixel], px, py, &sf))
            {
                o[0] = 1.0f; o[1] = 0.0f; o[2] = 1.0f;
                continue;
            }
            switch (mode)
            {
            case 1: hash_color(sf.oi, o); break;
            case 2: o[0] = o[1] = o[2] = gl_min(1.0f, 8.0f * sf.depth); break;
            case 3: case 5: hash_color(sf.ci, o); break;
            case 4: hash_color(sf.voxel, o); break;
            case 6: hash_color(sf.mat_byte, o); break;
            case 7: o[0] = sf.albedo[0]; o[1] = sf.albedo[1]; o[2] = sf.albedo[2]; break;
            case 8: for (int i = 0; i < 3; i++) o[i] = sf.nw[i] * 0.5f + 0.5f; break;
            default:
            {
                const float metallic = 0.1f, roughness = 0.8f, radiance = 3.0f;
                const float white[3] = { 1.0f, 1.0f, 1.0f };
                const float* albedo = mode == 9 ? white : sf.albedo;
                const float dm = sf.depth * cam->far_plane;
                float vv[3], v[3], l[3], spec[3], lo[3];
                for (int i = 0; i < 3; i++) vv[i] = cam->camera[i] - (cam->camera[i] + dm * sf.dws[i]);
                normalize3(vv, v);
                const float l0[3] = { 0.0f, 0.8f, 0.3f };
                normalize3(l0, l);
                for (int i = 0; i < 3; i++) spec[i] = 0.04f * (1.0f - metallic) + albedo[i] * metallic;
                tg_shade(sf.nw, v, l, albedo, spec, metallic, roughness, radiance, lo);
                for (int i = 0; i < 3; i++) o[i] = 0.1f * albedo[i] + lo[i];
            }
            }
        }
}

/* whole frame (rows [row0, row1)); out = W*H*3 floats */
void oracle_gi_render(const void* svo, const tgx_object* objects, const uint32_t* cluster_pointers, const uint32_t* c2o,
                      const uint8_t* material, const tgx_material* luts, const tgx_view* cam, const ogi_params* p,
                      const uint64_t* visbuf, float* out, uint32_t row0, uint32_t row1, int n_threads)
{
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    const uint32_t W = cam->width;
    if (row1 > cam->height) row1 = cam->height;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t y = row0; y < (int64_t)row1; y++)
        for (uint32_t x = 0; x < W; x++)
        {
            const uint64_t i = (uint64_t)y * W + x;
            oracle_gi_pixel(svo, objects, cluster_pointers, c2o, material, luts, cam, p, visbuf[i], x, (uint32_t)y,
                            &out[3 * i]);
        }
}
