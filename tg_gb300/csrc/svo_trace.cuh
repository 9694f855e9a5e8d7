// svo_trace.cuh -- hierarchical DDA through the one-bit SVO (device side).
//
// The reference traverses its pointer octree with a 5-deep stack and a 32^3
// leaf DDA (svo_functions.inc:1-329, CPU form tg_sparse_voxel_octree.c:558-740).
// Here the same voxel set is traversed over the occupancy pyramid of the new
// storage: cells of 2^k voxels for k = L-1 .. 5, then single voxels.  An
// occupied cell is entered (descend), an empty one is left through its
// nearest face (one step), and leaving the parent cell ascends.  The
// operations are exactly rounded, in the order of the CPU oracle
// (oracle/oracle_gi.c: oracle_trace), so hits, distances and face normals are
// bit-identical.
#pragma once

#include "tgx_internal.cuh"

struct SvoDev
{
    float mn[3];
    uint32_t L, B, NL;
    const uint32_t* table;
    const uint32_t* pool;
    const uint32_t* occ;
    const uint16_t* mat;
    uint64_t occ_off[10];
};

inline SvoDev svo_dev(const tgx_svo* s)
{
    SvoDev d;
    d.mn[0] = s->mn[0]; d.mn[1] = s->mn[1]; d.mn[2] = s->mn[2];
    d.L = s->L; d.B = s->B; d.NL = 1 + (s->L - 5);
    d.table = s->d_table; d.pool = s->d_pool; d.occ = s->d_occ; d.mat = s->d_mat;
    for (int i = 0; i < 10; i++) d.occ_off[i] = s->occ_off[i];
    return d;
}

__device__ __forceinline__ float svo_level_size(uint32_t li) { return li == 0 ? 1.0f : (float)(1u << (li + 4)); }
__device__ __forceinline__ int32_t svo_level_cells(const SvoDev& s, uint32_t li)
{
    return li == 0 ? (int32_t)(s.B << 5) : (int32_t)(s.B >> (li - 1));
}

__device__ __forceinline__ bool svo_occupied(const SvoDev& s, uint32_t li, int32_t cx, int32_t cy, int32_t cz)
{
    if (li == 0) {
        const uint32_t bx = (uint32_t)cx >> 5, by = (uint32_t)cy >> 5, bz = (uint32_t)cz >> 5;
        const uint32_t tv = __ldg(&s.table[((uint64_t)bz * s.B + by) * s.B + bx]);
        if (!tv) return false;
        const uint32_t v = ((uint32_t)cz & 31u) * 1024u + ((uint32_t)cy & 31u) * 32u + ((uint32_t)cx & 31u);
        return (__ldg(&s.pool[(uint64_t)(tv - 1) * 1024u + (v >> 5)]) >> (v & 31u)) & 1u;
    }
    const uint32_t k = li - 1;
    const uint64_t m = s.B >> k;
    const uint64_t idx = ((uint64_t)cz * m + (uint64_t)cy) * m + (uint64_t)cx;
    return (__ldg(&s.occ[s.occ_off[k] + (idx >> 5)]) >> (idx & 31u)) & 1u;
}

__device__ __forceinline__ uint32_t svo_material(const SvoDev& s, int32_t cx, int32_t cy, int32_t cz)
{
    if (!s.mat) return 0;
    const uint32_t bx = (uint32_t)cx >> 5, by = (uint32_t)cy >> 5, bz = (uint32_t)cz >> 5;
    const uint32_t tv = __ldg(&s.table[((uint64_t)bz * s.B + by) * s.B + bx]);
    if (!tv) return 0;
    const uint32_t v = ((uint32_t)cz & 31u) * 1024u + ((uint32_t)cy & 31u) * 32u + ((uint32_t)cx & 31u);
    return s.mat[(uint64_t)(tv - 1) * 32768u + v];
}

__device__ __forceinline__ int32_t svo_cell_at(float p, float inv_size, int32_t step, int32_t lo, int32_t hi)
{
    const float x = xmul(p, inv_size);
    float f = floorf(x);
    if (step < 0 && x == f) f = xsub(f, 1.0f);
    int32_t c = (int32_t)f;
    if (f < (float)lo) c = lo;
    if (f > (float)hi) c = hi;
    return c;
}

// Returns 1 on hit (t, grid voxel c, face axis or -1), 0 on miss, -1 when
// max_steps ran out.
static __device__ int svo_trace(const SvoDev& s, const float o[3], const float d[3], uint32_t max_steps, float& out_t,
                         int32_t out_c[3], int32_t& out_axis, uint32_t& out_steps)
{
    const float E = (float)(1u << s.L);
    float og[3], inv[3];
    int32_t st[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        og[a] = xsub(o[a], s.mn[a]);
        st[a] = d[a] > 0.0f ? 1 : d[a] < 0.0f ? -1 : 0;
        inv[a] = st[a] ? xdiv(1.0f, d[a]) : 0.0f;
    }
    out_steps = 0;
    if (!st[0] && !st[1] && !st[2]) return 0;
    float t0 = F32_MIN_TG, t1 = F32_MAX_TG;
    int32_t entry_axis = -1;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (!st[a]) {
            if (og[a] < 0.0f || og[a] >= E) return 0;
            continue;
        }
        const float ta = xmul(xsub(0.0f, og[a]), inv[a]);
        const float tb = xmul(xsub(E, og[a]), inv[a]);
        const float tn = ta < tb ? ta : tb;
        const float tf = ta < tb ? tb : ta;
        if (tn > t0) { t0 = tn; entry_axis = a; }
        if (tf < t1) t1 = tf;
    }
    float t = t0 > 0.0f ? t0 : 0.0f;
    if (!(t < t1)) return 0;
    int32_t last_axis = t0 > 0.0f ? entry_axis : -1;

    uint32_t li = s.NL - 1;
    int32_t c[3];
    {
        const float isz = xdiv(1.0f, svo_level_size(li));
        const int32_t hi = svo_level_cells(s, li) - 1;
#pragma unroll
        for (int a = 0; a < 3; a++) c[a] = svo_cell_at(xadd(og[a], xmul(t, d[a])), isz, st[a], 0, hi);
    }
    uint32_t steps = 0;
    while (steps < max_steps) {
        steps++;
        if (svo_occupied(s, li, c[0], c[1], c[2])) {
            if (li == 0) {
                out_t = t;
                out_c[0] = c[0]; out_c[1] = c[1]; out_c[2] = c[2];
                out_axis = last_axis;
                out_steps = steps;
                return 1;
            }
            const uint32_t shift = li == 1 ? 5u : 1u;
            li--;
            const float isz = xdiv(1.0f, svo_level_size(li));
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const int32_t lo = c[a] << shift, hi = lo + (1 << shift) - 1;
                c[a] = svo_cell_at(xadd(og[a], xmul(t, d[a])), isz, st[a], lo, hi);
            }
            continue;
        }
        const float size = svo_level_size(li);
        float tn[3];
#pragma unroll
        for (int a = 0; a < 3; a++)
            tn[a] = st[a] > 0 ? xmul(xsub(xmul((float)(c[a] + 1), size), og[a]), inv[a])
                  : st[a] < 0 ? xmul(xsub(xmul((float)c[a], size), og[a]), inv[a]) : F32_MAX_TG;
        int32_t am = 0;
        if (tn[1] < tn[am]) am = 1;
        if (tn[2] < tn[am]) am = 2;
        const float tam = am == 0 ? tn[0] : am == 1 ? tn[1] : tn[2];
        if (tam > t) t = tam;
        last_axis = am;
        int32_t prev = c[am];
        c[am] += st[am];
        const int32_t cur0 = c[am];
        if (cur0 < 0 || cur0 >= svo_level_cells(s, li)) { out_steps = steps; return 0; }
        int32_t cur = cur0;
        while (li < s.NL - 1) {
            const uint32_t shift = li == 0 ? 5u : 1u;
            if ((prev >> shift) == (cur >> shift)) break;
            prev >>= shift; cur >>= shift;
            c[0] >>= shift; c[1] >>= shift; c[2] >>= shift;
            li++;
        }
    }
    out_steps = steps;
    return -1;
}
