// svo_trace.cuh -- hierarchical DDA through the one-bit SVO (device side).
//
// The reference traverses its pointer octree with a 5-deep stack and a 32^3
// leaf DDA (svo_functions.inc:1-329, CPU form tg_sparse_voxel_octree.c:558-740).
// Here the same voxel set is traversed over the occupancy levels of the new
// storage: cells of 2^g voxels for g = L-1, ..., 9, 7, 5 (every other level
// of the block pyramid), g = 3 and 2 (sub-block masks of each 32^3 block),
// then single voxels.  An occupied cell is entered (descend), an empty one is
// left through its nearest face (one step), and leaving the parent cell
// ascends.  The operations are exactly rounded, in the order of the CPU
// oracle (oracle/oracle_gi.c: oracle_trace), so hits, distances and face
// normals are bit-identical.
#pragma once

#include "tgx_internal.cuh"

struct SvoDev
{
    float mn[3];
    uint32_t L, B, NL;
    const uint32_t* table;
    const uint32_t* pool;
    const uint32_t* sub;     // per slot 32 words: 4^3-cell mask (0-15), 8^3-cell mask (16-17)
    const uint32_t* occ;
    const uint16_t* mat;
    uint32_t occ_off[16];    // word offset of each pyramid level (level 0 = 32^3 blocks), zero padded
};

// log2 of the cell size of traversal level li: 0, 2, 3, 5, 7, 9, ... capped at L-1
__host__ __device__ __forceinline__ uint32_t svo_level_log2(uint32_t L, uint32_t li)
{
    return li == 0 ? 0u : li <= 2 ? li + 1u : min(2u * li - 1u, L - 1u);
}

__host__ __device__ __forceinline__ uint32_t svo_n_levels(uint32_t L)
{
    uint32_t n = 4;
    while (svo_level_log2(L, n - 1) < L - 1) n++;
    return n;
}

// byte offset, after the pyramid words, of the device copy of the level offsets (16-byte aligned)
inline uint64_t svo_occ_off_bytes(uint64_t occ_words) { return (occ_words * 4 + 15) & ~(uint64_t)15; }

inline SvoDev svo_dev(const tgx_svo* s)
{
    SvoDev d;
    d.mn[0] = s->mn[0]; d.mn[1] = s->mn[1]; d.mn[2] = s->mn[2];
    d.L = s->L; d.B = s->B; d.NL = svo_n_levels(s->L);
    d.table = s->d_table; d.pool = s->d_pool; d.sub = s->d_sub; d.occ = s->d_occ; d.mat = s->d_mat;
    for (int i = 0; i < 16; i++) d.occ_off[i] = i < 10 ? (uint32_t)s->occ_off[i] : 0u;
    return d;
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

// The cell of coordinate p at cells of size 1/inv_size, a point on a cell
// border going to the lower cell when the ray steps down, clamped to
// [lo, hi].  For |x| < 2^30 (always, for rays inside the cube) the floor is an
// exact integer and the clamp is done on integers; NaN and larger values take
// the float form, whose results the integer form equals wherever both apply.
__device__ __forceinline__ int32_t svo_cell_at(float p, float inv_size, int32_t step, int32_t lo, int32_t hi)
{
    const float x = xmul(p, inv_size);
    float f = floorf(x);
    if (fabsf(x) < 1073741824.0f) {
        const int32_t c = (int32_t)f - ((step < 0 && x == f) ? 1 : 0);
        return min(max(c, lo), hi);
    }
    if (step < 0 && x == f) f = xsub(f, 1.0f);
    int32_t c = (int32_t)f;
    if (f < (float)lo) c = lo;
    if (f > (float)hi) c = hi;
    return c;
}

// Resumable traversal state: the DDA of one ray, kept in registers so a
// persistent kernel can run it a few steps at a time.
struct RayState
{
    float og[3], d[3], inv[3];
    int32_t st[3];
    float t;
    int32_t c[3];
    int32_t last_axis;
    uint32_t li, steps;       // level (its cell size: svo_level_log2), steps used
    uint32_t tv;              // slot + 1 of the 32^3 block the sub-block levels (g < 5) are inside
};

constexpr int kTraceRunning = -2;

// One traversal level, for the step loop: where its occupancy bits are and
// how a cell's coordinates index them, so a step looks them up instead of
// deriving them from the level's log2 size each time.  Built per launch in
// shared memory (svo_level_tables).
struct alignas(16) LevelDesc
{
    const uint32_t* base;   // occupancy words: the pyramid level (g >= 5), or those of block slot 1 (g < 5)
    uint32_t stride;        // words per block slot (g < 5; the cell's words are base + (tv - 1) * stride), else 0
    uint32_t m;             // cells per axis of the indexed array
    uint32_t mk;            // coordinate mask (all ones above g = 5)
    uint32_t g;             // log2 of the cell size
    uint32_t sh_c;          // g minus the log2 cell size one level down (0 at li = 0)
    float inv_child;        // 2^-(log2 cell size one level down), exact
    float size;             // 2^g, exact
    uint32_t pad[3];
};
constexpr uint32_t kFirstLevelSize = 48;   // first_level[need]: need = g + the bit length of a coordinate step

// Fills lv[0 .. 15] and first_level[0 .. kFirstLevelSize) for SVO s, threads
// 0 .. kFirstLevelSize - 1 of the block; occ_off: the pyramid level offsets
// (a copy in shared memory, or s.occ_off); the caller synchronises.
// first_level[k] is the first traversal level whose cells have log2 size >= k,
// or NL when none below the root does (k > L - 1).
__device__ __forceinline__ void svo_level_tables(const uint32_t L, const uint32_t NL, const uint32_t B,
                                                 const uint32_t* occ, const uint32_t* pool, const uint32_t* sub,
                                                 const uint32_t* occ_off, LevelDesc* lv, uint8_t* first_level)
{
    const uint32_t i = threadIdx.x;
    if (i < 16u) {
        LevelDesc d = {};
        if (i < NL) {
            const uint32_t g = svo_level_log2(L, i);
            const uint32_t g_c = svo_level_log2(L, i ? i - 1u : 0u);
            d.g = g;
            d.sh_c = g - g_c;
            d.inv_child = __int_as_float((int)((127u - g_c) << 23));
            d.size = (float)(1u << g);
            if (g >= 5u) {
                d.base = occ + occ_off[(g - 5u) & 15u];
                d.stride = 0u;
                d.m = B >> (g - 5u);
                d.mk = 0xffffffffu;
            } else {
                d.base = g == 0u ? pool : sub + (g == 3u ? 16u : 0u);
                d.stride = g == 0u ? 1024u : 32u;
                d.m = 32u >> g;
                d.mk = d.m - 1u;
            }
        }
        lv[i] = d;
    }
    if (i < kFirstLevelSize) {
        uint32_t f = NL;
        if (i <= L - 1u)
            for (uint32_t li = 0; li < NL; li++)
                if (svo_level_log2(L, li) >= i) { f = li; break; }
        first_level[i] = (uint8_t)f;
    }
}

// Occupancy bit of cell c (grid coordinates at log2 size g); tv is the slot +
// 1 of the 32^3 block holding c, needed below the block level (g < 5).
__device__ __forceinline__ bool svo_occupied(const SvoDev& s, const uint32_t* occ_off, uint32_t g, const int32_t c[3],
                                             uint32_t tv)
{
    const bool sub = g < 5u;
    const uint32_t m = sub ? (32u >> g) : (s.B >> (g - 5u));
    const uint32_t mk = sub ? m - 1u : 0xffffffffu;
    const uint32_t v = (((uint32_t)c[2] & mk) * m + ((uint32_t)c[1] & mk)) * m + ((uint32_t)c[0] & mk);
    const uint32_t* base = !sub ? s.occ + occ_off[(g - 5u) & 15u]
                         : g == 0 ? s.pool + (uint64_t)(tv - 1u) * 1024u
                                  : s.sub + (uint64_t)(tv - 1u) * 32u + (g == 3 ? 16u : 0u);
    return (__ldg(&base[v >> 5]) >> (v & 31u)) & 1u;
}

// Sets up a ray.  Returns kTraceRunning when the DDA has to run, else the
// result (0: the ray misses the SVO cube or has no direction; 1: the entry
// voxel is set).
//
// The DDA starts where the top-down descent from the root would first find an
// empty cell, found bottom-up instead: the entry point's voxel, then its
// ancestors (the cell of every level that holds the point is the voxel's
// coordinates shifted right, with the same boundary rule) until an occupied
// one.  The descent's iterations are counted into r.steps as if they had
// run, so every result and the step budget stay those of the top-down walk.
// occ_off: the pyramid level offsets (shared memory in the persistent kernel).
__device__ __forceinline__ int svo_trace_begin(const SvoDev& s, const uint32_t* occ_off, const LevelDesc* lv,
                                               const float o[3], const float d[3], uint32_t max_steps, RayState& r)
{
    const float E = (float)(1u << s.L);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        r.d[a] = d[a];
        r.og[a] = xsub(o[a], s.mn[a]);
        r.st[a] = d[a] > 0.0f ? 1 : d[a] < 0.0f ? -1 : 0;
        r.inv[a] = r.st[a] ? xdiv(1.0f, d[a]) : 0.0f;
    }
    r.steps = 0;
    if (!r.st[0] && !r.st[1] && !r.st[2]) return 0;
    float t0 = F32_MIN_TG, t1 = F32_MAX_TG;
    int32_t entry_axis = -1;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (!r.st[a]) {
            if (r.og[a] < 0.0f || r.og[a] >= E) return 0;
            continue;
        }
        const float ta = xmul(xsub(0.0f, r.og[a]), r.inv[a]);
        const float tb = xmul(xsub(E, r.og[a]), r.inv[a]);
        const float tn = ta < tb ? ta : tb;
        const float tf = ta < tb ? tb : ta;
        if (tn > t0) { t0 = tn; entry_axis = a; }
        if (tf < t1) t1 = tf;
    }
    r.t = t0 > 0.0f ? t0 : 0.0f;
    if (!(r.t < t1)) return 0;
    r.last_axis = t0 > 0.0f ? entry_axis : -1;
    r.li = s.NL - 1;
    r.tv = 0;
    if (max_steps < s.NL) {   // the budget could run out inside the descent: run it
        const uint32_t g_root = s.L - 1u;
        const float isz = __int_as_float((int)((127u - g_root) << 23));
        const int32_t hi = (1 << (s.L - g_root)) - 1;
#pragma unroll
        for (int a = 0; a < 3; a++) r.c[a] = svo_cell_at(xadd(r.og[a], xmul(r.t, r.d[a])), isz, r.st[a], 0, hi);
        return kTraceRunning;
    }
    int32_t cv[3];
    const int32_t vhi = (1 << s.L) - 1;
#pragma unroll
    for (int a = 0; a < 3; a++) cv[a] = svo_cell_at(xadd(r.og[a], xmul(r.t, r.d[a])), 1.0f, r.st[a], 0, vhi);
    const uint32_t tv = __ldg(&s.table[((uint64_t)(cv[2] >> 5) * s.B + (uint64_t)(cv[1] >> 5)) * s.B + (uint64_t)(cv[0] >> 5)]);
    // coarsest empty level holding the point (-1: the voxel itself is set): the
    // levels below the lowest occupied one.  All levels' bits are loaded at once
    // (at most 8 levels for L <= 14) rather than one level per dependent step.
    uint32_t occ_mask = 0;
#pragma unroll
    for (uint32_t li = 0; li < 8u; li++) {
        if (li >= s.NL) break;   // the same in every lane
        const LevelDesc& ld = lv[li];
        const uint32_t g = ld.g;
        if (g < 5u && tv == 0u) continue;   // below an unallocated block: empty
        const uint32_t m = ld.m, mk = ld.mk;
        const uint32_t v = ((((uint32_t)cv[2] >> g) & mk) * m + (((uint32_t)cv[1] >> g) & mk)) * m +
                           (((uint32_t)cv[0] >> g) & mk);
        const uint32_t* base = ld.base + (uint64_t)(tv - 1u) * ld.stride;
        if ((__ldg(&base[v >> 5]) >> (v & 31u)) & 1u) occ_mask |= 1u << li;
    }
    const int32_t e = occ_mask ? __ffs((int)occ_mask) - 2 : (int32_t)s.NL - 1;
    if (e < 0) {   // the descent reaches the voxel: NL iterations, a hit
        r.steps = s.NL;
        r.li = 0;
        r.tv = tv;
        r.c[0] = cv[0]; r.c[1] = cv[1]; r.c[2] = cv[2];
        return 1;
    }
    r.li = (uint32_t)e;
    const uint32_t ge = svo_level_log2(s.L, (uint32_t)e);
    r.tv = ge < 5u ? tv : 0u;
    r.steps = s.NL - 1u - (uint32_t)e;
#pragma unroll
    for (int a = 0; a < 3; a++) r.c[a] = cv[a] >> ge;
    return kTraceRunning;
}

// Runs at most n loop iterations of the DDA (one iteration is one step of
// the max_steps budget).  Returns kTraceRunning, 1 on hit (r.t, r.c,
// r.last_axis), 0 on miss, -1 when max_steps ran out.  occ_off: the pyramid
// level offsets (shared memory in the persistent kernel).  Every iteration
// does one occupancy load and computes both the descent into the child cell
// and the step to the neighbour cell, then keeps one, so the lanes of a warp
// stay on one instruction stream whichever way their rays go.
__device__ __forceinline__ int svo_trace_run(const SvoDev& s, const LevelDesc* lv, const uint8_t* first_level,
                                             RayState& r, uint32_t max_steps, uint32_t n)
{
    for (uint32_t k = 0; k < n; k++) {
        if (r.steps >= max_steps) return -1;
        r.steps++;
        const LevelDesc& ld = lv[r.li & 15u];
        const uint32_t g = ld.g;
        // occupancy of the current cell
        const uint32_t m = ld.m, mk = ld.mk;
        const uint32_t v = (((uint32_t)r.c[2] & mk) * m + ((uint32_t)r.c[1] & mk)) * m + ((uint32_t)r.c[0] & mk);
        const uint32_t* base = ld.base + (uint64_t)(r.tv - 1u) * ld.stride;
        const bool occ = (__ldg(&base[v >> 5]) >> (v & 31u)) & 1u;
        if (occ && r.li == 0) return 1;
        // candidate 1: descend, the child cell by point location
        const uint32_t sh_c = ld.sh_c;
        const float isz = ld.inv_child;
        int32_t cd[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int32_t lo = r.c[a] << sh_c, hi = lo + (1 << sh_c) - 1;
            cd[a] = svo_cell_at(xadd(r.og[a], xmul(r.t, r.d[a])), isz, r.st[a], lo, hi);
        }
        // candidate 2: step through the nearest face
        const float size = ld.size;
        float tn[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            // the face the ray leaves through: c + 1 going up, c going down (one product chain per axis)
            const float face = (float)(r.c[a] + ((r.st[a] + 1) >> 1));
            const float tf = xmul(xsub(xmul(face, size), r.og[a]), r.inv[a]);
            tn[a] = r.st[a] != 0 ? tf : F32_MAX_TG;
        }
        const bool a1 = tn[1] < tn[0];
        const float t01 = a1 ? tn[1] : tn[0];
        const bool a2 = tn[2] < t01;
        const int32_t am = a2 ? 2 : a1 ? 1 : 0;
        const float tam = a2 ? tn[2] : t01;
        int32_t prev = a2 ? r.c[2] : a1 ? r.c[1] : r.c[0];
        const int32_t cur0 = prev + (a2 ? r.st[2] : a1 ? r.st[1] : r.st[0]);
        int32_t cs[3] = {am == 0 ? cur0 : r.c[0], am == 1 ? cur0 : r.c[1], am == 2 ? cur0 : r.c[2]};
        if (!occ && (cur0 < 0 || cur0 >= (1 << (s.L - g)))) return 0;
        // ascend to the level whose parent the step stayed in: the lowest level
        // li_u >= li whose parent (log2 size gp) holds both the old and the new
        // cell, i.e. gp > g + the highest bit in which their coordinates differ,
        // or the root level.  The same level the one-level-at-a-time climb
        // finds (checked exhaustively for L = 6..14), without a loop whose trip
        // count differs between the lanes of a warp.  Only taken for a step
        // that stays inside the cube (prev, cur0 >= 0).
        uint32_t li_u = r.li;
        const uint32_t diff = (uint32_t)(prev ^ cur0);
        if (diff) {
            const uint32_t need = g + 32u - (uint32_t)__clz((int)diff);   // the parent's log2 size must reach this
            const uint32_t lp = first_level[min(need, kFirstLevelSize - 1u)];   // first level that large, or NL
            li_u = min(s.NL - 1u, max(r.li, lp - 1u));
        }
        const uint32_t up = lv[li_u & 15u].g - g;
        cs[0] >>= up; cs[1] >>= up; cs[2] >>= up;
        // keep one candidate; entering a 32^3 block loads its slot
        const uint32_t tv_c = occ && g == 5u
            ? __ldg(&s.table[((uint64_t)r.c[2] * s.B + (uint64_t)r.c[1]) * s.B + (uint64_t)r.c[0]]) : r.tv;
        r.tv = tv_c;
        r.t = occ ? r.t : (tam > r.t ? tam : r.t);
        r.last_axis = occ ? r.last_axis : am;
        r.li = occ ? r.li - 1u : li_u;
#pragma unroll
        for (int a = 0; a < 3; a++) r.c[a] = occ ? cd[a] : cs[a];
    }
    return kTraceRunning;
}

// Whole-ray form.  Returns 1 on hit (t, grid voxel c, face axis or -1), 0 on
// miss, -1 when max_steps ran out.  lv, first_level: svo_level_tables.
static __device__ int svo_trace(const SvoDev& s, const LevelDesc* lv, const uint8_t* first_level, const float o[3],
                                const float d[3], uint32_t max_steps, float& out_t, int32_t out_c[3],
                                int32_t& out_axis, uint32_t& out_steps)
{
    RayState r;
    int res = svo_trace_begin(s, s.occ_off, lv, o, d, max_steps, r);
    if (res == kTraceRunning) res = svo_trace_run(s, lv, first_level, r, max_steps, 0xffffffffu);
    out_steps = r.steps;
    if (res == 1) {
        out_t = r.t;
        out_c[0] = r.c[0]; out_c[1] = r.c[1]; out_c[2] = r.c[2];
        out_axis = r.last_axis;
    }
    return res;
}
