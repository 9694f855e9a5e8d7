/*
 * oracle_svo.c -- CPU oracle of the one-bit SVO build.
 *
 * TEST INFRASTRUCTURE.  A restatement of tg's CPU builder
 * tg/src/graphics/tg_sparse_voxel_octree.c:23-542 with the side length as a
 * parameter (the reference fixes it at 1024, :11 and :468-470) and without
 * the node encoding: the output is the set of non-empty 32^3 leaf blocks and
 * their bits, which is what the reference's voxel buffer holds.  The
 * recursion, the per-child OBB/AABB test (tg_physics.c:226-392), the
 * voxelisation's corner lerp (:242-315) and its 7-corner world AABB (:180-194
 * uses corner 2 twice and never corner 3) are kept operation for operation.
 * The object rotation is the m4 the reference builds with tgm_m4_angle_axis
 * (:25); callers pass it precomputed in tgx_object.rotation.
 *
 * New with respect to the reference (which keeps no per-voxel material in its
 * SVO): each set voxel also gets the material code (lut << 8 | byte) + 1 of
 * the largest code among the cluster samples that set it, for the bounce
 * lighting's albedo lookup.
 */
#include "oracle_common.h"

#include <stdlib.h>

#define CSIDE 8u
#define BLOCK 32u

typedef struct { float x, y, z; } ov3;

static ov3 v3_sub(ov3 a, ov3 b) { ov3 r = { a.x - b.x, a.y - b.y, a.z - b.z }; return r; }
static ov3 v3_neg(ov3 a) { ov3 r = { -a.x, -a.y, -a.z }; return r; }
static float v3_dot(ov3 a, ov3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static float v3_mag(ov3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
static ov3 v3_normalized(ov3 a) { const float m = v3_mag(a); ov3 r = { a.x / m, a.y / m, a.z / m }; return r; }
static ov3 v3_min(ov3 a, ov3 b) { ov3 r = { a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z }; return r; }
static ov3 v3_max(ov3 a, ov3 b) { ov3 r = { a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z }; return r; }

static ov3 mulv4_xyz(const float* m, float x, float y, float z, float w)
{
    const float v[4] = { x, y, z, w };
    float r[4];
    or_m4_mulv4(m, v, r);
    ov3 o = { r[0], r[1], r[2] };
    return o;
}

static void cluster_offset(const tgx_object* od, uint32_t rel, float off[3], float ohe[3])
{
    const uint32_t nx = od->n_cluster_pointers_per_dim[0], ny = od->n_cluster_pointers_per_dim[1];
    off[0] = (float)((rel % nx) * CSIDE);
    off[1] = (float)(((rel / nx) % ny) * CSIDE);
    off[2] = (float)((rel / (nx * ny)) * CSIDE);
    const float h = (float)(CSIDE / 2);
    ohe[0] = (float)od->n_cluster_pointers_per_dim[0] * h;
    ohe[1] = (float)od->n_cluster_pointers_per_dim[1] * h;
    ohe[2] = (float)od->n_cluster_pointers_per_dim[2] * h;
}

/* tg_world_space_to_cluster_model_space, tg_sparse_voxel_octree.c:23-60 */
void oracle_ws2ms(const tgx_object* od, uint32_t rel, float out[16])
{
    float off[3], ohe[3], m1[16], m2[16], m3[16], m4[16];
    cluster_offset(od, rel, off, ohe);
    or_m4_translate(-od->translation[0], -od->translation[1], -od->translation[2], m1);
    or_m4_inverse(od->rotation, m2);
    or_m4_translate(ohe[0], ohe[1], ohe[2], m3);
    or_m4_translate(-off[0], -off[1], -off[2], m4);
    or_m4_mul(m4, m3, out);
    or_m4_mul(out, m2, out);
    or_m4_mul(out, m1, out);
}

/* tg_cluster_model_space_to_world_space, tg_sparse_voxel_octree.c:62-100 */
void oracle_cs2ws(const tgx_object* od, uint32_t rel, float out[16])
{
    float off[3], ohe[3], m1[16], m2[16], m4[16];
    cluster_offset(od, rel, off, ohe);
    or_m4_translate(off[0], off[1], off[2], m1);
    or_m4_translate(-ohe[0], -ohe[1], -ohe[2], m2);
    or_m4_translate(od->translation[0], od->translation[1], od->translation[2], m4);
    or_m4_mul(m4, od->rotation, out);
    or_m4_mul(out, m2, out);
    or_m4_mul(out, m1, out);
}

/* tg_intersect_aabb_obb_ignore_contact, tg_physics.c:226-392 */
int oracle_aabb_obb(ov3 mn, ov3 mx, const ov3* c)
{
    int sep;
    sep = 1; for (int i = 0; i < 8; i++) sep &= c[i].x <= mn.x; if (sep) return 0;
    sep = 1; for (int i = 0; i < 8; i++) sep &= c[i].x >= mx.x; if (sep) return 0;
    sep = 1; for (int i = 0; i < 8; i++) sep &= c[i].y <= mn.y; if (sep) return 0;
    sep = 1; for (int i = 0; i < 8; i++) sep &= c[i].y >= mx.y; if (sep) return 0;
    sep = 1; for (int i = 0; i < 8; i++) sep &= c[i].z <= mn.z; if (sep) return 0;
    sep = 1; for (int i = 0; i < 8; i++) sep &= c[i].z >= mx.z; if (sep) return 0;

    const ov3 nxp = v3_normalized(v3_sub(c[1], c[0]));
    const ov3 nyp = v3_normalized(v3_sub(c[2], c[0]));
    const ov3 nzp = v3_normalized(v3_sub(c[4], c[0]));
    const ov3 nrm[6] = { v3_neg(nxp), nxp, v3_neg(nyp), nyp, v3_neg(nzp), nzp };
    const float l0 = v3_mag(c[0]);
    const float l1 = v3_mag(c[7]);
    const ov3 zero = { 0.0f, 0.0f, 0.0f };
    const ov3 n0 = l0 == 0.0f ? zero : (ov3){ c[0].x / l0, c[0].y / l0, c[0].z / l0 };
    const ov3 n1 = l1 == 0.0f ? zero : (ov3){ c[7].x / l1, c[7].y / l1, c[7].z / l1 };
    float dist[6];
    dist[0] = l0 * v3_dot(n0, nrm[0]);
    dist[1] = l1 * v3_dot(n1, nrm[1]);
    dist[2] = l0 * v3_dot(n0, nrm[2]);
    dist[3] = l1 * v3_dot(n1, nrm[3]);
    dist[4] = l0 * v3_dot(n0, nrm[4]);
    dist[5] = l1 * v3_dot(n1, nrm[5]);
    const ov3 pts[8] = {
        { mn.x, mn.y, mn.z }, { mx.x, mn.y, mn.z }, { mn.x, mx.y, mn.z }, { mx.x, mx.y, mn.z },
        { mn.x, mn.y, mx.z }, { mx.x, mn.y, mx.z }, { mn.x, mx.y, mx.z }, { mx.x, mx.y, mx.z } };
    for (int p = 0; p < 6; p++)
    {
        sep = 1;
        for (int k = 0; k < 8; k++)
        {
            const float dd = v3_dot(nrm[p], pts[k]) - dist[p];
            sep &= dd >= 0.0f;
            if (!sep) break;
        }
        if (sep) return 0;
    }
    return 1;
}

static uint32_t trim_u32(float v) { return v > 0.0f ? (uint32_t)v : 0u; }

typedef struct
{
    const tgx_object* objects;
    const uint32_t*   cluster_pointers;
    const uint32_t*   c2o;
    const uint32_t*   bits;
    const uint8_t*    material;   /* 512 per cluster, or NULL */
    /* output blocks */
    uint32_t  n, cap;
    uint64_t* keys;     /* block index */
    uint32_t* words;    /* 1024 per block */
    uint16_t* mats;     /* 32768 per block: (lut << 8 | byte) + 1 of the max contributor, 0 = none */
    float     mn[3];
    uint32_t  bpa;      /* blocks per axis */
    uint64_t  samples;  /* voxel-centre samples evaluated */
} svo_state;

/* tg__construct_leaf_node, tg_sparse_voxel_octree.c:102-317 (bits only) */
static void leaf(svo_state* st, ov3 pmin, ov3 pmax, uint32_t n, const uint32_t* cps)
{
    uint32_t words[BLOCK * BLOCK * BLOCK / 32];
    static _Thread_local uint16_t mats[BLOCK * BLOCK * BLOCK];
    memset(words, 0, sizeof(words));
    if (st->material) memset(mats, 0, sizeof(mats));
    int any = 0;
    const ov3 pext = v3_sub(pmax, pmin);
    const float ws[8][3] = {
        { pmin.x, pmin.y, pmin.z }, { pmax.x, pmin.y, pmin.z }, { pmin.x, pmax.y, pmin.z }, { pmax.x, pmax.y, pmin.z },
        { pmin.x, pmin.y, pmax.z }, { pmax.x, pmin.y, pmax.z }, { pmin.x, pmax.y, pmax.z }, { pmax.x, pmax.y, pmax.z } };
    const float e = (float)CSIDE;
    const float cs[8][3] = { { 0, 0, 0 }, { e, 0, 0 }, { 0, e, 0 }, { e, e, 0 }, { 0, 0, e }, { e, 0, e }, { 0, e, e }, { e, e, e } };
    for (uint32_t ci = 0; ci < n; ci++)
    {
        const uint32_t cp = cps[ci];
        const uint32_t cidx = st->cluster_pointers[cp];
        const tgx_object* od = &st->objects[st->c2o[cidx]];
        const uint32_t rel = cp - od->first_cluster_pointer;
        float cs2ws[16], ws2cs[16];
        oracle_cs2ws(od, rel, cs2ws);
        ov3 cw[8];
        for (int k = 0; k < 8; k++) cw[k] = mulv4_xyz(cs2ws, cs[k][0], cs[k][1], cs[k][2], 1.0f);
        const ov3 min_c = v3_min(v3_min(v3_min(cw[0], cw[1]), v3_min(cw[2], cw[2])), v3_min(v3_min(cw[4], cw[6]), v3_min(cw[5], cw[7])));
        const ov3 max_c = v3_max(v3_max(v3_max(cw[0], cw[1]), v3_max(cw[2], cw[2])), v3_max(v3_max(cw[4], cw[6]), v3_max(cw[5], cw[7])));
        const ov3 floor_min_c = { floorf(min_c.x), floorf(min_c.y), floorf(min_c.z) };
        const ov3 ceil_max_c = { ceilf(max_c.x), ceilf(max_c.y), ceilf(max_c.z) };
        or_m4_inverse(cs2ws, ws2cs);
        ov3 bc[8];
        for (int k = 0; k < 8; k++) bc[k] = mulv4_xyz(ws2cs, ws[k][0], ws[k][1], ws[k][2], 1.0f);
        const ov3 tmin = v3_max(pmin, floor_min_c);
        const ov3 tmax = v3_min(pmax, ceil_max_c);
        /* :228-233.  The reference asserts both ends lie in [0, extent]
         * (:221-226); its 7-corner AABB can miss the block while the OBB test
         * passed, and then (u32) of a negative float is undefined.  Defined
         * here as an empty range: a negative end clamps to 0. */
        const uint32_t x0 = trim_u32(tmin.x - pmin.x), y0 = trim_u32(tmin.y - pmin.y), z0 = trim_u32(tmin.z - pmin.z);
        const uint32_t x1 = trim_u32(tmax.x - pmin.x), y1 = trim_u32(tmax.y - pmin.y), z1 = trim_u32(tmax.z - pmin.z);
        const uint32_t coff = cidx * 512u;
        for (uint32_t bz = z0; bz < z1; bz++)
        {
            const float tz = ((float)bz + 0.5f) / pext.z;
            const float omtz = 1.0f - tz;
            const float pz0x = omtz * bc[0].x + tz * bc[4].x, pz0y = omtz * bc[0].y + tz * bc[4].y, pz0z = omtz * bc[0].z + tz * bc[4].z;
            const float pz1x = omtz * bc[1].x + tz * bc[5].x, pz1y = omtz * bc[1].y + tz * bc[5].y, pz1z = omtz * bc[1].z + tz * bc[5].z;
            const float pz2x = omtz * bc[2].x + tz * bc[6].x, pz2y = omtz * bc[2].y + tz * bc[6].y, pz2z = omtz * bc[2].z + tz * bc[6].z;
            const float pz3x = omtz * bc[3].x + tz * bc[7].x, pz3y = omtz * bc[3].y + tz * bc[7].y, pz3z = omtz * bc[3].z + tz * bc[7].z;
            for (uint32_t by = y0; by < y1; by++)
            {
                const float ty = ((float)by + 0.5f) / pext.y;
                const float omty = 1.0f - ty;
                const float py0x = omty * pz0x + ty * pz2x, py0y = omty * pz0y + ty * pz2y, py0z = omty * pz0z + ty * pz2z;
                const float py1x = omty * pz1x + ty * pz3x, py1y = omty * pz1y + ty * pz3y, py1z = omty * pz1z + ty * pz3z;
                for (uint32_t bx = x0; bx < x1; bx++)
                {
                    st->samples++;
                    const float tx = ((float)bx + 0.5f) / pext.x;
                    const float omtx = 1.0f - tx;
                    const float cx = omtx * py0x + tx * py1x;
                    if (cx < 0.0f || cx >= (float)CSIDE) continue;
                    const float cy = omtx * py0y + tx * py1y;
                    if (cy < 0.0f || cy >= (float)CSIDE) continue;
                    const float cz = omtx * py0z + tx * py1z;
                    if (cz < 0.0f || cz >= (float)CSIDE) continue;
                    const uint32_t vx = (uint32_t)cx, vy = (uint32_t)cy, vz = (uint32_t)cz;
                    const uint32_t rvi = CSIDE * CSIDE * vz + CSIDE * vy + vx;
                    const uint32_t cvi = coff + rvi;
                    if (st->bits[cvi / 32u] & (1u << (cvi % 32u)))
                    {
                        const uint32_t bvi = (uint32_t)(pext.x * pext.y * (float)bz + pext.x * (float)by + (float)bx);
                        words[bvi / 32u] |= 1u << (bvi % 32u);
                        any = 1;
                        if (st->material)
                        {
                            const uint16_t code = (uint16_t)(((od->lut_idx << 8) | st->material[(uint64_t)cidx * 512u + rvi]) + 1u);
                            if (code > mats[bvi]) mats[bvi] = code;
                        }
                    }
                }
            }
        }
    }
    if (!any) return;
    if (st->n == st->cap)
    {
        st->cap = st->cap ? 2 * st->cap : 64;
        st->keys = realloc(st->keys, (size_t)st->cap * sizeof(uint64_t));
        st->words = realloc(st->words, (size_t)st->cap * 4096);
        if (st->material) st->mats = realloc(st->mats, (size_t)st->cap * 65536);
    }
    const uint64_t bx = (uint64_t)((pmin.x - st->mn[0]) / (float)BLOCK);
    const uint64_t by = (uint64_t)((pmin.y - st->mn[1]) / (float)BLOCK);
    const uint64_t bz = (uint64_t)((pmin.z - st->mn[2]) / (float)BLOCK);
    st->keys[st->n] = (bz * st->bpa + by) * st->bpa + bx;
    memcpy(&st->words[(size_t)st->n * 1024], words, 4096);
    if (st->material) memcpy(&st->mats[(size_t)st->n * 32768], mats, 65536);
    st->n++;
}

/* tg__construct_inner_node, tg_sparse_voxel_octree.c:319-464 */
static void inner(svo_state* st, ov3 pmin, ov3 pmax, uint32_t n, const uint32_t* cps)
{
    uint32_t cnt[8] = { 0 };
    uint32_t* lists = (uint32_t*)malloc((size_t)8 * (n ? n : 1) * sizeof(uint32_t));
    ov3 ce = v3_sub(pmax, pmin);
    ce.x *= 0.5f; ce.y *= 0.5f; ce.z *= 0.5f;
    for (uint32_t ci = 0; ci < n; ci++)
    {
        const uint32_t cp = cps[ci];
        const uint32_t cidx = st->cluster_pointers[cp];
        const tgx_object* od = &st->objects[st->c2o[cidx]];
        float ws2ms[16];
        oracle_ws2ms(od, cp - od->first_cluster_pointer, ws2ms);
        for (uint32_t c = 0; c < 8; c++)
        {
            const float dx = (float)(c % 2) * ce.x, dy = (float)((c / 2) % 2) * ce.y, dz = (float)((c / 4) % 2) * ce.z;
            const ov3 cmin = { pmin.x + dx, pmin.y + dy, pmin.z + dz };
            const ov3 cmax = { cmin.x + ce.x, cmin.y + ce.y, cmin.z + ce.z };
            const float w[8][3] = {
                { cmin.x, cmin.y, cmin.z }, { cmax.x, cmin.y, cmin.z }, { cmin.x, cmax.y, cmin.z }, { cmax.x, cmax.y, cmin.z },
                { cmin.x, cmin.y, cmax.z }, { cmax.x, cmin.y, cmax.z }, { cmin.x, cmax.y, cmax.z }, { cmax.x, cmax.y, cmax.z } };
            ov3 bc[8];
            for (int k = 0; k < 8; k++) bc[k] = mulv4_xyz(ws2ms, w[k][0], w[k][1], w[k][2], 1.0f);
            const ov3 zmin = { 0.0f, 0.0f, 0.0f }, zmax = { (float)CSIDE, (float)CSIDE, (float)CSIDE };
            if (oracle_aabb_obb(zmin, zmax, bc))
            {
                if (cnt[c] == 0 || lists[c * n + cnt[c] - 1] != cp) lists[c * n + cnt[c]++] = cp;
            }
        }
    }
    const uint32_t child_voxels = (uint32_t)ce.x * (uint32_t)ce.y * (uint32_t)ce.z;
    const int as_leaf = child_voxels == BLOCK * BLOCK * BLOCK;
    for (uint32_t c = 0; c < 8; c++)
    {
        if (!cnt[c]) continue;
        const float dx = (float)(c % 2) * ce.x, dy = (float)((c / 2) % 2) * ce.y, dz = (float)((c / 4) % 2) * ce.z;
        const ov3 cmin = { pmin.x + dx, pmin.y + dy, pmin.z + dz };
        const ov3 cmax = { cmin.x + ce.x, cmin.y + ce.y, cmin.z + ce.z };
        if (as_leaf) leaf(st, cmin, cmax, cnt[c], &lists[c * n]);
        else inner(st, cmin, cmax, cnt[c], &lists[c * n]);
    }
    free(lists);
}

static svo_state* g_sort_state;
static int cmp_idx(const void* a, const void* b)
{
    const uint64_t ka = g_sort_state->keys[*(const uint32_t*)a], kb = g_sort_state->keys[*(const uint32_t*)b];
    return ka < kb ? -1 : ka > kb;
}

/*
 * Builds the voxel set over [mn, mn + 2^extent_log2)^3.  Writes up to
 * `capacity` blocks sorted by block index (bz*B + by)*B + bx: out_block_xyz =
 * world min corner, out_words = 1024 words each.  Returns the number of
 * non-empty blocks; *out_samples = voxel-centre samples evaluated.
 */
int64_t oracle_svo_build_mat(const tgx_object* objects, uint32_t n_objects, uint32_t n_cluster_pointers,
                             const uint32_t* cluster_pointers, const uint32_t* c2o, const uint32_t* bits,
                             const uint8_t* material, const float mn[3], uint32_t extent_log2,
                             int32_t* out_block_xyz, uint32_t* out_words, uint16_t* out_mats, uint32_t capacity,
                             uint64_t* out_samples)
{
    svo_state st;
    memset(&st, 0, sizeof(st));
    st.objects = objects; st.cluster_pointers = cluster_pointers; st.c2o = c2o; st.bits = bits;
    st.material = out_mats ? material : NULL;
    memcpy(st.mn, mn, sizeof(st.mn));
    st.bpa = 1u << (extent_log2 - 5);

    /* :495-537: per object, all its cluster pointers, dropping empty clusters */
    uint32_t* cps = (uint32_t*)malloc((size_t)(n_cluster_pointers ? n_cluster_pointers : 1) * sizeof(uint32_t));
    uint32_t ncp = 0;
    uint32_t cur = 0;
    while (cur < n_cluster_pointers)
    {
        const tgx_object* od = &objects[c2o[cluster_pointers[cur]]];
        const uint32_t cnt = od->n_cluster_pointers_per_dim[0] * od->n_cluster_pointers_per_dim[1] * od->n_cluster_pointers_per_dim[2];
        cur += cnt;
        for (uint32_t r = 0; r < cnt; r++)
        {
            const uint32_t cp = od->first_cluster_pointer + r;
            const uint32_t cidx = cluster_pointers[cp];
            uint32_t any = 0;
            for (int w = 0; w < 16; w++) any |= bits[(uint64_t)cidx * 16u + w];
            if (any) cps[ncp++] = cp;
        }
    }
    (void)n_objects;
    const float ext = (float)(1u << extent_log2);
    const ov3 rmin = { mn[0], mn[1], mn[2] };
    const ov3 rmax = { mn[0] + ext, mn[1] + ext, mn[2] + ext };
    inner(&st, rmin, rmax, ncp, cps);
    free(cps);

    uint32_t* order = (uint32_t*)malloc((size_t)(st.n ? st.n : 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < st.n; i++) order[i] = i;
    g_sort_state = &st;
    qsort(order, st.n, sizeof(uint32_t), cmp_idx);
    for (uint32_t i = 0; i < st.n && i < capacity; i++)
    {
        const uint64_t k = st.keys[order[i]];
        const uint64_t bx = k % st.bpa, by = (k / st.bpa) % st.bpa, bz = k / ((uint64_t)st.bpa * st.bpa);
        out_block_xyz[3 * i + 0] = (int32_t)(mn[0] + (float)(bx * BLOCK));
        out_block_xyz[3 * i + 1] = (int32_t)(mn[1] + (float)(by * BLOCK));
        out_block_xyz[3 * i + 2] = (int32_t)(mn[2] + (float)(bz * BLOCK));
        memcpy(&out_words[(size_t)i * 1024], &st.words[(size_t)order[i] * 1024], 4096);
        if (st.material) memcpy(&out_mats[(size_t)i * 32768], &st.mats[(size_t)order[i] * 32768], 65536);
    }
    free(order);
    free(st.keys);
    free(st.words);
    free(st.mats);
    if (out_samples) *out_samples = st.samples;
    return (int64_t)st.n;
}

int64_t oracle_svo_build(const tgx_object* objects, uint32_t n_objects, uint32_t n_cluster_pointers,
                         const uint32_t* cluster_pointers, const uint32_t* c2o, const uint32_t* bits,
                         const float mn[3], uint32_t extent_log2,
                         int32_t* out_block_xyz, uint32_t* out_words, uint32_t capacity, uint64_t* out_samples)
{
    return oracle_svo_build_mat(objects, n_objects, n_cluster_pointers, cluster_pointers, c2o, bits, NULL, mn,
                                extent_log2, out_block_xyz, out_words, NULL, capacity, out_samples);
}

int oracle_aabb_obb_flat(const float mn[3], const float mx[3], const float corners[24])
{
    ov3 c[8];
    for (int i = 0; i < 8; i++) { c[i].x = corners[3 * i]; c[i].y = corners[3 * i + 1]; c[i].z = corners[3 * i + 2]; }
    const ov3 a = { mn[0], mn[1], mn[2] }, b = { mx[0], mx[1], mx[2] };
    return oracle_aabb_obb(a, b, c);
}
