/*
 * host_scene.c -- host-side scene helpers of libtgx: the synthetic scene
 * generator (stand-in for tg's CPU noise loop, tgvk_raytracer.c:870-978) and
 * the pinhole view builder (tg's camera helpers, tgvk_core.c:382-444).
 *
 * Compiled with -ffp-contract=off so the generated scenes are bit-identical
 * on x86-64 and aarch64 hosts: only +, -, *, /, sqrtf and floorf shape the
 * voxel bits and rotations (no libm transcendental enters a generated scene).
 * tgx_make_view calls sinf/cosf/tanf like the reference; views are inputs,
 * and tests that need bit-identical views on every host store them.
 */
#include "../../include/tgx.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- counter-based hashing (SplitMix64 finaliser) ---- */

static inline uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static inline uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t i)
{
    return mix64(mix64(seed * 0x2545F4914F6CDD1Dull ^ mix64(stream)) ^ i);
}

/* uniform float in [0, 1) with 24 random bits (exact) */
static inline float unit_f32(uint64_t h) { return (float)(h >> 40) * (1.0f / 16777216.0f); }

enum { ST_DIMS = 1, ST_TRANS, ST_QUAT, ST_BITS, ST_NOISE, ST_MAT, ST_LUT, ST_OBJLUT, ST_NOISEOFF };

/* Uniform random rotation: a unit quaternion drawn by rejection in the 4-ball
 * (uniform on S^3), turned into a column-major m4 with zero translation. */
static void random_rotation(uint64_t seed, uint64_t obj, float* m)
{
    float w = 0, x = 0, y = 0, z = 0, n2 = 0;
    for (uint64_t k = 0;; k++)
    {
        w = 2.0f * unit_f32(hash3(seed, ST_QUAT, obj * 4096 + 4 * k + 0)) - 1.0f;
        x = 2.0f * unit_f32(hash3(seed, ST_QUAT, obj * 4096 + 4 * k + 1)) - 1.0f;
        y = 2.0f * unit_f32(hash3(seed, ST_QUAT, obj * 4096 + 4 * k + 2)) - 1.0f;
        z = 2.0f * unit_f32(hash3(seed, ST_QUAT, obj * 4096 + 4 * k + 3)) - 1.0f;
        n2 = w * w + x * x + y * y + z * z;
        if (n2 > 0.01f && n2 <= 1.0f) break;
    }
    const float n = sqrtf(n2);
    w /= n; x /= n; y /= n; z /= n;
    memset(m, 0, 16 * sizeof(float));
    /* element (row r, column c) at m[4c + r] */
    m[0]  = 1.0f - 2.0f * (y * y + z * z);
    m[1]  = 2.0f * (x * y + w * z);
    m[2]  = 2.0f * (x * z - w * y);
    m[4]  = 2.0f * (x * y - w * z);
    m[5]  = 1.0f - 2.0f * (x * x + z * z);
    m[6]  = 2.0f * (y * z + w * x);
    m[8]  = 2.0f * (x * z + w * y);
    m[9]  = 2.0f * (y * z - w * x);
    m[10] = 1.0f - 2.0f * (x * x + y * y);
    m[15] = 1.0f;
}

static inline float smooth(float f) { return f * f * (3.0f - 2.0f * f); }

static inline float lattice(uint64_t seed, int64_t i, int64_t j, int64_t k)
{
    const uint64_t key = ((uint64_t)(i & 0x1FFFFF) << 42) | ((uint64_t)(j & 0x1FFFFF) << 21) | (uint64_t)(k & 0x1FFFFF);
    return unit_f32(hash3(seed, ST_NOISE, key));
}

/* 3D value noise: lattice values on an integer grid, smoothstep-weighted
 * trilinear interpolation.  p is in lattice units. */
static float value_noise(uint64_t seed, float px, float py, float pz)
{
    const float fx0 = floorf(px), fy0 = floorf(py), fz0 = floorf(pz);
    const int64_t ix = (int64_t)fx0, iy = (int64_t)fy0, iz = (int64_t)fz0;
    const float sx = smooth(px - fx0), sy = smooth(py - fy0), sz = smooth(pz - fz0);
    const float c000 = lattice(seed, ix, iy, iz),         c100 = lattice(seed, ix + 1, iy, iz);
    const float c010 = lattice(seed, ix, iy + 1, iz),     c110 = lattice(seed, ix + 1, iy + 1, iz);
    const float c001 = lattice(seed, ix, iy, iz + 1),     c101 = lattice(seed, ix + 1, iy, iz + 1);
    const float c011 = lattice(seed, ix, iy + 1, iz + 1), c111 = lattice(seed, ix + 1, iy + 1, iz + 1);
    const float x00 = c000 + sx * (c100 - c000), x10 = c010 + sx * (c110 - c010);
    const float x01 = c001 + sx * (c101 - c001), x11 = c011 + sx * (c111 - c011);
    const float y0 = x00 + sy * (x10 - x00), y1 = x01 + sy * (x11 - x01);
    return y0 + sz * (y1 - y0);
}

void tgx_free_generated_scene(tgx_gen_scene* s)
{
    if (!s) return;
    free(s->objects);
    free(s->cluster_pointers);
    free(s->cluster_idx_to_object_idx);
    free(s->voxel_bits);
    free(s->material_idx);
    free(s->luts);
    memset(s, 0, sizeof(*s));
}

/* Object records of a generated scene (dims, first pointer, translation, LUT,
 * rotation); returns the cluster count, or 0 when it would reach 2^31. */
uint64_t tgx__gen_objects(const tgx_gen_params* p, tgx_object* objects)
{
    const uint32_t n_obj = p->n_objects;
    const uint32_t span = p->max_clusters_per_axis - p->min_clusters_per_axis + 1;
    const uint32_t n_luts = p->n_luts ? p->n_luts : 1;
    uint64_t total = 0;
    for (uint32_t i = 0; i < n_obj; i++)
    {
        tgx_object* o = &objects[i];
        for (int a = 0; a < 3; a++)
            o->n_cluster_pointers_per_dim[a] = p->min_clusters_per_axis + (uint32_t)(hash3(p->seed, ST_DIMS, 3ull * i + a) % span);
        o->first_cluster_pointer = (uint32_t)total;
        total += (uint64_t)o->n_cluster_pointers_per_dim[0] * o->n_cluster_pointers_per_dim[1] * o->n_cluster_pointers_per_dim[2];
        /* kind 1 always spreads objects over the box; kind 0 only when the box is not empty */
        const int use_box = p->kind != 0 || (p->box_max[0] > p->box_min[0] && p->box_max[1] > p->box_min[1] &&
                                             p->box_max[2] > p->box_min[2]);
        for (int a = 0; a < 3; a++)
        {
            if (!use_box)
                o->translation[a] = p->fixed_translation[a];
            else
                o->translation[a] = p->box_min[a] + unit_f32(hash3(p->seed, ST_TRANS, 3ull * i + a)) * (p->box_max[a] - p->box_min[a]);
        }
        o->lut_idx = (uint32_t)(hash3(p->seed, ST_OBJLUT, i) % n_luts);
        random_rotation(p->seed, i, o->rotation);
    }
    return total >= (1ull << 31) ? 0 : total;
}

/* LUT entries: albedo U[0.05, 0.95], roughness U[0.1, 1.0] */
void tgx__gen_luts(const tgx_gen_params* p, tgx_material* luts)
{
    const uint32_t n_luts = p->n_luts ? p->n_luts : 1;
    for (uint32_t l = 0; l < n_luts * 256; l++)
    {
        for (int a = 0; a < 3; a++) luts[l].albedo[a] = 0.05f + 0.9f * unit_f32(hash3(p->seed, ST_LUT, 4ull * l + a));
        luts[l].roughness = 0.1f + 0.9f * unit_f32(hash3(p->seed, ST_LUT, 4ull * l + 3));
    }
}

tgx_status tgx_generate_scene(const tgx_gen_params* p, tgx_gen_scene* out)
{
    if (!p || !out || p->n_objects == 0 || p->min_clusters_per_axis == 0 ||
        p->max_clusters_per_axis < p->min_clusters_per_axis || p->kind > 1)
        return TGX_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    const uint32_t n_obj = p->n_objects;
    const uint32_t n_luts = p->n_luts ? p->n_luts : 1;

    out->objects = (tgx_object*)calloc(n_obj, sizeof(tgx_object));
    if (!out->objects) return TGX_ERR_OUT_OF_MEMORY;
    const uint64_t total = tgx__gen_objects(p, out->objects);
    if (total == 0) { tgx_free_generated_scene(out); return TGX_ERR_CAPACITY; }
    const uint32_t n_clusters = (uint32_t)total;

    out->cluster_pointers = (uint32_t*)malloc((size_t)n_clusters * 4);
    out->cluster_idx_to_object_idx = (uint32_t*)malloc((size_t)n_clusters * 4);
    out->voxel_bits = (uint32_t*)calloc((size_t)n_clusters * 16, 4);
    out->material_idx = (uint8_t*)malloc((size_t)n_clusters * 512);
    out->luts = (tgx_material*)malloc((size_t)n_luts * 256 * sizeof(tgx_material));
    if (!out->cluster_pointers || !out->cluster_idx_to_object_idx || !out->voxel_bits || !out->material_idx || !out->luts)
    {
        tgx_free_generated_scene(out);
        return TGX_ERR_OUT_OF_MEMORY;
    }
    /* fresh tg scenes get cluster index == cluster pointer (tgvk_raytracer.c:705-712, 859) */
    for (uint32_t i = 0; i < n_obj; i++)
    {
        const tgx_object* o = &out->objects[i];
        const uint32_t cnt = o->n_cluster_pointers_per_dim[0] * o->n_cluster_pointers_per_dim[1] * o->n_cluster_pointers_per_dim[2];
        for (uint32_t r = 0; r < cnt; r++)
        {
            out->cluster_pointers[o->first_cluster_pointer + r] = o->first_cluster_pointer + r;
            out->cluster_idx_to_object_idx[o->first_cluster_pointer + r] = i;
        }
    }
#ifdef _OPENMP
    if (p->threads) omp_set_num_threads((int)p->threads);
#endif
    const float period = p->noise_period > 0.0f ? p->noise_period : 64.0f;
    const uint32_t bern = (uint32_t)((double)p->bernoulli_p * 16777216.0);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t c = 0; c < (int64_t)n_clusters; c++)
    {
        const uint32_t oi = out->cluster_idx_to_object_idx[c];
        const tgx_object* o = &out->objects[oi];
        const uint32_t rel = (uint32_t)c - o->first_cluster_pointer;
        const uint32_t nx = o->n_cluster_pointers_per_dim[0], ny = o->n_cluster_pointers_per_dim[1];
        const uint32_t cx = rel % nx, cy = (rel / nx) % ny, cz = rel / (nx * ny);
        /* per-object lattice offset so objects do not share a noise field */
        const float ox = (float)(hash3(p->seed, ST_NOISEOFF, 3ull * oi + 0) % 4096u);
        const float oy = (float)(hash3(p->seed, ST_NOISEOFF, 3ull * oi + 1) % 4096u);
        const float oz = (float)(hash3(p->seed, ST_NOISEOFF, 3ull * oi + 2) % 4096u);
        uint32_t* w = &out->voxel_bits[(uint64_t)c * 16];
        uint8_t* mat = &out->material_idx[(uint64_t)c * 512];
        for (uint32_t v = 0; v < 512; v++)
        {
            const uint32_t vx = v & 7u, vy = (v >> 3) & 7u, vz = v >> 6;
            const uint64_t gvi = (uint64_t)c * 512u + v;
            int solid;
            if (p->kind == 0)
            {
                solid = (uint32_t)(hash3(p->seed, ST_BITS, gvi) >> 40) < bern;
            }
            else
            {
                const float X = (float)(8u * cx + vx) + 0.5f + ox;
                const float Y = (float)(8u * cy + vy) + 0.5f + oy;
                const float Z = (float)(8u * cz + vz) + 0.5f + oz;
                solid = value_noise(p->seed, X / period, Y / period, Z / period) > p->noise_threshold;
            }
            if (solid) w[v >> 5] |= 1u << (v & 31u);
            mat[v] = (uint8_t)(hash3(p->seed, ST_MAT, gvi) & 255u);
        }
    }
    tgx__gen_luts(p, out->luts);

    tgx_scene_desc* d = &out->desc;
    d->n_objects = n_obj;
    d->objects = out->objects;
    d->n_cluster_pointers = n_clusters;
    d->cluster_pointers = out->cluster_pointers;
    d->n_clusters = n_clusters;
    d->cluster_idx_to_object_idx = out->cluster_idx_to_object_idx;
    d->voxel_bits = out->voxel_bits;
    d->material_idx = out->material_idx;
    d->n_luts = n_luts;
    d->luts = out->luts;
    return TGX_OK;
}

/* ---- tg's camera helpers (tgvk_core.c:382-444), restated ---- */

static void m4_identity(float* m) { memset(m, 0, 64); m[0] = m[5] = m[10] = m[15] = 1.0f; }

static void m4_mul(const float* a, const float* b, float* out)
{
    float r[16];
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++)
            r[4 * c + row] = a[row] * b[4 * c] + a[4 + row] * b[4 * c + 1] + a[8 + row] * b[4 * c + 2] + a[12 + row] * b[4 * c + 3];
    memcpy(out, r, 64);
}

/* cofactor inverse in the order of tgm_m4_inverse (tg_math.c:2185-2234) */
static void m4_inverse(const float* m, float* out)
{
#define E(r, c) m[4 * (c) + (r)]
    const float m2323 = E(2,2) * E(3,3) - E(2,3) * E(3,2), m1323 = E(2,1) * E(3,3) - E(2,3) * E(3,1);
    const float m1223 = E(2,1) * E(3,2) - E(2,2) * E(3,1), m0323 = E(2,0) * E(3,3) - E(2,3) * E(3,0);
    const float m0223 = E(2,0) * E(3,2) - E(2,2) * E(3,0), m0123 = E(2,0) * E(3,1) - E(2,1) * E(3,0);
    const float m2313 = E(1,2) * E(3,3) - E(1,3) * E(3,2), m1313 = E(1,1) * E(3,3) - E(1,3) * E(3,1);
    const float m1213 = E(1,1) * E(3,2) - E(1,2) * E(3,1), m2312 = E(1,2) * E(2,3) - E(1,3) * E(2,2);
    const float m1312 = E(1,1) * E(2,3) - E(1,3) * E(2,1), m1212 = E(1,1) * E(2,2) - E(1,2) * E(2,1);
    const float m0313 = E(1,0) * E(3,3) - E(1,3) * E(3,0), m0213 = E(1,0) * E(3,2) - E(1,2) * E(3,0);
    const float m0312 = E(1,0) * E(2,3) - E(1,3) * E(2,0), m0212 = E(1,0) * E(2,2) - E(1,2) * E(2,0);
    const float m0113 = E(1,0) * E(3,1) - E(1,1) * E(3,0), m0112 = E(1,0) * E(2,1) - E(1,1) * E(2,0);
    const float det = 1.0f / (E(0,0) * (E(1,1) * m2323 - E(1,2) * m1323 + E(1,3) * m1223)
                            - E(0,1) * (E(1,0) * m2323 - E(1,2) * m0323 + E(1,3) * m0223)
                            + E(0,2) * (E(1,0) * m1323 - E(1,1) * m0323 + E(1,3) * m0123)
                            - E(0,3) * (E(1,0) * m1223 - E(1,1) * m0223 + E(1,2) * m0123));
    float r[16];
#define R(rr, cc) r[4 * (cc) + (rr)]
    R(0,0) = det *  (E(1,1) * m2323 - E(1,2) * m1323 + E(1,3) * m1223);
    R(0,1) = det * -(E(0,1) * m2323 - E(0,2) * m1323 + E(0,3) * m1223);
    R(0,2) = det *  (E(0,1) * m2313 - E(0,2) * m1313 + E(0,3) * m1213);
    R(0,3) = det * -(E(0,1) * m2312 - E(0,2) * m1312 + E(0,3) * m1212);
    R(1,0) = det * -(E(1,0) * m2323 - E(1,2) * m0323 + E(1,3) * m0223);
    R(1,1) = det *  (E(0,0) * m2323 - E(0,2) * m0323 + E(0,3) * m0223);
    R(1,2) = det * -(E(0,0) * m2313 - E(0,2) * m0313 + E(0,3) * m0213);
    R(1,3) = det *  (E(0,0) * m2312 - E(0,2) * m0312 + E(0,3) * m0212);
    R(2,0) = det *  (E(1,0) * m1323 - E(1,1) * m0323 + E(1,3) * m0123);
    R(2,1) = det * -(E(0,0) * m1323 - E(0,1) * m0323 + E(0,3) * m0123);
    R(2,2) = det *  (E(0,0) * m1313 - E(0,1) * m0313 + E(0,3) * m0113);
    R(2,3) = det * -(E(0,0) * m1312 - E(0,1) * m0312 + E(0,3) * m0112);
    R(3,0) = det * -(E(1,0) * m1223 - E(1,1) * m0223 + E(1,2) * m0123);
    R(3,1) = det *  (E(0,0) * m1223 - E(0,1) * m0223 + E(0,2) * m0123);
    R(3,2) = det * -(E(0,0) * m1213 - E(0,1) * m0213 + E(0,2) * m0113);
    R(3,3) = det *  (E(0,0) * m1212 - E(0,1) * m0212 + E(0,2) * m0112);
#undef R
#undef E
    memcpy(out, r, 64);
}

tgx_status tgx_make_view(const float position[3], float pitch, float yaw, float fov_y, uint32_t width,
                         uint32_t height, float near_plane, float far_plane, tgx_view* v)
{
    if (!position || !v || width == 0 || height == 0 || !(far_plane > near_plane) || !(near_plane > 0.0f))
        return TGX_ERR_INVALID_ARGUMENT;
    /* tgm_m4_euler(pitch, yaw, 0) = Rz * (Ry * Rx)  (tg_math.c:2020-2028) */
    float rx[16], ry[16], rz[16], e[16], r[16], p[16], pr[16], ivp[16];
    m4_identity(rx); m4_identity(ry); m4_identity(rz);
    const float cx = cosf(pitch), sx = sinf(pitch), cy = cosf(yaw), sy = sinf(yaw);
    rx[5] = cx; rx[6] = sx; rx[9] = -sx; rx[10] = cx;            /* tgm_m4_rotate_x, tg_math.c:2501-2529 */
    ry[0] = cy; ry[2] = -sy; ry[8] = sy; ry[10] = cy;            /* tgm_m4_rotate_y, tg_math.c:2531-2559 */
    m4_mul(ry, rx, e);
    m4_mul(rz, e, e);
    m4_inverse(e, r);                                            /* tg_camera_rotation, tgvk_core.c:382-388 */
    /* tgm_m4_perspective (tg_math.c:2469-2499) */
    const float aspect = (float)width / (float)height;
    const float t = tanf(fov_y / 2.0f);
    memset(p, 0, 64);
    p[0] = 1.0f / (aspect * t);
    p[5] = -1.0f / t;
    p[10] = far_plane / (near_plane - far_plane);
    p[11] = -1.0f;
    p[14] = -(2.0f * far_plane * near_plane) / (far_plane - near_plane);
    m4_mul(p, r, pr);
    m4_inverse(pr, ivp);                                         /* tgvk_core.c:437 */
    const float corners[4][2] = { { -1.0f, 1.0f }, { 1.0f, 1.0f }, { 1.0f, -1.0f }, { -1.0f, -1.0f } };
    float* outs[4] = { v->ray_bl, v->ray_br, v->ray_tr, v->ray_tl };
    for (int k = 0; k < 4; k++)
    {
        const float in[4] = { corners[k][0], corners[k][1], 1.0f, 1.0f };
        float o[3];
        for (int row = 0; row < 3; row++)
            o[row] = in[0] * ivp[row] + in[1] * ivp[4 + row] + in[2] * ivp[8 + row] + in[3] * ivp[12 + row];
        const float mag = sqrtf(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        outs[k][0] = o[0] / mag; outs[k][1] = o[1] / mag; outs[k][2] = o[2] / mag; outs[k][3] = 0.0f;
    }
    v->camera[0] = position[0]; v->camera[1] = position[1]; v->camera[2] = position[2]; v->camera[3] = 1.0f;
    v->near_plane = near_plane;
    v->far_plane = far_plane;
    v->width = width;
    v->height = height;
    return TGX_OK;
}

int tgx_vis_decode(uint64_t packed, float* out_depth, uint32_t* out_cluster_pointer, uint32_t* out_voxel_idx)
{
    /* tgvk_raytracer.c:1639-1653 */
    const float depth = (float)(packed >> 40) / 16777215.0f;
    if (out_depth) *out_depth = depth;
    if (depth < 1.0f)
    {
        if (out_cluster_pointer) *out_cluster_pointer = (uint32_t)(packed >> 9) & 2147483647u;
        if (out_voxel_idx) *out_voxel_idx = (uint32_t)packed & 511u;
        return 1;
    }
    if (out_cluster_pointer) *out_cluster_pointer = UINT32_MAX;
    if (out_voxel_idx) *out_voxel_idx = UINT32_MAX;
    return 0;
}
