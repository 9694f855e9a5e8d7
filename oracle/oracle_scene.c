/*
 * oracle_scene.c -- the oracle's own copy of the seeded synthetic scene
 * generator and of tg's pinhole view builder.
 *
 * TEST INFRASTRUCTURE.  bench.py's CPU reference arm must build its inputs
 * without the product library, so the oracle carries its own restatement of
 * the generator's definition:
 *
 *   - counter hash h(seed, stream, i) = f(f(seed * 0x2545F4914F6CDD1D ^ f(stream)) ^ i)
 *     with f the SplitMix64 finaliser (Steele, Lea, Flood 2014);
 *   - u(h) = (h >> 40) / 2^24, a uniform float with 24 exact bits;
 *   - clusters per axis min + h(DIMS, 3i+a) % span; translations box_min +
 *     u(TRANS, 3i+a) (box_max - box_min); LUT index h(OBJLUT, i) % n_luts;
 *   - rotation from a unit quaternion drawn by rejection in the 4-ball
 *     (u(QUAT, 4096 i + 4k + c) * 2 - 1, accepted when 0.01 < |q|^2 <= 1);
 *   - kind 0: a voxel is solid when (h(BITS, 512 c + v) >> 40) < p * 2^24;
 *     kind 1: 3D value noise (smoothstep-weighted trilinear lattice values
 *     u(NOISE, key)) at the voxel centre plus a per-object lattice offset
 *     h(NOISEOFF, 3 o + a) % 4096, in units of the period, above the threshold;
 *   - material byte h(MAT, 512 c + v) & 255; LUT entries albedo
 *     0.05 + 0.9 u(LUT, 4l + a), roughness 0.1 + 0.9 u(LUT, 4l + 3).
 *
 * tests/test_oracle_scene.py checks that it gives the product generator's
 * scene byte for byte.  The view builder follows tg's camera helpers
 * (tgvk_core.c:382-444: tg_camera_rotation, perspective, the inverse of
 * P * R and the four normalised corner rays; tgm_m4_euler tg_math.c:2020-2028,
 * tgm_m4_rotate_x/y :2501-2559, tgm_m4_perspective :2469-2499).
 */
#include "oracle_common.h"

#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { OS_DIMS = 1, OS_TRANS, OS_QUAT, OS_BITS, OS_NOISE, OS_MAT, OS_LUT, OS_OBJLUT, OS_NOISEOFF };

static inline uint64_t os_fin(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x ^= x >> 30; x *= 0xBF58476D1CE4E5B9ull;
    x ^= x >> 27; x *= 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

static inline uint64_t os_hash(uint64_t seed, uint64_t stream, uint64_t i)
{
    return os_fin(os_fin(seed * 0x2545F4914F6CDD1Dull ^ os_fin(stream)) ^ i);
}

static inline float os_unit(uint64_t h) { return (float)(h >> 40) * (1.0f / 16777216.0f); }

static void os_rotation(uint64_t seed, uint64_t obj, float* m)
{
    float q[4] = { 0, 0, 0, 0 }, n2 = 0.0f;
    for (uint64_t k = 0;; k++)
    {
        for (int c = 0; c < 4; c++) q[c] = 2.0f * os_unit(os_hash(seed, OS_QUAT, obj * 4096 + 4 * k + c)) - 1.0f;
        n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        if (n2 > 0.01f && n2 <= 1.0f) break;
    }
    const float n = sqrtf(n2);
    const float w = q[0] / n, x = q[1] / n, y = q[2] / n, z = q[3] / n;
    memset(m, 0, 16 * sizeof(float));
    OM(m, 0, 0) = 1.0f - 2.0f * (y * y + z * z);
    OM(m, 1, 0) = 2.0f * (x * y + w * z);
    OM(m, 2, 0) = 2.0f * (x * z - w * y);
    OM(m, 0, 1) = 2.0f * (x * y - w * z);
    OM(m, 1, 1) = 1.0f - 2.0f * (x * x + z * z);
    OM(m, 2, 1) = 2.0f * (y * z + w * x);
    OM(m, 0, 2) = 2.0f * (x * z + w * y);
    OM(m, 1, 2) = 2.0f * (y * z - w * x);
    OM(m, 2, 2) = 1.0f - 2.0f * (x * x + y * y);
    OM(m, 3, 3) = 1.0f;
}

static inline float os_lattice(uint64_t seed, int64_t i, int64_t j, int64_t k)
{
    const uint64_t key = ((uint64_t)(i & 0x1FFFFF) << 42) | ((uint64_t)(j & 0x1FFFFF) << 21) | (uint64_t)(k & 0x1FFFFF);
    return os_unit(os_hash(seed, OS_NOISE, key));
}

static inline float os_smooth(float f) { return f * f * (3.0f - 2.0f * f); }
static inline float os_lerp(float a, float b, float s) { return a + s * (b - a); }

static float os_noise(uint64_t seed, float px, float py, float pz)
{
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const int64_t i = (int64_t)fx, j = (int64_t)fy, k = (int64_t)fz;
    const float sx = os_smooth(px - fx), sy = os_smooth(py - fy), sz = os_smooth(pz - fz);
    float y[2];
    for (int dz = 0; dz < 2; dz++)
    {
        const float x0 = os_lerp(os_lattice(seed, i, j, k + dz), os_lattice(seed, i + 1, j, k + dz), sx);
        const float x1 = os_lerp(os_lattice(seed, i, j + 1, k + dz), os_lattice(seed, i + 1, j + 1, k + dz), sx);
        y[dz] = os_lerp(x0, x1, sy);
    }
    return os_lerp(y[0], y[1], sz);
}

/* Object records; returns the cluster count (0 when it would reach 2^31). */
uint64_t oracle_gen_objects(const tgx_gen_params* p, tgx_object* objects)
{
    const uint32_t span = p->max_clusters_per_axis - p->min_clusters_per_axis + 1;
    const uint32_t n_luts = p->n_luts ? p->n_luts : 1;
    const int box = p->kind != 0 || (p->box_max[0] > p->box_min[0] && p->box_max[1] > p->box_min[1] &&
                                     p->box_max[2] > p->box_min[2]);
    uint64_t total = 0;
    for (uint32_t i = 0; i < p->n_objects; i++)
    {
        tgx_object* o = &objects[i];
        uint64_t cnt = 1;
        for (int a = 0; a < 3; a++)
        {
            o->n_cluster_pointers_per_dim[a] = p->min_clusters_per_axis + (uint32_t)(os_hash(p->seed, OS_DIMS, 3ull * i + a) % span);
            cnt *= o->n_cluster_pointers_per_dim[a];
            o->translation[a] = box ? p->box_min[a] + os_unit(os_hash(p->seed, OS_TRANS, 3ull * i + a)) * (p->box_max[a] - p->box_min[a])
                                    : p->fixed_translation[a];
        }
        o->first_cluster_pointer = (uint32_t)total;
        total += cnt;
        o->lut_idx = (uint32_t)(os_hash(p->seed, OS_OBJLUT, i) % n_luts);
        os_rotation(p->seed, i, o->rotation);
    }
    return total >= (1ull << 31) ? 0 : total;
}

/* The scene arrays for objects from oracle_gen_objects: cluster pointers equal
 * cluster indices (as tg fills a fresh scene), bits, material bytes, LUTs. */
void oracle_gen_fill(const tgx_gen_params* p, const tgx_object* objects, uint32_t n_clusters, uint32_t* cluster_pointers,
                     uint32_t* c2o, uint32_t* bits, uint8_t* mats, tgx_material* luts)
{
    for (uint32_t i = 0; i < p->n_objects; i++)
    {
        const tgx_object* o = &objects[i];
        const uint32_t cnt = o->n_cluster_pointers_per_dim[0] * o->n_cluster_pointers_per_dim[1] * o->n_cluster_pointers_per_dim[2];
        for (uint32_t r = 0; r < cnt; r++)
        {
            cluster_pointers[o->first_cluster_pointer + r] = o->first_cluster_pointer + r;
            c2o[o->first_cluster_pointer + r] = i;
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
        const uint32_t oi = c2o[c];
        const tgx_object* o = &objects[oi];
        const uint32_t rel = (uint32_t)c - o->first_cluster_pointer;
        const uint32_t nx = o->n_cluster_pointers_per_dim[0], ny = o->n_cluster_pointers_per_dim[1];
        const uint32_t cc[3] = { rel % nx, (rel / nx) % ny, rel / (nx * ny) };
        float off[3];
        for (int a = 0; a < 3; a++) off[a] = (float)(os_hash(p->seed, OS_NOISEOFF, 3ull * oi + a) % 4096u);
        uint32_t w[16] = { 0 };
        for (uint32_t v = 0; v < 512; v++)
        {
            const uint64_t g = (uint64_t)c * 512u + v;
            int solid;
            if (p->kind == 0)
                solid = (uint32_t)(os_hash(p->seed, OS_BITS, g) >> 40) < bern;
            else
            {
                const uint32_t vv[3] = { v & 7u, (v >> 3) & 7u, v >> 6 };
                float q[3];
                for (int a = 0; a < 3; a++) q[a] = ((float)(8u * cc[a] + vv[a]) + 0.5f + off[a]) / period;
                solid = os_noise(p->seed, q[0], q[1], q[2]) > p->noise_threshold;
            }
            w[v >> 5] |= (uint32_t)solid << (v & 31u);
            mats[g] = (uint8_t)(os_hash(p->seed, OS_MAT, g) & 255u);
        }
        memcpy(&bits[(uint64_t)c * 16], w, sizeof(w));
    }
    const uint32_t n_luts = p->n_luts ? p->n_luts : 1;
    for (uint32_t l = 0; l < n_luts * 256; l++)
    {
        for (int a = 0; a < 3; a++) luts[l].albedo[a] = 0.05f + 0.9f * os_unit(os_hash(p->seed, OS_LUT, 4ull * l + a));
        luts[l].roughness = 0.1f + 0.9f * os_unit(os_hash(p->seed, OS_LUT, 4ull * l + 3));
    }
}

/* tg's view: camera rotation R = inverse(Rz(0) * (Ry(yaw) * Rx(pitch))), the
 * perspective P, and the corner rays normalize((inverse(P R) * (x, y, 1, 1)).xyz)
 * for (x, y) = (-1, 1), (1, 1), (1, -1), (-1, -1). */
int oracle_make_view(const float position[3], float pitch, float yaw, float fov_y, uint32_t width, uint32_t height,
                     float near_plane, float far_plane, tgx_view* v)
{
    if (!position || !v || width == 0 || height == 0 || !(far_plane > near_plane) || !(near_plane > 0.0f)) return 1;
    float rx[16], ry[16], rz[16], e[16], r[16], pm[16], pr[16], ivp[16];
    memset(rx, 0, 64); memset(ry, 0, 64); memset(rz, 0, 64);
    for (int i = 0; i < 4; i++) OM(rx, i, i) = OM(ry, i, i) = OM(rz, i, i) = 1.0f;
    const float cp = cosf(pitch), sp = sinf(pitch), cy = cosf(yaw), sy = sinf(yaw);
    OM(rx, 1, 1) = cp; OM(rx, 2, 1) = sp; OM(rx, 1, 2) = -sp; OM(rx, 2, 2) = cp;
    OM(ry, 0, 0) = cy; OM(ry, 2, 0) = -sy; OM(ry, 0, 2) = sy; OM(ry, 2, 2) = cy;
    or_m4_mul(ry, rx, e);
    or_m4_mul(rz, e, e);
    or_m4_inverse(e, r);
    const float aspect = (float)width / (float)height;
    const float t = tanf(fov_y / 2.0f);
    memset(pm, 0, 64);
    OM(pm, 0, 0) = 1.0f / (aspect * t);
    OM(pm, 1, 1) = -1.0f / t;
    OM(pm, 2, 2) = far_plane / (near_plane - far_plane);
    OM(pm, 3, 2) = -1.0f;
    OM(pm, 2, 3) = -(2.0f * far_plane * near_plane) / (far_plane - near_plane);
    or_m4_mul(pm, r, pr);
    or_m4_inverse(pr, ivp);
    static const float xy[4][2] = { { -1.0f, 1.0f }, { 1.0f, 1.0f }, { 1.0f, -1.0f }, { -1.0f, -1.0f } };
    float* dst[4] = { v->ray_bl, v->ray_br, v->ray_tr, v->ray_tl };
    for (int k = 0; k < 4; k++)
    {
        const float in[4] = { xy[k][0], xy[k][1], 1.0f, 1.0f };
        float o[4];
        or_m4_mulv4(ivp, in, o);
        const float mag = sqrtf(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        dst[k][0] = o[0] / mag; dst[k][1] = o[1] / mag; dst[k][2] = o[2] / mag; dst[k][3] = 0.0f;
    }
    for (int i = 0; i < 3; i++) v->camera[i] = position[i];
    v->camera[3] = 1.0f;
    v->near_plane = near_plane;
    v->far_plane = far_plane;
    v->width = width;
    v->height = height;
    return 0;
}
