/*
 * oracle_vis.c -- CPU oracle of the visibility pass.
 *
 * TEST INFRASTRUCTURE.  A line-by-line restatement of tg's fragment shader
 * tg/assets/shaders/raytracer/visibility.frag:22-207 (with collide.inc:3-24,
 * common.inc:40-46 and clear.comp:15-21) in IEEE binary32, source order, no
 * FMA contraction.  The rasteriser's job (which fragments run) is replaced by
 * "every pixel against every cluster" (mode 0) or by a conservative
 * per-cluster screen rectangle computed in double precision (mode 1); the
 * shader's own ray/box test (visibility.frag:78) is the only arbiter in both,
 * applied as the raster pipeline applies it (or_ray_cluster: a ray parallel
 * to a slab it does not cross produces no fragment).
 *
 * GLSL leaves the rounding of inverse(), normalize(), mix() and matrix
 * products to the driver, so the oracle pins them to tg's C math, which the
 * engine uses for the same quantities on the host:
 *   inverse      -> tgm_m4_inverse     (tg_math.c:2185-2234)
 *   A * B        -> tgm_m4_mul         (tg_math.c:2374-2399)
 *   M * v        -> tgm_m4_mulv4       (tg_math.c:2428-2438)
 *   normalize(v) -> tgm_v3_normalized  (tg_math.c:1175-1184, three divisions)
 *   mix(a,b,t)   -> a*(1-t) + b*t      (GLSL 4.50 8.3; tgm_v3_lerp tg_math.c:1091-1098)
 * gl_FragCoord is the pixel centre (x+0.5, y+0.5) with y = 0 the top row
 * (Vulkan framebuffer origin).  The empty word is UINT64_MAX.
 */
#include "oracle_common.h"

#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CLUSTER_SIDE 8u

/*
 * One fragment of visibility.frag for pixel (px, py) and cluster pointer
 * `cluster_pointer`.  Returns 1 and writes *out_packed when the shader would
 * execute its atomicMin (visibility.frag:194-207), else 0.
 */
int oracle_vis_pair(const tgx_object* objects, const uint32_t* cluster_pointers,
                    const uint32_t* cluster_idx_to_object_idx, const uint32_t* voxel_bits,
                    const tgx_view* cam, uint32_t cluster_pointer, uint32_t px, uint32_t py,
                    uint64_t* out_packed)
{
    /* visibility.frag:24-27 */
    const uint32_t cluster_idx = cluster_pointers[cluster_pointer];
    const uint32_t object_idx = cluster_idx_to_object_idx[cluster_idx];
    const tgx_object* od = &objects[object_idx];

    /* :29-33 */
    const float frag_x = (float)px + 0.5f;
    const float frag_y = (float)py + 0.5f;
    const float fx = frag_x / (float)cam->width;
    const float fy = 1.0f - frag_y / (float)cam->height;

    /* :35-48 */
    const uint32_t nx = od->n_cluster_pointers_per_dim[0];
    const uint32_t ny = od->n_cluster_pointers_per_dim[1];
    const uint32_t rel = cluster_pointer - od->first_cluster_pointer;
    const uint32_t rx = rel % nx;
    const uint32_t ry = (rel / nx) % ny;
    const uint32_t rz = rel / (nx * ny);
    const float off_x = (float)(rx * CLUSTER_SIDE);
    const float off_y = (float)(ry * CLUSTER_SIDE);
    const float off_z = (float)(rz * CLUSTER_SIDE);
    const float cluster_extent = (float)CLUSTER_SIDE;
    const float cluster_half_extent = cluster_extent * 0.5f;
    const float ohe_x = cluster_half_extent * (float)od->n_cluster_pointers_per_dim[0];
    const float ohe_y = cluster_half_extent * (float)od->n_cluster_pointers_per_dim[1];
    const float ohe_z = cluster_half_extent * (float)od->n_cluster_pointers_per_dim[2];

    /* :57-62  ws2ms = ws2ms3 * ws2ms2 * ws2ms1 * ws2ms0 (left-associative) */
    float m0[16], m1[16], m2[16], m3[16], ws2ms[16];
    or_m4_translate(-od->translation[0], -od->translation[1], -od->translation[2], m0);
    or_m4_inverse(od->rotation, m1);
    or_m4_translate(ohe_x, ohe_y, ohe_z, m2);
    or_m4_translate(-off_x, -off_y, -off_z, m3);
    or_m4_mul(m3, m2, ws2ms);
    or_m4_mul(ws2ms, m1, ws2ms);
    or_m4_mul(ws2ms, m0, ws2ms);

    /* :65-69 */
    const float o_ws[4] = { cam->camera[0], cam->camera[1], cam->camera[2], 1.0f };
    float o4[4];
    or_m4_mulv4(ws2ms, o_ws, o4);
    const float o[3] = { o4[0], o4[1], o4[2] };

    float d_ws[4];
    for (int i = 0; i < 3; i++)
    {
        const float a = cam->ray_bl[i] * (1.0f - fy) + cam->ray_tl[i] * fy;   /* mix(bl, tl, fy) */
        const float b = cam->ray_br[i] * (1.0f - fy) + cam->ray_tr[i] * fy;   /* mix(br, tr, fy) */
        d_ws[i] = a * (1.0f - fx) + b * fx;                                     /* mix(a, b, fx)   */
    }
    d_ws[3] = 0.0f;
    float d4[4];
    or_m4_mulv4(ws2ms, d_ws, d4);
    const float mag = sqrtf(d4[0] * d4[0] + d4[1] * d4[1] + d4[2] * d4[2]);
    const float d[3] = { d4[0] / mag, d4[1] / mag, d4[2] / mag };

    /* :71-78 */
    const float cmin[3] = { 0.0f, 0.0f, 0.0f };
    const float cmax[3] = { cluster_extent, cluster_extent, cluster_extent };
    float depth = OR_F32_MAX;
    uint32_t voxel_idx = 0;
    float enter, exit_;
    if (or_ray_cluster(o, d, cmin, cmax, &enter, &exit_))
    {
        /* :83-84 */
        float hit[3], xyz[3];
        for (int i = 0; i < 3; i++)
        {
            hit[i] = enter > 0.0f ? o[i] + enter * d[i] : o[i];
            xyz[i] = or_gmin(or_gmax(floorf(hit[i]), cmin[i]), cmax[i] - 1.0f);   /* clamp */
        }
        int32_t x = (int32_t)xyz[0], y = (int32_t)xyz[1], z = (int32_t)xyz[2];
        int32_t step_x = 0, step_y = 0, step_z = 0;
        float t_max_x = OR_F32_MAX, t_max_y = OR_F32_MAX, t_max_z = OR_F32_MAX;
        float t_delta_x = OR_F32_MAX, t_delta_y = OR_F32_MAX, t_delta_z = OR_F32_MAX;

        /* :102-137 */
        if (d[0] > 0.0f) { step_x = 1; t_max_x = enter + ((float)(x + 1) - hit[0]) / d[0]; t_delta_x = 1.0f / d[0]; }
        else if (d[0] < 0.0f) { step_x = -1; t_max_x = enter + (hit[0] - (float)x) / -d[0]; t_delta_x = 1.0f / -d[0]; }
        if (d[1] > 0.0f) { step_y = 1; t_max_y = enter + ((float)(y + 1) - hit[1]) / d[1]; t_delta_y = 1.0f / d[1]; }
        else if (d[1] < 0.0f) { step_y = -1; t_max_y = enter + (hit[1] - (float)y) / -d[1]; t_delta_y = 1.0f / -d[1]; }
        if (d[2] > 0.0f) { step_z = 1; t_max_z = enter + ((float)(z + 1) - hit[2]) / d[2]; t_delta_z = 1.0f / d[2]; }
        else if (d[2] < 0.0f) { step_z = -1; t_max_z = enter + (hit[2] - (float)z) / -d[2]; t_delta_z = 1.0f / -d[2]; }

        /* :139-191 */
        const uint64_t cluster_offset_in_voxels = (uint64_t)cluster_idx * 512u;
        for (;;)
        {
            const uint32_t rvi = CLUSTER_SIDE * CLUSTER_SIDE * (uint32_t)z + CLUSTER_SIDE * (uint32_t)y + (uint32_t)x;
            const uint64_t vox = cluster_offset_in_voxels + rvi;
            const uint32_t slot = voxel_bits[vox / 32u];
            if (slot & (1u << (uint32_t)(vox % 32u)))
            {
                const float vmin[3] = { cmin[0] + (float)x, cmin[1] + (float)y, cmin[2] + (float)z };
                const float vmax[3] = { cmin[0] + (float)(x + 1), cmin[1] + (float)(y + 1), cmin[2] + (float)(z + 1) };
                float ve, vx;
                or_ray_aabb(o, d, vmin, vmax, &ve, &vx);
                depth = or_gmax(0.0f, ve / cam->far_plane);
                voxel_idx = rvi;
                break;
            }
            if (t_max_x < t_max_y)
            {
                if (t_max_x < t_max_z) { t_max_x += t_delta_x; x += step_x; if (x < 0 || x >= (int32_t)CLUSTER_SIDE) break; }
                else                   { t_max_z += t_delta_z; z += step_z; if (z < 0 || z >= (int32_t)CLUSTER_SIDE) break; }
            }
            else
            {
                if (t_max_y < t_max_z) { t_max_y += t_delta_y; y += step_y; if (y < 0 || y >= (int32_t)CLUSTER_SIDE) break; }
                else                   { t_max_z += t_delta_z; z += step_z; if (z < 0 || z >= (int32_t)CLUSTER_SIDE) break; }
            }
        }
    }

    /* :194-207 */
    if (depth <= 1.0f)
    {
        const uint64_t depth_24b = (uint64_t)(depth * 16777215.0f) << 40;
        const uint64_t ptr_31b = (uint64_t)cluster_pointer << 9;
        *out_packed = depth_24b | ptr_31b | (uint64_t)voxel_idx;
        return 1;
    }
    return 0;
}

static inline void atomic_min_u64(uint64_t* p, uint64_t v)
{
    uint64_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) { }
}

/*
 * Conservative screen rectangle of a cluster for one view, in double
 * precision: the eight world corners of the cluster box are projected through
 * the affine corner-ray model d(fx,fy) = bl + fx(br-bl) + fy(tl-bl) and the
 * pixel bounding box is widened by `margin` pixels.  Any corner closer than
 * 0.05 along the view axis yields the whole screen.  Returns 0 if the
 * cluster lies entirely behind the camera.
 */
static int cluster_rect(const tgx_object* od, uint32_t rel, const tgx_view* cam, int margin,
                        int32_t* x0, int32_t* x1, int32_t* y0, int32_t* y1)
{
    const uint32_t nx = od->n_cluster_pointers_per_dim[0], ny = od->n_cluster_pointers_per_dim[1];
    const double off[3] = { (double)(rel % nx) * 8.0, (double)((rel / nx) % ny) * 8.0, (double)(rel / (nx * ny)) * 8.0 };
    const double ohe[3] = { 4.0 * od->n_cluster_pointers_per_dim[0], 4.0 * od->n_cluster_pointers_per_dim[1], 4.0 * od->n_cluster_pointers_per_dim[2] };
    /* columns of the basis [bl | br-bl | tl-bl] */
    double B[3][3];
    for (int i = 0; i < 3; i++)
    {
        B[i][0] = cam->ray_bl[i];
        B[i][1] = (double)cam->ray_br[i] - cam->ray_bl[i];
        B[i][2] = (double)cam->ray_tl[i] - cam->ray_bl[i];
    }
    const double det = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1])
                     - B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0])
                     + B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
    double inv[3][3];
    inv[0][0] = (B[1][1] * B[2][2] - B[1][2] * B[2][1]) / det;
    inv[0][1] = (B[0][2] * B[2][1] - B[0][1] * B[2][2]) / det;
    inv[0][2] = (B[0][1] * B[1][2] - B[0][2] * B[1][1]) / det;
    inv[1][0] = (B[1][2] * B[2][0] - B[1][0] * B[2][2]) / det;
    inv[1][1] = (B[0][0] * B[2][2] - B[0][2] * B[2][0]) / det;
    inv[1][2] = (B[0][2] * B[1][0] - B[0][0] * B[1][2]) / det;
    inv[2][0] = (B[1][0] * B[2][1] - B[1][1] * B[2][0]) / det;
    inv[2][1] = (B[0][1] * B[2][0] - B[0][0] * B[2][1]) / det;
    inv[2][2] = (B[0][0] * B[1][1] - B[0][1] * B[1][0]) / det;
    /* forward axis for the near test: centre ray */
    double fwd[3];
    double fl = 0.0;
    for (int i = 0; i < 3; i++) { fwd[i] = 0.25 * ((double)cam->ray_bl[i] + cam->ray_br[i] + cam->ray_tr[i] + cam->ray_tl[i]); fl += fwd[i] * fwd[i]; }
    fl = sqrt(fl);
    /* inward normals of the four side planes of the frustum (through the camera) */
    const float* cr[4] = { cam->ray_bl, cam->ray_br, cam->ray_tr, cam->ray_tl };
    double pn[4][3];
    for (int k = 0; k < 4; k++)
    {
        const float* a = cr[k];
        const float* b = cr[(k + 1) % 4];
        pn[k][0] = (double)a[1] * b[2] - (double)a[2] * b[1];
        pn[k][1] = (double)a[2] * b[0] - (double)a[0] * b[2];
        pn[k][2] = (double)a[0] * b[1] - (double)a[1] * b[0];
        const double s = pn[k][0] * fwd[0] + pn[k][1] * fwd[1] + pn[k][2] * fwd[2];
        const double l = sqrt(pn[k][0] * pn[k][0] + pn[k][1] * pn[k][1] + pn[k][2] * pn[k][2]);
        for (int i = 0; i < 3; i++) pn[k][i] = (s < 0 ? -pn[k][i] : pn[k][i]) / l;
    }
    int outside[4] = { 1, 1, 1, 1 };
    double fx_min = 1e300, fx_max = -1e300, fy_min = 1e300, fy_max = -1e300;
    int all_behind = 1, full = 0;
    for (int k = 0; k < 8; k++)
    {
        const double lc[3] = { off[0] + ((k & 1) ? 8.0 : 0.0) - ohe[0], off[1] + ((k & 2) ? 8.0 : 0.0) - ohe[1], off[2] + ((k & 4) ? 8.0 : 0.0) - ohe[2] };
        double p[3];
        for (int r = 0; r < 3; r++)
            p[r] = OM(od->rotation, r, 0) * lc[0] + OM(od->rotation, r, 1) * lc[1] + OM(od->rotation, r, 2) * lc[2]
                 + (double)od->translation[r] - cam->camera[r];
        const double depth = (p[0] * fwd[0] + p[1] * fwd[1] + p[2] * fwd[2]) / fl;
        if (depth > -0.05) all_behind = 0;
        const double pl = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        for (int k = 0; k < 4; k++)
            if (pn[k][0] * p[0] + pn[k][1] * p[1] + pn[k][2] * p[2] > -(0.01 + 1e-6 * pl)) outside[k] = 0;
        if (depth < 0.05) { full = 1; continue; }
        const double s = inv[0][0] * p[0] + inv[0][1] * p[1] + inv[0][2] * p[2];
        const double a = inv[1][0] * p[0] + inv[1][1] * p[1] + inv[1][2] * p[2];
        const double b = inv[2][0] * p[0] + inv[2][1] * p[1] + inv[2][2] * p[2];
        if (s <= 0.0) { full = 1; continue; }
        const double fxp = a / s, fyp = b / s;
        if (fxp < fx_min) fx_min = fxp;
        if (fxp > fx_max) fx_max = fxp;
        if (fyp < fy_min) fy_min = fyp;
        if (fyp > fy_max) fy_max = fyp;
    }
    if (all_behind || outside[0] || outside[1] || outside[2] || outside[3]) return 0;
    const double W = cam->width, H = cam->height;
    if (full)
    {
        *x0 = 0; *x1 = (int32_t)cam->width - 1; *y0 = 0; *y1 = (int32_t)cam->height - 1;
        return 1;
    }
    /* fx = (x+0.5)/W, fy = 1 - (y+0.5)/H */
    double xa = fx_min * W - 0.5 - margin, xb = fx_max * W - 0.5 + margin;
    double ya = (1.0 - fy_max) * H - 0.5 - margin, yb = (1.0 - fy_min) * H - 0.5 + margin;
    if (xb < 0.0 || ya > H - 1.0 || yb < 0.0 || xa > W - 1.0) return 0;
    if (xa < 0.0) xa = 0.0;
    if (ya < 0.0) ya = 0.0;
    if (xb > W - 1.0) xb = W - 1.0;
    if (yb > H - 1.0) yb = H - 1.0;
    *x0 = (int32_t)floor(xa); *x1 = (int32_t)ceil(xb);
    *y0 = (int32_t)floor(ya); *y1 = (int32_t)ceil(yb);
    return 1;
}

/*
 * The whole pass for one view: clear (clear.comp) then every fragment.
 * mode 0: every pixel x every cluster pointer; mode 1: conservative
 * per-cluster rectangles.  Only rows [row0, row1) are evaluated and written
 * (out still holds the full W*H frame).  Returns the number of pairs run.
 */
uint64_t oracle_vis_render(const tgx_object* objects, uint32_t n_cluster_pointers, const uint32_t* cluster_pointers,
                           const uint32_t* cluster_idx_to_object_idx, const uint32_t* voxel_bits,
                           const tgx_view* cam, uint64_t* out, int mode, uint32_t row0, uint32_t row1, int n_threads)
{
    const uint32_t W = cam->width, H = cam->height;
    if (row1 > H) row1 = H;
    for (uint64_t i = (uint64_t)row0 * W; i < (uint64_t)row1 * W; i++) out[i] = UINT64_MAX;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    uint64_t pairs = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+:pairs)
    for (int64_t cp = 0; cp < (int64_t)n_cluster_pointers; cp++)
    {
        const uint32_t cluster_idx = cluster_pointers[cp];
        const tgx_object* od = &objects[cluster_idx_to_object_idx[cluster_idx]];
        int32_t x0 = 0, x1 = (int32_t)W - 1, y0 = 0, y1 = (int32_t)H - 1;
        if (mode == 1)
        {
            /* a cluster without set bits never writes (the DDA finds nothing) */
            uint32_t any = 0;
            for (int w = 0; w < 16; w++) any |= voxel_bits[(uint64_t)cluster_idx * 16u + w];
            if (!any) continue;
            if (!cluster_rect(od, (uint32_t)cp - od->first_cluster_pointer, cam, 2, &x0, &x1, &y0, &y1)) continue;
        }
        if (y0 < (int32_t)row0) y0 = (int32_t)row0;
        if (y1 > (int32_t)row1 - 1) y1 = (int32_t)row1 - 1;
        for (int32_t y = y0; y <= y1; y++)
            for (int32_t x = x0; x <= x1; x++)
            {
                uint64_t v;
                pairs++;
                if (oracle_vis_pair(objects, cluster_pointers, cluster_idx_to_object_idx, voxel_bits, cam,
                                    (uint32_t)cp, (uint32_t)x, (uint32_t)y, &v))
                    atomic_min_u64(&out[(uint64_t)y * W + x], v);
            }
    }
    return pairs;
}

/* ---- exported primitives (pinned against the reference's own C functions) ---- */

void oracle_m4_inverse(const float* m, float* out) { or_m4_inverse(m, out); }
void oracle_m4_mul(const float* a, const float* b, float* out) { or_m4_mul(a, b, out); }
int oracle_ray_aabb(const float o[3], const float d[3], const float mn[3], const float mx[3], float* enter, float* exit_)
{
    return or_ray_aabb(o, d, mn, mx, enter, exit_);
}

/*
 * The cluster DDA of visibility.frag:78-191 alone, for a cluster-space ray
 * (o, d) against one cluster's 16 bit words.  Returns 1 and the first set
 * voxel (x, y, z), or 0.  Used to pin the transcription against the
 * reference's C DDA tg_amanatides_woo (tg_amanatides_woo.c:3-114) on rays
 * that start on the cluster's faces, where both walk the same cells.
 */
int oracle_cluster_dda(const float o[3], const float d[3], const uint32_t* words, int32_t out_xyz[3])
{
    const float cmin[3] = { 0.0f, 0.0f, 0.0f }, cmax[3] = { 8.0f, 8.0f, 8.0f };
    float enter, exit_;
    out_xyz[0] = out_xyz[1] = out_xyz[2] = -1;
    if (!or_ray_cluster(o, d, cmin, cmax, &enter, &exit_)) return 0;
    float hit[3], xyz[3];
    for (int i = 0; i < 3; i++)
    {
        hit[i] = enter > 0.0f ? o[i] + enter * d[i] : o[i];
        xyz[i] = or_gmin(or_gmax(floorf(hit[i]), 0.0f), 7.0f);
    }
    int32_t p[3] = { (int32_t)xyz[0], (int32_t)xyz[1], (int32_t)xyz[2] };
    int32_t step[3] = { 0, 0, 0 };
    float tmax[3] = { OR_F32_MAX, OR_F32_MAX, OR_F32_MAX }, tdel[3] = { OR_F32_MAX, OR_F32_MAX, OR_F32_MAX };
    for (int i = 0; i < 3; i++)
    {
        if (d[i] > 0.0f) { step[i] = 1; tmax[i] = enter + ((float)(p[i] + 1) - hit[i]) / d[i]; tdel[i] = 1.0f / d[i]; }
        else if (d[i] < 0.0f) { step[i] = -1; tmax[i] = enter + (hit[i] - (float)p[i]) / -d[i]; tdel[i] = 1.0f / -d[i]; }
    }
    for (;;)
    {
        const uint32_t rvi = 64u * (uint32_t)p[2] + 8u * (uint32_t)p[1] + (uint32_t)p[0];
        if (words[rvi / 32u] & (1u << (rvi % 32u)))
        {
            out_xyz[0] = p[0]; out_xyz[1] = p[1]; out_xyz[2] = p[2];
            return 1;
        }
        int a;
        if (tmax[0] < tmax[1]) a = tmax[0] < tmax[2] ? 0 : 2;
        else a = tmax[1] < tmax[2] ? 1 : 2;
        tmax[a] += tdel[a];
        p[a] += step[a];
        if (p[a] < 0 || p[a] >= 8) return 0;
    }
}
