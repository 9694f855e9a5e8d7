/*
 * oracle_common.h -- shared helpers of the CPU oracle.
 *
 * TEST INFRASTRUCTURE.  The oracle restates the reference's arithmetic in
 * plain C (IEEE binary32, round-to-nearest, source order, no FMA contraction:
 * every file is compiled with -ffp-contract=off).  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg load it; the product never does.
 *
 * Matrices are column-major float[16] like tg's m4 (tg_math.h:240-275):
 * element (row r, column c) is m[4*c + r].
 */
#ifndef ORACLE_COMMON_H
#define ORACLE_COMMON_H

#include <stdint.h>
#include <string.h>
#include <math.h>

#include "../include/tgx.h"

#define OR_F32_MAX      3.402823466e+38f     /* TG_F32_MAX, common.inc:20 */
#define OR_F32_MIN      (-OR_F32_MAX)        /* TG_F32_MIN, common.inc:21 */
#define OR_F32_EPSILON  1.192092896e-07f     /* TG_F32_EPSILON, common.inc:23 */

#define OM(m, r, c) ((m)[4 * (c) + (r)])

/* GLSL min/max (GLSL 4.50 8.3): min(x,y) = y < x ? y : x, max(x,y) = x < y ? y : x. */
static inline float or_gmin(float x, float y) { return y < x ? y : x; }
static inline float or_gmax(float x, float y) { return x < y ? y : x; }

/* tgm_m4_mul, tg_math.c:2374-2399: each element summed over k = 0..3 left to right. */
static inline void or_m4_mul(const float* a, const float* b, float* out)
{
    float r[16];
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++)
            OM(r, row, c) = OM(a, row, 0) * OM(b, 0, c) + OM(a, row, 1) * OM(b, 1, c)
                          + OM(a, row, 2) * OM(b, 2, c) + OM(a, row, 3) * OM(b, 3, c);
    memcpy(out, r, sizeof(r));
}

/* tgm_m4_mulv4, tg_math.c:2428-2438. */
static inline void or_m4_mulv4(const float* m, const float v[4], float out[4])
{
    float r[4];
    for (int row = 0; row < 4; row++)
        r[row] = v[0] * OM(m, row, 0) + v[1] * OM(m, row, 1) + v[2] * OM(m, row, 2) + v[3] * OM(m, row, 3);
    memcpy(out, r, sizeof(r));
}

/* tgm_m4_translate, tg_math.c:2669-2694. */
static inline void or_m4_translate(float x, float y, float z, float* out)
{
    memset(out, 0, 16 * sizeof(float));
    OM(out, 0, 0) = 1.0f; OM(out, 1, 1) = 1.0f; OM(out, 2, 2) = 1.0f; OM(out, 3, 3) = 1.0f;
    OM(out, 0, 3) = x; OM(out, 1, 3) = y; OM(out, 2, 3) = z;
}

/* tgm_m4_inverse, tg_math.c:2185-2234 (cofactor expansion, det = 1/(...)).
 * m.mRC in the reference is row R, column C. */
static inline void or_m4_inverse(const float* m, float* out)
{
#define E(r, c) OM(m, r, c)
    const float m2323 = E(2,2) * E(3,3) - E(2,3) * E(3,2);
    const float m1323 = E(2,1) * E(3,3) - E(2,3) * E(3,1);
    const float m1223 = E(2,1) * E(3,2) - E(2,2) * E(3,1);
    const float m0323 = E(2,0) * E(3,3) - E(2,3) * E(3,0);
    const float m0223 = E(2,0) * E(3,2) - E(2,2) * E(3,0);
    const float m0123 = E(2,0) * E(3,1) - E(2,1) * E(3,0);
    const float m2313 = E(1,2) * E(3,3) - E(1,3) * E(3,2);
    const float m1313 = E(1,1) * E(3,3) - E(1,3) * E(3,1);
    const float m1213 = E(1,1) * E(3,2) - E(1,2) * E(3,1);
    const float m2312 = E(1,2) * E(2,3) - E(1,3) * E(2,2);
    const float m1312 = E(1,1) * E(2,3) - E(1,3) * E(2,1);
    const float m1212 = E(1,1) * E(2,2) - E(1,2) * E(2,1);
    const float m0313 = E(1,0) * E(3,3) - E(1,3) * E(3,0);
    const float m0213 = E(1,0) * E(3,2) - E(1,2) * E(3,0);
    const float m0312 = E(1,0) * E(2,3) - E(1,3) * E(2,0);
    const float m0212 = E(1,0) * E(2,2) - E(1,2) * E(2,0);
    const float m0113 = E(1,0) * E(3,1) - E(1,1) * E(3,0);
    const float m0112 = E(1,0) * E(2,1) - E(1,1) * E(2,0);
    const float det = 1.0f / (
        E(0,0) * (E(1,1) * m2323 - E(1,2) * m1323 + E(1,3) * m1223) -
        E(0,1) * (E(1,0) * m2323 - E(1,2) * m0323 + E(1,3) * m0223) +
        E(0,2) * (E(1,0) * m1323 - E(1,1) * m0323 + E(1,3) * m0123) -
        E(0,3) * (E(1,0) * m1223 - E(1,1) * m0223 + E(1,2) * m0123));
    float r[16];
    OM(r,0,0) = det *  (E(1,1) * m2323 - E(1,2) * m1323 + E(1,3) * m1223);
    OM(r,0,1) = det * -(E(0,1) * m2323 - E(0,2) * m1323 + E(0,3) * m1223);
    OM(r,0,2) = det *  (E(0,1) * m2313 - E(0,2) * m1313 + E(0,3) * m1213);
    OM(r,0,3) = det * -(E(0,1) * m2312 - E(0,2) * m1312 + E(0,3) * m1212);
    OM(r,1,0) = det * -(E(1,0) * m2323 - E(1,2) * m0323 + E(1,3) * m0223);
    OM(r,1,1) = det *  (E(0,0) * m2323 - E(0,2) * m0323 + E(0,3) * m0223);
    OM(r,1,2) = det * -(E(0,0) * m2313 - E(0,2) * m0313 + E(0,3) * m0213);
    OM(r,1,3) = det *  (E(0,0) * m2312 - E(0,2) * m0312 + E(0,3) * m0212);
    OM(r,2,0) = det *  (E(1,0) * m1323 - E(1,1) * m0323 + E(1,3) * m0123);
    OM(r,2,1) = det * -(E(0,0) * m1323 - E(0,1) * m0323 + E(0,3) * m0123);
    OM(r,2,2) = det *  (E(0,0) * m1313 - E(0,1) * m0313 + E(0,3) * m0113);
    OM(r,2,3) = det * -(E(0,0) * m1312 - E(0,1) * m0312 + E(0,3) * m0112);
    OM(r,3,0) = det * -(E(1,0) * m1223 - E(1,1) * m0223 + E(1,2) * m0123);
    OM(r,3,1) = det *  (E(0,0) * m1223 - E(0,1) * m0223 + E(0,2) * m0123);
    OM(r,3,2) = det * -(E(0,0) * m1213 - E(0,1) * m0213 + E(0,2) * m0113);
    OM(r,3,3) = det *  (E(0,0) * m1212 - E(0,1) * m0212 + E(0,2) * m0112);
#undef E
    memcpy(out, r, sizeof(r));
}

/* tg_intersect_ray_aabb: GLSL collide.inc:3-24 == C tg_physics.c:394-406
 * (tgm_v3_div_zero_check, tg_math.c:1044-1051).  Returns hit, writes enter/exit. */
static inline int or_ray_aabb(const float o[3], const float d[3], const float mn[3], const float mx[3],
                              float* enter, float* exit_)
{
    float v0[3], v1[3];
    for (int i = 0; i < 3; i++)
    {
        v0[i] = (d[i] == 0.0f) ? OR_F32_MIN : ((mn[i] - o[i]) / d[i]);
        v1[i] = (d[i] == 0.0f) ? OR_F32_MAX : ((mx[i] - o[i]) / d[i]);
    }
    const float nx = or_gmin(v0[0], v1[0]), ny = or_gmin(v0[1], v1[1]), nz = or_gmin(v0[2], v1[2]);
    const float fx = or_gmax(v0[0], v1[0]), fy = or_gmax(v0[1], v1[1]), fz = or_gmax(v0[2], v1[2]);
    *enter = or_gmax(or_gmax(nx, ny), nz);
    *exit_ = or_gmin(or_gmin(fx, fy), fz);
    return *exit_ > 0.0f && *enter <= *exit_;
}

/*
 * The cluster-box test of visibility.frag:78 as the raster pipeline applies
 * it: the shader only runs for pixels the box's rasterised faces cover
 * (tgvk_raytracer.c:1293, cluster_functions.inc:1-38), i.e. pixels whose ray
 * crosses the box.  collide.inc:5-10 substitutes -/+F32_MAX for an axis with a
 * zero direction component without checking that the origin lies inside that
 * slab, so on its own it would accept rays parallel to a slab they never
 * cross -- fragments the rasteriser never generates.  Those pairs are misses
 * here.  Everything else is or_ray_aabb, operation for operation.
 */
static inline int or_ray_cluster(const float o[3], const float d[3], const float mn[3], const float mx[3],
                                 float* enter, float* exit_)
{
    const int hit = or_ray_aabb(o, d, mn, mx, enter, exit_);
    for (int i = 0; i < 3; i++)
        if (d[i] == 0.0f && (o[i] < mn[i] || o[i] > mx[i])) return 0;
    return hit;
}

#endif
