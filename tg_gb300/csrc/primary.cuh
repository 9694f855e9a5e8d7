// primary.cuh -- decode of a visibility word into its primary surface point.
//
// Follows shading.frag:116-228: the packed word gives the depth field, the
// cluster pointer and the voxel; the shader rebuilds the cluster-space ray
// (the same ws2ms and origin as the visibility pass), intersects the voxel box
// and takes the dominant axis of (hit point - voxel centre) as the face normal,
// rotated to world space.  Every step is an exactly rounded binary32 operation
// in the order of the CPU oracle, so GI and shading results are bit-exact.
#pragma once

#include "tgx_internal.cuh"

struct PrimarySurface
{
    float depth;          // depth field / (2^24 - 1)
    uint32_t ptr, voxel, ci, oi;
    uint32_t mat_byte;    // material index byte of the voxel (0 without a material grid)
    bool box_hit;         // the voxel box was hit in cluster space (else nw is 0)
    float nw[3];          // world face normal (0 when box_hit is false)
    float dws[3];         // corner-lerped pixel ray (not normalised, common.inc:40-46)
    float dn[3];          // dws normalised
    float te;             // entry distance along dn (0 when the camera is inside the voxel)
    float albedo[3];      // LUT albedo of the voxel (0.5 grey without materials)
};

// false for a sky pixel
__device__ __forceinline__ bool primary_surface(const tgx_object* __restrict__ objects,
                                                const uint32_t* __restrict__ cluster_pointers,
                                                const uint32_t* __restrict__ c2o, const uint8_t* __restrict__ material,
                                                const tgx_material* __restrict__ luts, const tgx_view& cam,
                                                unsigned long long word, uint32_t px, uint32_t py, PrimarySurface& ps)
{
    const float fx = xdiv(xadd((float)px, 0.5f), (float)cam.width);
    const float fy = xsub(1.0f, xdiv(xadd((float)py, 0.5f), (float)cam.height));
    ps.depth = xdiv((float)(word >> 40), 16777215.0f);
    if (!(ps.depth < 1.0f)) return false;
    const uint32_t ptr = (uint32_t)(word >> 9) & 2147483647u;
    const uint32_t voxel = (uint32_t)word & 511u;
    const uint32_t ci = cluster_pointers[ptr];
    const uint32_t oi = c2o[ci];
    ps.ptr = ptr; ps.voxel = voxel; ps.ci = ci; ps.oi = oi;
    const tgx_object& od = objects[oi];
    const uint32_t nx = od.n_cluster_pointers_per_dim[0], ny = od.n_cluster_pointers_per_dim[1];
    const uint32_t rel = ptr - od.first_cluster_pointer;
    const float offx = (float)((rel % nx) * 8u), offy = (float)(((rel / nx) % ny) * 8u), offz = (float)((rel / (nx * ny)) * 8u);
    const float half = xmul(8.0f, 0.5f);
    float rot[16], m0[16], m1[16], m2[16], m3[16], ws2ms[16];
#pragma unroll
    for (int k = 0; k < 16; k++) rot[k] = od.rotation[k];
    dm4_translate(-od.translation[0], -od.translation[1], -od.translation[2], m0);
    dm4_inverse(rot, m1);
    dm4_translate(xmul(half, (float)od.n_cluster_pointers_per_dim[0]), xmul(half, (float)od.n_cluster_pointers_per_dim[1]),
                  xmul(half, (float)od.n_cluster_pointers_per_dim[2]), m2);
    dm4_translate(-offx, -offy, -offz, m3);
    dm4_mul(m3, m2, ws2ms);
    dm4_mul(ws2ms, m1, ws2ms);
    dm4_mul(ws2ms, m0, ws2ms);
    float o4[3];
    dm4_mulv4(ws2ms, cam.camera[0], cam.camera[1], cam.camera[2], 1.0f, o4);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float aa = xadd(xmul(cam.ray_bl[i], xsub(1.0f, fy)), xmul(cam.ray_tl[i], fy));
        const float bb = xadd(xmul(cam.ray_br[i], xsub(1.0f, fy)), xmul(cam.ray_tr[i], fy));
        ps.dws[i] = xadd(xmul(aa, xsub(1.0f, fx)), xmul(bb, fx));
    }
    float d4[3];
    dm4_mulv4(ws2ms, ps.dws[0], ps.dws[1], ps.dws[2], 0.0f, d4);
    const float mag = xsqrt(xadd(xadd(xmul(d4[0], d4[0]), xmul(d4[1], d4[1])), xmul(d4[2], d4[2])));
    const float dm[3] = {xdiv(d4[0], mag), xdiv(d4[1], mag), xdiv(d4[2], mag)};
    const float vmin[3] = {(float)(voxel % 8u), (float)((voxel / 8u) % 8u), (float)(voxel / 64u)};
    float enter, exit_;
    ps.nw[0] = ps.nw[1] = ps.nw[2] = 0.0f;
    ps.box_hit = ray_aabb(o4[0], o4[1], o4[2], dm[0], dm[1], dm[2], vmin[0], vmin[1], vmin[2], xadd(vmin[0], 1.0f),
                          xadd(vmin[1], 1.0f), xadd(vmin[2], 1.0f), enter, exit_);
    if (ps.box_hit) {
        float nm[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float hm = enter > 0.0f ? xadd(o4[i], xmul(enter, dm[i])) : o4[i];
            nm[i] = xsub(hm, xadd(vmin[i], 0.5f));
        }
        auto sgn = [](float v) { return v > 0.0f ? 1.0f : v < 0.0f ? -1.0f : 0.0f; };
        if (fabsf(nm[0]) > fabsf(nm[1])) {
            nm[1] = 0.0f;
            if (fabsf(nm[0]) > fabsf(nm[2])) { nm[0] = sgn(nm[0]); nm[2] = 0.0f; }
            else { nm[2] = sgn(nm[2]); nm[0] = 0.0f; }
        } else {
            nm[0] = 0.0f;
            if (fabsf(nm[1]) > fabsf(nm[2])) { nm[1] = sgn(nm[1]); nm[2] = 0.0f; }
            else { nm[2] = sgn(nm[2]); nm[1] = 0.0f; }
        }
        float r4[3];
        dm4_mulv4(rot, nm[0], nm[1], nm[2], 0.0f, r4);
        const float rl = xsqrt(xadd(xadd(xmul(r4[0], r4[0]), xmul(r4[1], r4[1])), xmul(r4[2], r4[2])));
        if (rl > 0.0f) { ps.nw[0] = xdiv(r4[0], rl); ps.nw[1] = xdiv(r4[1], rl); ps.nw[2] = xdiv(r4[2], rl); }
    }
    const float dl = xsqrt(xadd(xadd(xmul(ps.dws[0], ps.dws[0]), xmul(ps.dws[1], ps.dws[1])), xmul(ps.dws[2], ps.dws[2])));
#pragma unroll
    for (int i = 0; i < 3; i++) ps.dn[i] = xdiv(ps.dws[i], dl);
    ps.te = ps.box_hit && enter > 0.0f ? enter : 0.0f;
    ps.albedo[0] = ps.albedo[1] = ps.albedo[2] = 0.5f;
    ps.mat_byte = 0;
    if (material) ps.mat_byte = material[(uint64_t)ci * 512u + voxel];
    if (material && luts) {
        const tgx_material& m = luts[od.lut_idx * 256u + ps.mat_byte];
        ps.albedo[0] = m.albedo[0]; ps.albedo[1] = m.albedo[1]; ps.albedo[2] = m.albedo[2];
    }
    return true;
}
