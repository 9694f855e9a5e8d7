// shade.cu -- the shading pass on the visibility buffer (shading.frag:116-316).
//
// One thread per pixel: the primary surface from the visibility word (the
// same decode as the GI pass), the material's LUT albedo, and tg's direct
// shading: GGX distribution, Smith/Schlick geometry and Schlick Fresnel with
// a fixed light normalize(0, 0.8, 0.3) of radiance 3, metallic 0.1, roughness
// 0.8, plus an ambient term 0.1 * albedo.  The shader's debug views (object,
// cluster, voxel and LUT-index hashes, depth, colour, normal, white shading)
// are the other modes.  Sky pixels are magenta, as in the shader.
//
// GLSL leaves the rounding of normalize, mix, clamp and pow to the driver;
// here they are pinned: normalize = three divisions by the length (tg's
// tgm_v3_normalized), pow(t, 5) = (t t)(t t) t, clamp and min/max with GLSL's
// comparisons.  The CPU oracle (oracle_shade_pixel) evaluates the same steps.

#include "primary.cuh"

namespace {

constexpr float kPi = 3.14159265358979323846f;   // TG_PI (common.inc)

__device__ __forceinline__ float dot3(const float* a, const float* b)
{
    return xadd(xadd(xmul(a[0], b[0]), xmul(a[1], b[1])), xmul(a[2], b[2]));
}

__device__ __forceinline__ void normalize3(const float* v, float* out)
{
    const float l = xsqrt(dot3(v, v));
    out[0] = xdiv(v[0], l); out[1] = xdiv(v[1], l); out[2] = xdiv(v[2], l);
}

// GLSL max(x, y) = x < y ? y : x and min(x, y) = y < x ? y : x
__device__ __forceinline__ float gl_max(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gl_min(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float clamp01(float x) { return gl_min(gl_max(x, 0.0f), 1.0f); }

__device__ __forceinline__ float ggx_distribution(float c_ndh, float roughness)
{
    const float a = xmul(roughness, roughness);
    const float a2 = xmul(a, a);
    float den = xadd(xmul(xmul(c_ndh, c_ndh), xsub(a2, 1.0f)), 1.0f);
    den = xmul(xmul(kPi, den), den);
    return xdiv(a2, den);
}

__device__ __forceinline__ float schlick_ggx(float n_dot_v, float roughness)
{
    const float r = xadd(roughness, 1.0f);
    const float k = xdiv(xmul(r, r), 8.0f);
    return xdiv(n_dot_v, xadd(xmul(n_dot_v, xsub(1.0f, k)), k));
}

__device__ __forceinline__ float fresnel_schlick(float u, float roughness)
{
    const float fl = xsub(1.0f, roughness);
    const float t = xsub(1.0f, u);
    const float t2 = xmul(t, t);
    return xadd(fl, xmul(xsub(1.0f, fl), xmul(xmul(t2, t2), t)));
}

// tg_shade (shading.frag:85-110)
__device__ void tg_shade(const float* n, const float* v, const float* l, const float* diffuse_albedo,
                         const float* specular_albedo, float metallic, float roughness, float radiance, float* out)
{
    float hv[3] = {xadd(v[0], l[0]), xadd(v[1], l[1]), xadd(v[2], l[2])}, h[3];
    normalize3(hv, h);
    const float c_hdn = clamp01(dot3(h, n));
    const float c_ldn = clamp01(dot3(n, l));
    const float c_ndv = clamp01(dot3(n, v));
    const float d = ggx_distribution(c_hdn, roughness);
    const float f = fresnel_schlick(c_ndv, roughness);
    const float g = xmul(schlick_ggx(c_ldn, roughness), schlick_ggx(c_ndv, roughness));
    const float dfg = xmul(xmul(d, f), g);
    const float den = xmul(xmul(4.0f, c_ndv), c_ldn);
    const float q = xdiv(dfg, gl_max(den, 0.001f));
    const float kd = xmul(xsub(1.0f, f), xsub(1.0f, metallic));
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float spec = xmul(specular_albedo[i], q);
        const float diff = xdiv(xmul(kd, diffuse_albedo[i]), kPi);
        out[i] = xmul(xmul(xadd(diff, spec), radiance), c_ldn);
    }
}

// MurmurHash3 finaliser (util.inc:47-56)
__device__ __forceinline__ uint32_t hash_u32(uint32_t v)
{
    v ^= v >> 16;
    v *= 0x85ebca6bu;
    v ^= v >> 13;
    v *= 0xc2b2ae35u;
    v ^= v >> 16;
    return v;
}

__device__ __forceinline__ void hash_color(uint32_t v, float* out)
{
    const uint32_t h0 = hash_u32(v), h1 = hash_u32(h0), h2 = hash_u32(h1);
    out[0] = xdiv((float)h0, 4294967295.0f);
    out[1] = xdiv((float)h1, 4294967295.0f);
    out[2] = xdiv((float)h2, 4294967295.0f);
}

__global__ void __launch_bounds__(128) k_shade(const tgx_object* __restrict__ objects,
                                              const uint32_t* __restrict__ cluster_pointers,
                                              const uint32_t* __restrict__ c2o, const uint8_t* __restrict__ material,
                                              const tgx_material* __restrict__ luts, tgx_view cam,
                                              const unsigned long long* __restrict__ visbuf, uint32_t mode,
                                              float4* __restrict__ out)
{
    const uint32_t px = blockIdx.x * 16 + (threadIdx.x & 15u);
    const uint32_t py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= cam.width || py >= cam.height) return;
    const uint32_t pixel = py * cam.width + px;
    PrimarySurface ps;
    if (!primary_surface(objects, cluster_pointers, c2o, material, luts, cam, visbuf[pixel], px, py, ps)) {
        out[pixel] = make_float4(1.0f, 0.0f, 1.0f, 1.0f);
        return;
    }
    float c[3];
    switch (mode) {
    case TGX_SHADE_OBJECT_INDEX: hash_color(ps.oi, c); break;
    case TGX_SHADE_DEPTH: c[0] = c[1] = c[2] = gl_min(1.0f, xmul(8.0f, ps.depth)); break;
    case TGX_SHADE_CLUSTER_INDEX:
    case TGX_SHADE_BLOCKS: hash_color(ps.ci, c); break;
    case TGX_SHADE_VOXEL_INDEX: hash_color(ps.voxel, c); break;
    case TGX_SHADE_COLOR_LUT_INDEX: hash_color(ps.mat_byte, c); break;
    case TGX_SHADE_COLOR: c[0] = ps.albedo[0]; c[1] = ps.albedo[1]; c[2] = ps.albedo[2]; break;
    case TGX_SHADE_NORMAL:
#pragma unroll
        for (int i = 0; i < 3; i++) c[i] = xadd(xmul(ps.nw[i], 0.5f), 0.5f);
        break;
    default: {
        const float metallic = 0.1f, roughness = 0.8f, radiance = 3.0f;
        const float white[3] = {1.0f, 1.0f, 1.0f};
        const float* albedo = mode == TGX_SHADE_SHADING ? white : ps.albedo;
        const float dm = xmul(ps.depth, cam.far_plane);
        float vv[3], v[3], l[3], spec[3], lo[3];
#pragma unroll
        for (int i = 0; i < 3; i++) vv[i] = xsub(cam.camera[i], xadd(cam.camera[i], xmul(dm, ps.dws[i])));
        normalize3(vv, v);
        const float l0[3] = {0.0f, 0.8f, 0.3f};
        normalize3(l0, l);
#pragma unroll
        for (int i = 0; i < 3; i++) spec[i] = xadd(xmul(0.04f, xsub(1.0f, metallic)), xmul(albedo[i], metallic));
        tg_shade(ps.nw, v, l, albedo, spec, metallic, roughness, radiance, lo);
#pragma unroll
        for (int i = 0; i < 3; i++) c[i] = xadd(xmul(0.1f, albedo[i]), lo[i]);
    }
    }
    out[pixel] = make_float4(c[0], c[1], c[2], 1.0f);
}

}  // namespace

extern "C" tgx_status tgx_shade(tgx_ctx* c, const tgx_scene* sc, const tgx_view* view, const uint64_t* d_visbuf,
                                uint32_t mode, float* d_rgba)
{
    if (!c || !sc || !view || !d_visbuf || !d_rgba) { tgx_set_error("tgx_shade: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    if (view->width == 0 || view->height == 0 || mode > TGX_SHADE_SHADING) {
        tgx_set_error("tgx_shade: empty view or mode %u outside 0..%u", mode, (unsigned)TGX_SHADE_SHADING);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    const dim3 grid((view->width + 15) / 16, (view->height + 7) / 8);
    TGX_LAUNCH(c, TR_GI, grid, 128, 0, k_shade, sc->d_objects, sc->d_cluster_pointers, sc->d_c2o, sc->d_material,
               sc->d_luts, *view, (const unsigned long long*)d_visbuf, mode, (float4*)d_rgba);
    return TGX_OK;
}
