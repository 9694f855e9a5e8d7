// gi.cu -- plain SVO bounce lighting (GI) from the visibility buffer.
//
// The reference has no GI pass: shading.frag:285-316 shades with one constant
// light and an ambient term, and its only secondary rays are a disabled CPU
// debug probe (tgvk_raytracer.c:1390-1434).  This pass defines the bounce
// lighting the SVO was built for (README.md:46-48), with the semantics of the
// CPU oracle (oracle/oracle_gi.c) and its exact operation order:
//
//   - the primary hit is decoded from the visibility word with shading.frag's
//     cluster-space hit point and face normal (:116-228), rotated to world;
//   - direct light: a directional sun, Lambertian albedo from the object's
//     LUT, visibility from an SVO shadow ray;
//   - indirect light: spp cosine-weighted rays (Malley's method, Duff et al.
//     basis) traced through the SVO; a miss sees the sky, a hit adds the sun
//     light arriving there (with its own shadow ray) and, for 2 bounces, one
//     more cosine-weighted ray from that hit;
//   - random numbers: Philox4x32-10 keyed by the seed, counter (pixel, sample,
//     bounce | frame << 8, draw).
//
// One thread per pixel.  Results equal the oracle's bit for bit.

#include "svo_trace.cuh"

namespace {

constexpr float kInvPi = 0.318309886f;
constexpr uint32_t kMaxBounces = 4;

struct GiParams
{
    uint32_t spp, bounces, max_steps, frame;
    unsigned long long seed;
    float sun_dir[3], sun_radiance[3], sky_radiance[3], offset;
};
static_assert(sizeof(GiParams) == sizeof(tgx_gi_params), "GI parameter layout");

__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0;
        const uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[1] = lo1;
        c[3] = lo0;
        c[0] = n0;
        c[2] = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

__device__ __forceinline__ float u01(uint32_t x) { return xmul((float)(x >> 8), 1.0f / 16777216.0f); }

__device__ void sample_cosine(const float n[3], uint32_t pixel, uint32_t sample, uint32_t bounce, const GiParams& p,
                              float out[3])
{
    const float sign = n[2] >= 0.0f ? 1.0f : -1.0f;
    const float a = xdiv(-1.0f, xadd(sign, n[2]));
    const float b = xmul(xmul(n[0], n[1]), a);
    const float t1[3] = {xadd(1.0f, xmul(xmul(xmul(sign, n[0]), n[0]), a)), xmul(sign, b), xmul(-sign, n[0])};
    const float t2[3] = {b, xadd(sign, xmul(xmul(n[1], n[1]), a)), -n[1]};
    for (uint32_t draw = 0; draw < 8; draw++) {
        uint32_t c[4] = {pixel, sample, bounce | (p.frame << 8), draw};
        philox(c, (uint32_t)p.seed, (uint32_t)(p.seed >> 32));
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const float u = xsub(xmul(2.0f, u01(c[2 * k])), 1.0f);
            const float v = xsub(xmul(2.0f, u01(c[2 * k + 1])), 1.0f);
            const float r2 = xadd(xmul(u, u), xmul(v, v));
            if (r2 < 1.0f) {
                const float z = xsqrt(xsub(1.0f, r2));
#pragma unroll
                for (int i = 0; i < 3; i++) out[i] = xadd(xadd(xmul(u, t1[i]), xmul(v, t2[i])), xmul(z, n[i]));
                return;
            }
        }
    }
    out[0] = n[0]; out[1] = n[1]; out[2] = n[2];
}

__device__ __forceinline__ void svo_albedo(const SvoDev& s, const int32_t c[3], const tgx_material* luts, float out[3])
{
    const uint32_t code = svo_material(s, c[0], c[1], c[2]);
    if (!code || !luts) { out[0] = out[1] = out[2] = 0.5f; return; }
    const tgx_material& m = luts[code - 1u];
    out[0] = m.albedo[0]; out[1] = m.albedo[1]; out[2] = m.albedo[2];
}

__device__ void direct_sun(const SvoDev& s, const float o2[3], const float n[3], const float a[3], const GiParams& p,
                           uint32_t* exhausted, float out[3])
{
    out[0] = out[1] = out[2] = 0.0f;
    const float ndl = xadd(xadd(xmul(n[0], p.sun_dir[0]), xmul(n[1], p.sun_dir[1])), xmul(n[2], p.sun_dir[2]));
    if (!(ndl > 0.0f)) return;
    float t; int32_t c[3], ax; uint32_t stp;
    const int r = svo_trace(s, o2, p.sun_dir, p.max_steps, t, c, ax, stp);
    if (r < 0) atomicAdd(exhausted, 1u);
    if (r == 1) return;
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = xmul(xmul(xmul(a[i], kInvPi), p.sun_radiance[i]), ndl);
}

// radiance arriving at o along w, for the rest of a path that has used `bounce` bounces
__device__ void incoming(const SvoDev& s, const float o_in[3], const float w_in[3], uint32_t pixel, uint32_t sample,
                         const tgx_material* luts, const GiParams& p, uint32_t* exhausted, float out[3])
{
    float D[kMaxBounces][3], A[kMaxBounces][3];
    float o[3] = {o_in[0], o_in[1], o_in[2]}, w[3] = {w_in[0], w_in[1], w_in[2]};
    int hits = 0;
    bool missed = false;
    for (uint32_t bounce = 0; bounce < p.bounces; bounce++) {
        float t; int32_t c[3], ax; uint32_t stp;
        const int r = svo_trace(s, o, w, p.max_steps, t, c, ax, stp);
        if (r < 0) atomicAdd(exhausted, 1u);
        if (r != 1) { missed = true; break; }
        float n2[3] = {0.0f, 0.0f, 0.0f};
        if (ax >= 0) {
            n2[ax] = w[ax] > 0.0f ? -1.0f : 1.0f;
        } else {
            int m = 0;
            if (fabsf(w[1]) > fabsf(w[m])) m = 1;
            if (fabsf(w[2]) > fabsf(w[m])) m = 2;
            n2[m] = w[m] > 0.0f ? -1.0f : 1.0f;
        }
        svo_albedo(s, c, luts, A[hits]);
        float o3[3];
#pragma unroll
        for (int i = 0; i < 3; i++) o3[i] = xadd(xadd(o[i], xmul(t, w[i])), xmul(n2[i], p.offset));
        direct_sun(s, o3, n2, A[hits], p, exhausted, D[hits]);
        hits++;
        if (bounce + 1 < p.bounces) {
            sample_cosine(n2, pixel, sample, bounce + 1, p, w);
            o[0] = o3[0]; o[1] = o3[1]; o[2] = o3[2];
        }
    }
    // innermost value, then outward: value = D + A * value
    float v[3];
    int j;
    if (missed) {
        v[0] = p.sky_radiance[0]; v[1] = p.sky_radiance[1]; v[2] = p.sky_radiance[2];
        j = hits - 1;
    } else {
        v[0] = D[hits - 1][0]; v[1] = D[hits - 1][1]; v[2] = D[hits - 1][2];
        j = hits - 2;
    }
    for (; j >= 0; j--)
#pragma unroll
        for (int i = 0; i < 3; i++) v[i] = xadd(D[j][i], xmul(A[j][i], v[i]));
    out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
}

// Primary hit of a pixel from its visibility word (shading.frag:116-228):
// returns false for sky; else the offset origin o2, world normal nw and albedo a.
__device__ bool primary_hit(const tgx_object* __restrict__ objects, const uint32_t* __restrict__ cluster_pointers,
                            const uint32_t* __restrict__ c2o, const uint8_t* __restrict__ material,
                            const tgx_material* __restrict__ luts, const tgx_view& cam, const GiParams& p,
                            unsigned long long word, uint32_t px, uint32_t py, float o2[3], float nw[3], float a[3])
{
    const float fx = xdiv(xadd((float)px, 0.5f), (float)cam.width);
    const float fy = xsub(1.0f, xdiv(xadd((float)py, 0.5f), (float)cam.height));
    const float depth = xdiv((float)(word >> 40), 16777215.0f);
    if (!(depth < 1.0f)) return false;
    const uint32_t ptr = (uint32_t)(word >> 9) & 2147483647u;
    const uint32_t voxel = (uint32_t)word & 511u;
    const uint32_t ci = cluster_pointers[ptr];
    const tgx_object& od = objects[c2o[ci]];
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
    float dws[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float aa = xadd(xmul(cam.ray_bl[i], xsub(1.0f, fy)), xmul(cam.ray_tl[i], fy));
        const float bb = xadd(xmul(cam.ray_br[i], xsub(1.0f, fy)), xmul(cam.ray_tr[i], fy));
        dws[i] = xadd(xmul(aa, xsub(1.0f, fx)), xmul(bb, fx));
    }
    float d4[3];
    dm4_mulv4(ws2ms, dws[0], dws[1], dws[2], 0.0f, d4);
    const float mag = xsqrt(xadd(xadd(xmul(d4[0], d4[0]), xmul(d4[1], d4[1])), xmul(d4[2], d4[2])));
    const float dm[3] = {xdiv(d4[0], mag), xdiv(d4[1], mag), xdiv(d4[2], mag)};
    const float vmin[3] = {(float)(voxel % 8u), (float)((voxel / 8u) % 8u), (float)(voxel / 64u)};
    float enter, exit_;
    nw[0] = nw[1] = nw[2] = 0.0f;
    const bool hit = ray_aabb(o4[0], o4[1], o4[2], dm[0], dm[1], dm[2], vmin[0], vmin[1], vmin[2], xadd(vmin[0], 1.0f),
                              xadd(vmin[1], 1.0f), xadd(vmin[2], 1.0f), enter, exit_);
    if (hit) {
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
        if (rl > 0.0f) { nw[0] = xdiv(r4[0], rl); nw[1] = xdiv(r4[1], rl); nw[2] = xdiv(r4[2], rl); }
    }
    const float dl = xsqrt(xadd(xadd(xmul(dws[0], dws[0]), xmul(dws[1], dws[1])), xmul(dws[2], dws[2])));
    const float dn[3] = {xdiv(dws[0], dl), xdiv(dws[1], dl), xdiv(dws[2], dl)};
    if (nw[0] == 0.0f && nw[1] == 0.0f && nw[2] == 0.0f) { nw[0] = -dn[0]; nw[1] = -dn[1]; nw[2] = -dn[2]; }
    const float te = hit && enter > 0.0f ? enter : 0.0f;
    a[0] = a[1] = a[2] = 0.5f;
    if (material && luts) {
        const tgx_material& m = luts[od.lut_idx * 256u + material[(uint64_t)ci * 512u + voxel]];
        a[0] = m.albedo[0]; a[1] = m.albedo[1]; a[2] = m.albedo[2];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) o2[i] = xadd(xadd(cam.camera[i], xmul(te, dn[i])), xmul(nw[i], p.offset));
    return true;
}

__global__ void __launch_bounds__(128) k_gi(SvoDev s, const tgx_object* __restrict__ objects,
                                           const uint32_t* __restrict__ cluster_pointers,
                                           const uint32_t* __restrict__ c2o, const uint8_t* __restrict__ material,
                                           const tgx_material* __restrict__ luts, tgx_view cam, GiParams p,
                                           const unsigned long long* __restrict__ visbuf, float* __restrict__ out,
                                           uint32_t* __restrict__ exhausted)
{
    const uint32_t px = blockIdx.x * 16 + (threadIdx.x & 15u);
    const uint32_t py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= cam.width || py >= cam.height) return;
    const uint32_t pixel = py * cam.width + px;
    float* res = out + 3ull * pixel;
    float o2[3], nw[3], a[3];
    if (!primary_hit(objects, cluster_pointers, c2o, material, luts, cam, p, visbuf[pixel], px, py, o2, nw, a)) {
        res[0] = p.sky_radiance[0]; res[1] = p.sky_radiance[1]; res[2] = p.sky_radiance[2];
        return;
    }
    float L[3];
    direct_sun(s, o2, nw, a, p, exhausted, L);
    float acc[3] = {0.0f, 0.0f, 0.0f};
    for (uint32_t smp = 0; smp < p.spp; smp++) {
        float w[3], li[3];
        sample_cosine(nw, pixel, smp, 0, p, w);
        incoming(s, o2, w, pixel, smp, luts, p, exhausted, li);
#pragma unroll
        for (int i = 0; i < 3; i++) acc[i] = xadd(acc[i], li[i]);
    }
    const float inv_spp = xdiv(1.0f, (float)(p.spp ? p.spp : 1u));
#pragma unroll
    for (int i = 0; i < 3; i++) res[i] = xadd(L[i], xmul(a[i], xmul(acc[i], inv_spp)));
}

// ---------------------------------------------------------------------------
// learned-cache GI
// ---------------------------------------------------------------------------

struct CacheHit
{
    float p[3];      // hit point (world)
    float n[3];      // face normal
    float w[3];      // direction the bounce ray travelled
    int32_t c[3];    // grid voxel
};

struct CacheGiConst
{
    float box_min[3];
    float box_inv[3];    // 1 / (box_max - box_min)
    uint32_t n_train, train_spp;
};

__device__ __forceinline__ void cache_input(const CacheGiConst& q, const float p[3], const float n[3], const float w[3],
                                            float* x)
{
#pragma unroll
    for (int i = 0; i < 3; i++) {
        x[i] = fminf(fmaxf((p[i] - q.box_min[i]) * q.box_inv[i], 0.0f), 1.0f);
        x[3 + i] = n[i];
        x[6 + i] = -w[i];   // outgoing direction, toward the shading point
    }
}

// Pass 1: primary hit, direct light, bounce rays; hits become cache queries.
__global__ void __launch_bounds__(128) k_gi_cache_queries(
    SvoDev s, const tgx_object* __restrict__ objects, const uint32_t* __restrict__ cluster_pointers,
    const uint32_t* __restrict__ c2o, const uint8_t* __restrict__ material, const tgx_material* __restrict__ luts,
    tgx_view cam, GiParams p, CacheGiConst q, const unsigned long long* __restrict__ visbuf,
    float* __restrict__ pix_state /* W*H*6: direct L, albedo */, int32_t* __restrict__ qidx /* W*H*spp */,
    float* __restrict__ qx /* n*9 */, CacheHit* __restrict__ hits, uint32_t* __restrict__ counters,
    uint32_t capacity, uint32_t* __restrict__ exhausted)
{
    const uint32_t px = blockIdx.x * 16 + (threadIdx.x & 15u);
    const uint32_t py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= cam.width || py >= cam.height) return;
    const uint32_t pixel = py * cam.width + px;
    float* st = pix_state + 6ull * pixel;
    int32_t* qi = qidx + (uint64_t)pixel * p.spp;
    float o2[3], nw[3], a[3];
    if (!primary_hit(objects, cluster_pointers, c2o, material, luts, cam, p, visbuf[pixel], px, py, o2, nw, a)) {
        st[0] = p.sky_radiance[0]; st[1] = p.sky_radiance[1]; st[2] = p.sky_radiance[2];
        st[3] = st[4] = st[5] = -1.0f;   // sky marker
        for (uint32_t k = 0; k < p.spp; k++) qi[k] = -1;
        return;
    }
    float L[3];
    direct_sun(s, o2, nw, a, p, exhausted, L);
    st[0] = L[0]; st[1] = L[1]; st[2] = L[2];
    st[3] = a[0]; st[4] = a[1]; st[5] = a[2];
    for (uint32_t smp = 0; smp < p.spp; smp++) {
        float w[3];
        sample_cosine(nw, pixel, smp, 0, p, w);
        float t; int32_t c[3], ax; uint32_t stp;
        const int r = svo_trace(s, o2, w, p.max_steps, t, c, ax, stp);
        if (r < 0) atomicAdd(exhausted, 1u);
        if (r != 1) { qi[smp] = -1; continue; }
        float n2[3] = {0.0f, 0.0f, 0.0f};
        if (ax >= 0) n2[ax] = w[ax] > 0.0f ? -1.0f : 1.0f;
        else {
            int m = 0;
            if (fabsf(w[1]) > fabsf(w[m])) m = 1;
            if (fabsf(w[2]) > fabsf(w[m])) m = 2;
            n2[m] = w[m] > 0.0f ? -1.0f : 1.0f;
        }
        const uint32_t slot = atomicAdd(&counters[0], 1u);
        if (slot >= capacity) { qi[smp] = -2; continue; }
        qi[smp] = (int32_t)slot;
        CacheHit h;
#pragma unroll
        for (int i = 0; i < 3; i++) {
            h.p[i] = xadd(o2[i], xmul(t, w[i]));
            h.n[i] = n2[i];
            h.w[i] = w[i];
            h.c[i] = c[i];
        }
        hits[slot] = h;
        cache_input(q, h.p, h.n, h.w, qx + 9ull * slot);
    }
}

// Pass 3: pixel = direct + albedo * mean(sky or cache prediction).
__global__ void __launch_bounds__(256) k_gi_cache_resolve(uint32_t n_pixels, GiParams p,
                                                         const float* __restrict__ pix_state,
                                                         const int32_t* __restrict__ qidx,
                                                         const float* __restrict__ qrgb, float* __restrict__ out)
{
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= n_pixels) return;
    const float* st = pix_state + 6ull * pixel;
    float* res = out + 3ull * pixel;
    if (st[3] < 0.0f) { res[0] = st[0]; res[1] = st[1]; res[2] = st[2]; return; }
    float acc[3] = {0.0f, 0.0f, 0.0f};
    for (uint32_t k = 0; k < p.spp; k++) {
        const int32_t q = qidx[(uint64_t)pixel * p.spp + k];
#pragma unroll
        for (int i = 0; i < 3; i++)
            acc[i] = xadd(acc[i], q >= 0 ? fmaxf(qrgb[3ull * q + i], 0.0f) : (q == -1 ? p.sky_radiance[i] : 0.0f));
    }
    const float inv_spp = xdiv(1.0f, (float)(p.spp ? p.spp : 1u));
#pragma unroll
    for (int i = 0; i < 3; i++) res[i] = xadd(st[i], xmul(st[3 + i], xmul(acc[i], inv_spp)));
}

// Training targets: radiance leaving a bounce hit toward where its ray came
// from, estimated with train_spp plain SVO paths (bounces-1 further bounces).
__global__ void __launch_bounds__(128) k_gi_cache_targets(SvoDev s, const tgx_material* __restrict__ luts, GiParams p,
                                                         CacheGiConst q, const CacheHit* __restrict__ hits,
                                                         const uint32_t* __restrict__ counters, uint32_t capacity,
                                                         float* __restrict__ tx, float* __restrict__ tt,
                                                         uint32_t* __restrict__ exhausted)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.n_train) return;
    const uint32_t n_hits = min(counters[0], capacity);
    if (n_hits == 0) {
#pragma unroll
        for (int k = 0; k < 9; k++) tx[9ull * i + k] = 0.0f;
        tt[3ull * i] = tt[3ull * i + 1] = tt[3ull * i + 2] = 0.0f;
        return;
    }
    uint32_t ctr[4] = {i, 0x7fffffffu, p.frame, 0x5eedu};
    philox(ctr, (uint32_t)p.seed ^ 0xA5A5A5A5u, (uint32_t)(p.seed >> 32));
    const CacheHit h = hits[ctr[0] % n_hits];
    float a2[3];
    svo_albedo(s, h.c, luts, a2);
    float o3[3];
#pragma unroll
    for (int k = 0; k < 3; k++) o3[k] = xadd(h.p[k], xmul(h.n[k], p.offset));
    float D[3];
    direct_sun(s, o3, h.n, a2, p, exhausted, D);
    float acc[3] = {0.0f, 0.0f, 0.0f};
    GiParams pp = p;
    pp.bounces = p.bounces > 1 ? p.bounces - 1 : 1;
    pp.frame = p.frame | 0x800000u;   // decorrelated from the pixel streams
    for (uint32_t k = 0; k < q.train_spp; k++) {
        float w[3], li[3];
        sample_cosine(h.n, i, k, 0, pp, w);
        if (p.bounces > 1) {
            incoming(s, o3, w, i, k, luts, pp, exhausted, li);
        } else {
            li[0] = li[1] = li[2] = 0.0f;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) acc[c] = xadd(acc[c], li[c]);
    }
    const float inv = xdiv(1.0f, (float)(q.train_spp ? q.train_spp : 1u));
    float tgt[3];
#pragma unroll
    for (int c = 0; c < 3; c++) tgt[c] = xadd(D[c], xmul(a2[c], xmul(acc[c], inv)));
    cache_input(q, h.p, h.n, h.w, tx + 9ull * i);
    tt[3ull * i] = tgt[0]; tt[3ull * i + 1] = tgt[1]; tt[3ull * i + 2] = tgt[2];
}

}  // namespace

extern "C" tgx_status tgx_gi_render(tgx_ctx* c, const tgx_scene* sc, const tgx_svo* svo, const tgx_view* view,
                                    const uint64_t* d_visbuf, const tgx_gi_params* params, float* d_rgb)
{
    if (!c || !sc || !svo || !view || !d_visbuf || !params || !d_rgb) {
        tgx_set_error("tgx_gi_render: NULL argument");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (view->width == 0 || view->height == 0) { tgx_set_error("tgx_gi_render: empty view"); return TGX_ERR_INVALID_ARGUMENT; }
    if (params->bounces < 1 || params->bounces > kMaxBounces) {
        tgx_set_error("tgx_gi_render: bounces must be 1..%u", kMaxBounces);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    GiParams p;
    memcpy(&p, params, sizeof(p));
    if (p.max_steps == 0) p.max_steps = 256;
    TGX_TRY(devbuf_reserve(c->svo_counters, 4 * 4 + 64));
    uint32_t* exhausted = (uint32_t*)c->svo_counters.ptr + 8;
    const dim3 grid((view->width + 15) / 16, (view->height + 7) / 8);
    TGX_LAUNCH(c, TR_GI, grid, 128, 0, k_gi, svo_dev(svo), sc->d_objects, sc->d_cluster_pointers, sc->d_c2o,
               sc->d_material, sc->d_luts, *view, p, (const unsigned long long*)d_visbuf, d_rgb, exhausted);
    return TGX_OK;
}

extern "C" tgx_status tgx_gi_render_cached(tgx_ctx* c, const tgx_scene* sc, const tgx_svo* svo, tgx_cache* cache,
                                           const tgx_view* view, const uint64_t* d_visbuf,
                                           const tgx_gi_params* params, const tgx_cache_gi_params* cp, float* d_rgb)
{
    if (!c || !sc || !svo || !cache || !view || !d_visbuf || !params || !cp || !d_rgb) {
        tgx_set_error("tgx_gi_render_cached: NULL argument");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (view->width == 0 || view->height == 0 || params->spp == 0 || params->bounces < 1 || params->bounces > kMaxBounces) {
        tgx_set_error("tgx_gi_render_cached: bad view or parameters");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    GiParams p;
    memcpy(&p, params, sizeof(p));
    if (p.max_steps == 0) p.max_steps = 256;
    CacheGiConst q;
    for (int i = 0; i < 3; i++) {
        const float ext = cp->box_max[i] - cp->box_min[i];
        if (!(ext > 0.0f)) { tgx_set_error("tgx_gi_render_cached: empty scene box"); return TGX_ERR_INVALID_ARGUMENT; }
        q.box_min[i] = cp->box_min[i];
        q.box_inv[i] = 1.0f / ext;
    }
    q.n_train = cp->n_train;
    q.train_spp = cp->train_spp ? cp->train_spp : 16;
    const uint64_t n_pix = (uint64_t)view->width * view->height;
    const uint64_t capacity = n_pix * p.spp;
    if (capacity > 0x7fffffffull) { tgx_set_error("tgx_gi_render_cached: too many queries"); return TGX_ERR_CAPACITY; }
    const size_t bytes = n_pix * 6 * 4 + capacity * 4 + capacity * 9 * 4 + capacity * sizeof(CacheHit) + capacity * 3 * 4 +
                         (size_t)q.n_train * 12 * 4 + 256;
    TGX_TRY(devbuf_reserve(c->gi_scratch, bytes));
    char* b = (char*)c->gi_scratch.ptr;
    uint32_t* counters = (uint32_t*)b; b += 256;
    float* pix_state = (float*)b; b += n_pix * 6 * 4;
    int32_t* qidx = (int32_t*)b; b += capacity * 4;
    float* qx = (float*)b; b += capacity * 9 * 4;
    float* qrgb = (float*)b; b += capacity * 3 * 4;
    CacheHit* hits = (CacheHit*)b; b += capacity * sizeof(CacheHit);
    float* tx = (float*)b; b += (size_t)q.n_train * 9 * 4;
    float* tt = (float*)b;
    TGX_TRY(devbuf_reserve(c->svo_counters, 4 * 4 + 64));
    uint32_t* exhausted = (uint32_t*)c->svo_counters.ptr + 8;
    TGX_CUDA(cudaMemsetAsync(counters, 0, 256, c->stream));
    const dim3 grid((view->width + 15) / 16, (view->height + 7) / 8);
    TGX_LAUNCH(c, TR_GI, grid, 128, 0, k_gi_cache_queries, svo_dev(svo), sc->d_objects, sc->d_cluster_pointers,
               sc->d_c2o, sc->d_material, sc->d_luts, *view, p, q, (const unsigned long long*)d_visbuf, pix_state, qidx,
               qx, hits, counters, (uint32_t)capacity, exhausted);
    // inference over all potential queries: unused slots past the hit count are never read
    TGX_TRY(cache_infer_counted(c, cache, counters, (uint32_t)capacity, qx, qrgb));
    TGX_LAUNCH(c, TR_GI, (uint32_t)((n_pix + 255) / 256), 256, 0, k_gi_cache_resolve, (uint32_t)n_pix, p, pix_state,
               qidx, qrgb, d_rgb);
    if (q.n_train && cp->train_steps) {
        TGX_LAUNCH(c, TR_GI, (q.n_train + 127) / 128, 128, 0, k_gi_cache_targets, svo_dev(svo), sc->d_luts, p, q, hits,
                   counters, (uint32_t)capacity, tx, tt, exhausted);
        const uint32_t per = q.n_train / cp->train_steps;
        for (uint32_t k = 0; k < cp->train_steps && per; k++)
            TGX_TRY(tgx_cache_train_step(c, cache, per, tx + 9ull * per * k, tt + 3ull * per * k, cp->lr));
    }
    return TGX_OK;
}
