// gi.cu -- SVO bounce lighting (GI) from the visibility buffer, plain and
// with the learned radiance cache.
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
//   - indirect light: spp cosine-weighted paths (Malley's method, Duff et al.
//     basis) of up to `bounces` SVO bounces, accumulated forward with their
//     throughput; a miss sees the sky, a hit adds the sun light arriving
//     there (with its own shadow ray);
//   - sample directions: a randomised R2 point set per (key, bounce) with
//     Philox4x32-10 rotations keyed by the seed, key = pixel index.
//
// Execution is a wavefront over path roots (one per geometry pixel, or one
// per training sample of the cache):
//
//   k_gi_roots      primary hits -> compacted roots; sky pixels written
//   k_gi_emit       first bounce ray of every (root, sample), root shadow rays
//   k_trace_queue   persistent SVO traversal of a ray list: each lane takes
//                   rays from a warp-aggregated queue and runs their DDA a few
//                   steps at a time, so a lane whose ray ends picks up the next
//                   ray instead of idling until the warp's longest ray is done
//   k_gi_shade      consumes the hits of one bounce: sky, or albedo + shadow
//                   ray + next bounce ray
//   k_gi_finish     last shadow results, per-root sums in sample order, output
//
// Results equal the oracle's bit for bit.

#include "primary.cuh"
#include "svo_trace.cuh"

#include <algorithm>

namespace {

constexpr float kInvPi = 0.318309886f;
constexpr uint32_t kMaxBounces = 4;
constexpr uint64_t kMaxPathsPerChunk = 16ull << 20;   // paths in flight per wavefront chunk

struct GiParams
{
    uint32_t spp, bounces, max_steps, frame;
    unsigned long long seed;
    float sun_dir[3], sun_radiance[3], sky_radiance[3], offset;
};
static_assert(sizeof(GiParams) == sizeof(tgx_gi_params), "GI parameter layout");

// Records of the wavefront passes, aligned so that a thread moves each with
// vector loads and stores (8 or 16 bytes) instead of one word at a time.
struct __align__(8) Ray
{
    float o[3], d[3];   // d = 0: no ray
};

struct __align__(8) RayHit
{
    float t;
    int32_t c[3];
    int32_t axis;
    int32_t res;        // 1 hit, 0 miss, -1 step budget ran out
};

struct __align__(8) PathRoot
{
    float o[3];         // offset surface point
    float n[3];         // normal
    float a[3];         // albedo for the root's direct term
    uint32_t key;       // Philox key and output index (pixel, or training sample)
};

struct __align__(16) PathState
{
    float v[3];         // radiance gathered so far
    float T[3];         // throughput
    float a[3];         // albedo of the last hit (its shadow ray is pending)
    float ndl;
    uint32_t flags;
    uint32_t pad;
};
enum : uint32_t { P_ALIVE = 1u, P_SHADOW = 2u };
static_assert(sizeof(Ray) == 24 && sizeof(RayHit) == 24 && sizeof(PathRoot) == 40 && sizeof(PathState) == 48,
              "record sizes: the alignment adds no padding");

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

// sin and cos on [-pi/4, pi/4]: Taylor series of degree 7 and 8 in Horner
// form with exactly rounded operations (the oracle evaluates the same steps)
__device__ __forceinline__ float sin_q(float x)
{
    const float x2 = xmul(x, x);
    return xmul(x, xadd(1.0f, xmul(x2, xadd(-0.16666667f, xmul(x2, xadd(0.0083333333f, xmul(x2, -0.00019841270f)))))));
}
__device__ __forceinline__ float cos_q(float x)
{
    const float x2 = xmul(x, x);
    return xadd(1.0f, xmul(x2, xadd(-0.5f, xmul(x2, xadd(0.041666668f,
                                                         xmul(x2, xadd(-0.0013888889f, xmul(x2, 0.000024801587f))))))));
}

// Cosine-weighted direction about unit n for sample `sample` of `key`:
// randomised quasi-Monte Carlo.  R2 point (Roberts 2018, 32-bit fixed point)
// at index `sample`, rotated by Philox counter (key, bounce, frame, tag);
// concentric map to the disk (Shirley and Chiu 1997), lifted to the
// hemisphere (Malley), in the basis of Duff et al. (2017).
__device__ void sample_cosine(const float n[3], uint32_t key, uint32_t sample, uint32_t bounce, const GiParams& p,
                              float out[3])
{
    const float sign = n[2] >= 0.0f ? 1.0f : -1.0f;
    const float a = xdiv(-1.0f, xadd(sign, n[2]));
    const float b = xmul(xmul(n[0], n[1]), a);
    const float t1[3] = {xadd(1.0f, xmul(xmul(xmul(sign, n[0]), n[0]), a)), xmul(sign, b), xmul(-sign, n[0])};
    const float t2[3] = {b, xadd(sign, xmul(xmul(n[1], n[1]), a)), -n[1]};
    uint32_t c[4] = {key, bounce, p.frame, 0x52325351u};
    philox(c, (uint32_t)p.seed, (uint32_t)(p.seed >> 32));
    const float u = xsub(xmul(2.0f, u01(sample * 3242174889u + c[0])), 1.0f);
    const float v = xsub(xmul(2.0f, u01(sample * 2447445413u + c[1])), 1.0f);
    float dx = 0.0f, dy = 0.0f;
    if (fabsf(u) > fabsf(v)) {
        const float phi = xmul(0.78539819f, xdiv(v, u));
        dx = xmul(u, cos_q(phi));
        dy = xmul(u, sin_q(phi));
    } else if (v != 0.0f) {
        const float phi = xmul(0.78539819f, xdiv(u, v));
        dx = xmul(v, sin_q(phi));
        dy = xmul(v, cos_q(phi));
    }
    const float r2 = xadd(xmul(dx, dx), xmul(dy, dy));
    const float z = r2 < 1.0f ? xsqrt(xsub(1.0f, r2)) : 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = xadd(xadd(xmul(dx, t1[i]), xmul(dy, t2[i])), xmul(z, n[i]));
}

__device__ __forceinline__ void svo_albedo(const SvoDev& s, const int32_t c[3], const tgx_material* luts, float out[3])
{
    const uint32_t code = svo_material(s, c[0], c[1], c[2]);
    if (!code || !luts) { out[0] = out[1] = out[2] = 0.5f; return; }
    const tgx_material& m = luts[code - 1u];
    out[0] = m.albedo[0]; out[1] = m.albedo[1]; out[2] = m.albedo[2];
}

// Primary hit of a pixel from its visibility word (shading.frag:116-228):
// returns false for sky; else the offset origin o2, world normal nw and albedo a.
__device__ bool primary_hit(const tgx_object* __restrict__ objects, const uint32_t* __restrict__ cluster_pointers,
                            const uint32_t* __restrict__ c2o, const uint8_t* __restrict__ material,
                            const tgx_material* __restrict__ luts, const tgx_view& cam, const GiParams& p,
                            unsigned long long word, uint32_t px, uint32_t py, float o2[3], float nw[3], float a[3])
{
    PrimarySurface ps;
    if (!primary_surface(objects, cluster_pointers, c2o, material, luts, cam, word, px, py, ps)) return false;
    // no voxel-box hit in cluster space: face the camera
    const bool none = ps.nw[0] == 0.0f && ps.nw[1] == 0.0f && ps.nw[2] == 0.0f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        nw[i] = none ? -ps.dn[i] : ps.nw[i];
        a[i] = ps.albedo[i];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) o2[i] = xadd(xadd(cam.camera[i], xmul(ps.te, ps.dn[i])), xmul(nw[i], p.offset));
    return true;
}

__device__ __forceinline__ float sun_cos(const float n[3], const GiParams& p)
{
    return xadd(xadd(xmul(n[0], p.sun_dir[0]), xmul(n[1], p.sun_dir[1])), xmul(n[2], p.sun_dir[2]));
}

// sun light reflected by a Lambertian surface of albedo a, unshadowed
__device__ __forceinline__ void sun_term(const float a[3], float ndl, const GiParams& p, float out[3])
{
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] = xmul(xmul(xmul(a[i], kInvPi), p.sun_radiance[i]), ndl);
}

__device__ __forceinline__ void set_ray(Ray& r, const float o[3], const float d[3])
{
    float2* q = reinterpret_cast<float2*>(&r);   // three 8-byte stores
    q[0] = make_float2(o[0], o[1]);
    q[1] = make_float2(o[2], d[0]);
    q[2] = make_float2(d[1], d[2]);
}

__device__ __forceinline__ void null_ray(Ray& r)
{
    float2* q = reinterpret_cast<float2*>(&r);
    q[0] = q[1] = q[2] = make_float2(0.0f, 0.0f);
}

// face normal of an SVO hit: the face crossed, or the dominant axis when the
// ray started inside the voxel
__device__ __forceinline__ void hit_normal(int32_t axis, const float d[3], float n2[3])
{
    int m = axis;
    if (m < 0) {
        m = fabsf(d[1]) > fabsf(d[0]) ? 1 : 0;
        if (fabsf(d[2]) > fabsf(m ? d[1] : d[0])) m = 2;
    }
#pragma unroll
    for (int i = 0; i < 3; i++) n2[i] = i == m ? (d[i] > 0.0f ? -1.0f : 1.0f) : 0.0f;
}

// Slot in an append buffer for every lane with want = true (one atomic per warp).
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want)
{
    const uint32_t active = __activemask();
    const uint32_t mask = __ballot_sync(active, want);
    if (!mask) return 0;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = __ffs(mask) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(active, base, leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void write_hit(RayHit* h, int res, const RayState& r)
{
    RayHit o;
    o.t = r.t;
    o.c[0] = r.c[0]; o.c[1] = r.c[1]; o.c[2] = r.c[2];
    o.axis = r.last_axis;
    o.res = res;
    *h = o;
}

// Persistent traversal of two ray lists: a (n * mul_a rays) then b (n * mul_b
// rays), n read from the device.  No CTA waits on another: a CTA that starts
// after the queue is drained exits at once.
//
// A warp sets rays up 32 at a time, one per lane, and parks the ones whose
// DDA has to run in a per-warp ring of 64 states in shared memory; a lane
// whose ray ended takes the next parked state.  The set-up (entry slab, the
// bottom-up start) then runs on full warps instead of on the few lanes that
// happen to need a ray at a refill.
constexpr uint32_t kTraceWarps = 4;     // 128 threads
constexpr uint32_t kRing = 64;          // parked states per warp

__global__ void __launch_bounds__(32 * kTraceWarps) k_trace_queue(SvoDev s, const Ray* __restrict__ ra,
                                                                  RayHit* __restrict__ ha, uint32_t mul_a,
                                                                  const Ray* __restrict__ rb, RayHit* __restrict__ hb,
                                                                  uint32_t mul_b, const uint32_t* __restrict__ n_dev,
                                                                  uint32_t max_steps, uint32_t steps_per_round,
                                                                  uint32_t* __restrict__ queue,
                                                                  uint32_t* __restrict__ exhausted,
                                                                  unsigned long long* __restrict__ work)
{
    __shared__ uint32_t occ_off[16];
    __shared__ LevelDesc lv[16];
    __shared__ uint8_t first_level[kFirstLevelSize];
    __shared__ RayState ring[kTraceWarps][kRing];
    __shared__ uint32_t ring_item[kTraceWarps][kRing];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < 16; i++) occ_off[i] = s.occ_off[i];
    }
    __syncthreads();
    svo_level_tables(s.L, s.NL, s.B, s.occ, s.pool, s.sub, occ_off, lv, first_level);
    __syncthreads();
    const uint32_t n = *n_dev;
    const uint32_t n_a = n * mul_a, n_tot = n_a + n * mul_b;
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    RayState r;
    uint32_t item = 0;
    bool have = false;
    uint32_t head = 0, count = 0;   // the warp's ring (warp-uniform)
    bool drained = false;           // the ray queue is exhausted (warp-uniform)
    uint32_t done_steps = 0, done_rays = 0;   // this lane's finished rays and their DDA steps
    for (;;) {
        const uint32_t need_mask = __ballot_sync(0xffffffffu, !have);
        const uint32_t n_need = (uint32_t)__popc(need_mask);
        // set up rays, 32 at a time, until the ring can serve every idle lane
        while (n_need && count < n_need && !drained) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(queue, 32u);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + 32u >= n_tot) drained = true;
            const uint32_t it = base + lane;
            bool running = false;
            RayState rs;
            if (it < n_tot) {
                const Ray ray = it < n_a ? ra[it] : rb[it - n_a];
                const int res = svo_trace_begin(s, occ_off, lv, ray.o, ray.d, max_steps, rs);
                if (res == kTraceRunning) {
                    running = true;
                } else {
                    write_hit(it < n_a ? &ha[it] : &hb[it - n_a], res, rs);
                    done_steps += rs.steps;
                    done_rays++;
                }
            }
            const uint32_t run_mask = __ballot_sync(0xffffffffu, running);
            if (running) {
                const uint32_t slot = (head + count + (uint32_t)__popc(run_mask & lt_mask)) & (kRing - 1u);
                ring[w][slot] = rs;
                ring_item[w][slot] = it;
            }
            count += (uint32_t)__popc(run_mask);
            __syncwarp();
        }
        // idle lanes take parked states in lane order
        const uint32_t take = min(n_need, count);
        if (!have) {
            const uint32_t rank = (uint32_t)__popc(need_mask & lt_mask);
            if (rank < take) {
                const uint32_t slot = (head + rank) & (kRing - 1u);
                r = ring[w][slot];
                item = ring_item[w][slot];
                have = true;
            }
        }
        head = (head + take) & (kRing - 1u);
        count -= take;
        __syncwarp();
        if (!__any_sync(0xffffffffu, have) && drained && count == 0) break;
        if (have) {
            const int res = svo_trace_run(s, lv, first_level, r, max_steps, steps_per_round);
            if (res != kTraceRunning) {
                if (res < 0) atomicAdd(exhausted, 1u);
                write_hit(item < n_a ? &ha[item] : &hb[item - n_a], res, r);
                done_steps += r.steps;
                done_rays++;
                have = false;
            }
        }
    }
    // the frame's traversal work: one pair of 64-bit atomics per warp
    unsigned long long ws = done_steps, wr = done_rays;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ws += __shfl_down_sync(0xffffffffu, ws, o);
        wr += __shfl_down_sync(0xffffffffu, wr, o);
    }
    if (lane == 0 && wr) {
        atomicAdd(&work[0], ws);
        atomicAdd(&work[1], wr);
    }
}

// Roots of the geometry pixels; sky pixels get the sky radiance.
__global__ void __launch_bounds__(128) k_gi_roots(const tgx_object* __restrict__ objects,
                                                  const uint32_t* __restrict__ cluster_pointers,
                                                  const uint32_t* __restrict__ c2o, const uint8_t* __restrict__ material,
                                                  const tgx_material* __restrict__ luts, tgx_view cam, GiParams p,
                                                  const unsigned long long* __restrict__ visbuf, float* __restrict__ out,
                                                  PathRoot* __restrict__ roots, uint32_t* __restrict__ n_roots)
{
    const uint32_t px = blockIdx.x * 16 + (threadIdx.x & 15u);
    const uint32_t py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= cam.width || py >= cam.height) return;
    const uint32_t pixel = py * cam.width + px;
    PathRoot rt;
    const bool geo = primary_hit(objects, cluster_pointers, c2o, material, luts, cam, p, visbuf[pixel], px, py, rt.o,
                                 rt.n, rt.a);
    if (!geo) {
        out[3ull * pixel + 0] = p.sky_radiance[0];
        out[3ull * pixel + 1] = p.sky_radiance[1];
        out[3ull * pixel + 2] = p.sky_radiance[2];
    }
    const uint32_t slot = warp_append(n_roots, geo);
    if (geo) {
        rt.key = pixel;
        roots[slot] = rt;
    }
}

// First bounce ray of every path (root r, sample s0 + j) of a chunk of cs
// samples; with root_rays, also the shadow ray of every root.
__global__ void __launch_bounds__(256) k_gi_emit(const PathRoot* __restrict__ roots, const uint32_t* __restrict__ n_dev,
                                                 uint32_t cs, uint32_t s0, GiParams p, Ray* __restrict__ rays,
                                                 PathState* __restrict__ st, Ray* __restrict__ root_rays)
{
    const uint32_t n = *n_dev;
    const uint64_t n_paths = (uint64_t)n * cs;
    const uint64_t n_items = n_paths + (root_rays ? n : 0u);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_items; i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < n_paths) {
            const uint32_t r = (uint32_t)i / cs;   // paths in flight < 2^32: 32-bit division
            const PathRoot& rt = roots[r];
            float w[3];
            sample_cosine(rt.n, rt.key, s0 + ((uint32_t)i - r * cs), 0, p, w);
            set_ray(rays[i], rt.o, w);
            if (!st) continue;   // first-bounce queries keep no path state
            PathState ps;
            ps.v[0] = ps.v[1] = ps.v[2] = 0.0f;
            ps.T[0] = ps.T[1] = ps.T[2] = 1.0f;
            ps.a[0] = ps.a[1] = ps.a[2] = 0.0f;
            ps.ndl = 0.0f;
            ps.flags = P_ALIVE;
            ps.pad = 0;
            st[i] = ps;
        } else {
            const uint32_t r = (uint32_t)(i - n_paths);
            const PathRoot& rt = roots[r];
            if (sun_cos(rt.n, p) > 0.0f) set_ray(root_rays[r], rt.o, p.sun_dir);
            else null_ray(root_rays[r]);
        }
    }
}

// Consumes the pending shadow ray of bounce k-1 and the hit of bounce k.
__global__ void __launch_bounds__(256) k_gi_shade(SvoDev s, const tgx_material* __restrict__ luts,
                                                  const PathRoot* __restrict__ roots, const uint32_t* __restrict__ n_dev,
                                                  uint32_t cs, uint32_t s0, uint32_t k, GiParams p,
                                                  Ray* __restrict__ rb, const RayHit* __restrict__ hb,
                                                  Ray* __restrict__ rs, const RayHit* __restrict__ hs,
                                                  PathState* __restrict__ st)
{
    const uint64_t n_paths = (uint64_t)(*n_dev) * cs;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_paths; i += (uint64_t)gridDim.x * blockDim.x) {
        PathState ps = st[i];
        if (ps.flags & P_SHADOW) {
            float D[3] = {0.0f, 0.0f, 0.0f};
            if (ps.ndl > 0.0f && hs[i].res != 1) sun_term(ps.a, ps.ndl, p, D);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                ps.v[c] = xadd(ps.v[c], xmul(ps.T[c], D[c]));
                ps.T[c] = xmul(ps.T[c], ps.a[c]);
            }
            ps.flags &= ~P_SHADOW;
        }
        Ray nb, ns;
        null_ray(nb);
        null_ray(ns);
        if (ps.flags & P_ALIVE) {
            const RayHit h = hb[i];
            const Ray ray = rb[i];
            if (h.res != 1) {
#pragma unroll
                for (int c = 0; c < 3; c++) ps.v[c] = xadd(ps.v[c], xmul(ps.T[c], p.sky_radiance[c]));
                ps.flags &= ~P_ALIVE;
            } else {
                float n2[3], o3[3];
                hit_normal(h.axis, ray.d, n2);
                svo_albedo(s, h.c, luts, ps.a);
#pragma unroll
                for (int c = 0; c < 3; c++) o3[c] = xadd(xadd(ray.o[c], xmul(h.t, ray.d[c])), xmul(n2[c], p.offset));
                ps.ndl = sun_cos(n2, p);
                ps.flags |= P_SHADOW;
                if (ps.ndl > 0.0f) set_ray(ns, o3, p.sun_dir);
                if (k + 1 < p.bounces) {
                    float w2[3];
                    const uint32_t r = (uint32_t)i / cs;
                    sample_cosine(n2, roots[r].key, s0 + ((uint32_t)i - r * cs), k + 1, p, w2);
                    set_ray(nb, o3, w2);
                } else {
                    ps.flags &= ~P_ALIVE;
                }
            }
        }
        rb[i] = nb;
        rs[i] = ns;
        st[i] = ps;
    }
}

// Per root: the last pending shadows, the chunk's samples added in order to
// the running sum; on the last chunk out[key] = direct + albedo * sum / spp.
__global__ void __launch_bounds__(256) k_gi_finish(const PathRoot* __restrict__ roots, const uint32_t* __restrict__ n_dev,
                                                   uint32_t cs, GiParams p, const RayHit* __restrict__ hs,
                                                   const PathState* __restrict__ st, const RayHit* __restrict__ root_hits,
                                                   float* __restrict__ acc_buf, bool first, bool last, uint32_t spp,
                                                   float* __restrict__ out)
{
    const uint32_t n = *n_dev;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        float acc[3] = {0.0f, 0.0f, 0.0f};
        if (!first) { acc[0] = acc_buf[3ull * r]; acc[1] = acc_buf[3ull * r + 1]; acc[2] = acc_buf[3ull * r + 2]; }
        for (uint32_t j = 0; j < cs; j++) {
            const uint64_t i = (uint64_t)r * cs + j;
            const PathState& ps = st[i];
            float v[3] = {ps.v[0], ps.v[1], ps.v[2]};
            if (ps.flags & P_SHADOW) {
                float D[3] = {0.0f, 0.0f, 0.0f};
                if (ps.ndl > 0.0f && hs[i].res != 1) sun_term(ps.a, ps.ndl, p, D);
#pragma unroll
                for (int c = 0; c < 3; c++) v[c] = xadd(v[c], xmul(ps.T[c], D[c]));
            }
#pragma unroll
            for (int c = 0; c < 3; c++) acc[c] = xadd(acc[c], v[c]);
        }
        if (!last) {
            acc_buf[3ull * r] = acc[0]; acc_buf[3ull * r + 1] = acc[1]; acc_buf[3ull * r + 2] = acc[2];
            continue;
        }
        const PathRoot& rt = roots[r];
        float L[3] = {0.0f, 0.0f, 0.0f};
        const float ndl = sun_cos(rt.n, p);
        if (ndl > 0.0f && root_hits[r].res != 1) sun_term(rt.a, ndl, p, L);
        const float inv_spp = xdiv(1.0f, (float)(spp ? spp : 1u));
#pragma unroll
        for (int c = 0; c < 3; c++) out[3ull * rt.key + c] = xadd(L[c], xmul(rt.a[c], xmul(acc[c], inv_spp)));
    }
}

// ---------------------------------------------------------------------------
// learned-cache GI
// ---------------------------------------------------------------------------

// The cache stores demodulated radiance: the radiance leaving a bounce hit
// divided by the hit voxel's albedo.  Albedo is per-voxel noise in the
// material grids, so the quotient (direct irradiance / pi plus the mean
// incoming radiance) is far smoother than the radiance itself; queries
// multiply the albedo back in.
struct CacheHit
{
    float p[3];      // hit point (world)
    float n[3];      // face normal
    float w[3];      // direction the bounce ray travelled
    float a[3];      // albedo of the hit voxel
    int32_t c[3];    // grid voxel
};

struct CacheGiConst
{
    float box_min[3];
    float box_inv[3];    // 1 / (box_max - box_min)
    uint32_t n_train, train_spp;
    uint32_t n_train_primary;   // training samples of the pixel-point network per frame
    float primary_weight;
    float primary_variance_scale;
};

enum CacheCounter { CC_ROOTS = 0, CC_QUERIES = 1, CC_TRAIN_ROOTS = 2, CC_QUEUE = 3 };

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

// First-bounce hits of a chunk of samples become cache queries.
__global__ void __launch_bounds__(256) k_gi_query_shade(SvoDev s, const tgx_material* __restrict__ luts, CacheGiConst q,
                                                        const uint32_t* __restrict__ n_dev, uint32_t cs, uint32_t s0,
                                                        uint32_t spp, const Ray* __restrict__ rb,
                                                        const RayHit* __restrict__ hb, int32_t* __restrict__ qidx,
                                                        float* __restrict__ qx, CacheHit* __restrict__ hits,
                                                        uint32_t* __restrict__ counters, uint32_t capacity)
{
    const uint64_t n_paths = (uint64_t)(*n_dev) * cs;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_paths; i += (uint64_t)gridDim.x * blockDim.x) {
        const RayHit h = hb[i];
        const uint32_t r = (uint32_t)i / cs;   // paths in flight < 2^32: 32-bit division
        int32_t* qi = qidx + (uint64_t)r * spp + s0 + ((uint32_t)i - r * cs);
        const bool hit = h.res == 1;
        const uint32_t slot = warp_append(&counters[CC_QUERIES], hit);
        if (!hit) { *qi = -1; continue; }
        if (slot >= capacity) { *qi = -2; continue; }
        *qi = (int32_t)slot;
        const Ray ray = rb[i];
        CacheHit ch;
        hit_normal(h.axis, ray.d, ch.n);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            ch.p[c] = xadd(ray.o[c], xmul(h.t, ray.d[c]));
            ch.w[c] = ray.d[c];
            ch.c[c] = h.c[c];
        }
        svo_albedo(s, h.c, luts, ch.a);
        hits[slot] = ch;
        cache_input(q, ch.p, ch.n, ch.w, qx + 9ull * slot);
    }
}

// Queries of the pixel-point network: each pixel's surface point (root origin
// less the offset), its normal and the camera ray's direction.
__global__ void __launch_bounds__(256) k_gi_primary_queries(const PathRoot* __restrict__ roots,
                                                            const uint32_t* __restrict__ n_dev, GiParams p,
                                                            CacheGiConst q, float cam_x, float cam_y, float cam_z,
                                                            float* __restrict__ qx)
{
    const uint32_t n = *n_dev;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const PathRoot& rt = roots[r];
        const float cam[3] = {cam_x, cam_y, cam_z};
        float x[3], w[3], len2 = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            x[c] = rt.o[c] - rt.n[c] * p.offset;
            w[c] = x[c] - cam[c];
            len2 += w[c] * w[c];
        }
        const float inv = len2 > 0.0f ? rsqrtf(len2) : 0.0f;
#pragma unroll
        for (int c = 0; c < 3; c++) w[c] *= inv;
        cache_input(q, x, rt.n, w, qx + 9ull * r);
    }
}

// The pixel-point network's training batch: n_train_primary random pixels,
// each with its query and this frame's sample mean of incoming light.
__global__ void __launch_bounds__(256) k_gi_primary_batch(GiParams p, CacheGiConst q, const uint32_t* __restrict__ n_dev,
                                                          const float* __restrict__ pqx, const float* __restrict__ pmean,
                                                          float* __restrict__ tx, float* __restrict__ tt)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.n_train_primary) return;
    const uint32_t n = *n_dev;
    uint32_t ctr[4] = {i, 0x7ffffffeu, p.frame, 0x9e1du};
    philox(ctr, (uint32_t)p.seed ^ 0x3C3C3C3Cu, (uint32_t)(p.seed >> 32));
    const uint32_t r = n ? ctr[0] % n : 0u;
#pragma unroll
    for (int k = 0; k < 9; k++) tx[9ull * i + k] = n ? pqx[9ull * r + k] : 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) tt[3ull * i + k] = n ? pmean[3ull * r + k] : 0.0f;
}

// pixel = direct + albedo * mean(sky, or hit albedo * cache prediction)
// With the pixel-point network (prim_rgb), the incoming light is shrunk from
// the sample mean m toward the network's prediction P at the pixel's point:
// e = m + k (P - m).  With one sample k = w; with more, this pass stores the
// pixel's statistics for k_gi_cache_blend: the variance v of its mean and its
// disagreement d2 = |P - m|^2, both as they reach the output (times the
// albedo) and relative to the predicted pixel (|direct + albedo P|^2 + 0.03,
// the relMSE weight).  The sample mean is kept (pmean) as that network's
// training target.
__global__ void __launch_bounds__(256) k_gi_cache_resolve(const PathRoot* __restrict__ roots,
                                                         const uint32_t* __restrict__ n_dev, GiParams p,
                                                         const RayHit* __restrict__ root_hits,
                                                         const int32_t* __restrict__ qidx,
                                                         const float* __restrict__ qrgb,
                                                         const CacheHit* __restrict__ hits,
                                                         const float* __restrict__ prim_rgb, float primary_weight,
                                                         float* __restrict__ pmean, float2* __restrict__ pstat,
                                                         float* __restrict__ out)
{
    const uint32_t n = *n_dev;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const PathRoot& rt = roots[r];
        float acc[3] = {0.0f, 0.0f, 0.0f}, sq[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t k = 0; k < p.spp; k++) {
            const int32_t qv = qidx[(uint64_t)r * p.spp + k];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const float f = qv >= 0 ? xmul(hits[qv].a[i], fmaxf(qrgb[3ull * qv + i], 0.0f))
                                        : (qv == -1 ? p.sky_radiance[i] : 0.0f);
                acc[i] = xadd(acc[i], f);
                sq[i] += f * f;
            }
        }
        float L[3] = {0.0f, 0.0f, 0.0f};
        const float ndl = sun_cos(rt.n, p);
        if (ndl > 0.0f && root_hits[r].res != 1) sun_term(rt.a, ndl, p, L);
        const float inv_spp = xdiv(1.0f, (float)(p.spp ? p.spp : 1u));
        float m[3], pr[3];
#pragma unroll
        for (int i = 0; i < 3; i++) {
            m[i] = xmul(acc[i], inv_spp);
            if (pmean) pmean[3ull * r + i] = m[i];
        }
        if (prim_rgb) {
#pragma unroll
            for (int i = 0; i < 3; i++) pr[i] = fmaxf(prim_rgb[3ull * r + i], 0.0f);
            if (pstat) {   // the blend waits for the neighbourhood's statistics (k_gi_cache_blend)
                const float ns = (float)p.spp;
                float v = 0.0f, d2 = 0.0f, nrm = 0.03f;
#pragma unroll
                for (int i = 0; i < 3; i++) {
                    const float a2 = rt.a[i] * rt.a[i];
                    v += a2 * fmaxf(sq[i] - ns * m[i] * m[i], 0.0f);
                    d2 += a2 * (pr[i] - m[i]) * (pr[i] - m[i]);
                    const float y = L[i] + rt.a[i] * pr[i];
                    nrm += y * y;
                }
                v /= (ns - 1.0f) * ns;
                pstat[rt.key] = make_float2(v / nrm, d2 / nrm);
                continue;
            }
        }
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float e = prim_rgb ? m[i] + primary_weight * (pr[i] - m[i]) : m[i];
            out[3ull * rt.key + i] = xadd(L[i], xmul(rt.a[i], e));
        }
    }
}

// The shrinkage weight.  Over the geometry pixels of the (2R+1)^2 window the
// mean relative variance vn and mean relative disagreement dn give the
// network's local squared error b2 = max(dn - vn, 0); the pixel's variance is
// its own estimate v mixed with vn, vm = a v + (1 - a) vn with
// a = (spp - 1) / (spp - 1/2) (0.67 at 2 spp, 0.8 at 3), so that a pixel whose few
// samples spread far apart leans toward the network.  Then
// k = min(w, s vm / (s vm + b2)), s the variance scale: the k that minimises
// the expected error of m + k (P - m) for noise vm and network error b2.
constexpr int kBlendRadius = 6;   // a 13x13 window

__global__ void __launch_bounds__(256) k_gi_cache_blend(const PathRoot* __restrict__ roots,
                                                       const uint32_t* __restrict__ n_dev, GiParams p,
                                                       const RayHit* __restrict__ root_hits,
                                                       const float* __restrict__ pmean, const float* __restrict__ prim_rgb,
                                                       const float2* __restrict__ pstat, uint32_t width, uint32_t height,
                                                       float primary_weight, float variance_scale,
                                                       float* __restrict__ out)
{
    const uint32_t n = *n_dev;
    const float a = (float)(p.spp - 1) / ((float)p.spp - 0.5f);
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const PathRoot& rt = roots[r];
        const int x = (int)(rt.key % width), y = (int)(rt.key / width);
        const int x0 = max(x - kBlendRadius, 0), x1 = min(x + kBlendRadius, (int)width - 1);
        const int y0 = max(y - kBlendRadius, 0), y1 = min(y + kBlendRadius, (int)height - 1);
        float sv = 0.0f, sd = 0.0f, cnt = 0.0f;
        for (int yy = y0; yy <= y1; yy++) {
            const float2* row = pstat + (size_t)yy * width;
            for (int xx = x0; xx <= x1; xx++) {
                const float2 t = __ldg(row + xx);
                if (t.x == t.x) { sv += t.x; sd += t.y; cnt += 1.0f; }   // NaN: no geometry there
            }
        }
        const float vn = sv / cnt, b2 = fmaxf(sd - sv, 0.0f) / cnt;   // cnt >= 1: the pixel itself
        const float vm = variance_scale * (a * pstat[rt.key].x + (1.0f - a) * vn);
        const float kw = vm > 0.0f ? fminf(primary_weight, vm / (vm + b2)) : 0.0f;
        float L[3] = {0.0f, 0.0f, 0.0f};
        const float ndl = sun_cos(rt.n, p);
        if (ndl > 0.0f && root_hits[r].res != 1) sun_term(rt.a, ndl, p, L);
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const float m = pmean[3ull * r + i], pr = fmaxf(prim_rgb[3ull * r + i], 0.0f);
            out[3ull * rt.key + i] = xadd(L[i], xmul(rt.a[i], m + kw * (pr - m)));
        }
    }
}

// Training roots: n_train bounce hits of this frame, one picked at random
// from each of n_train equal strata of the hit list (so every hit is
// equally likely, and neighbouring roots come from neighbouring pixels and
// trace together).  Root i's sample goes to batch slot key(i), which deals
// the strata round-robin over the `steps` Adam steps: each step sees the
// whole frame.  The target at each is the demodulated radiance (direct /
// albedo + mean incoming) toward where its ray came from, estimated by the
// path passes.
__global__ void __launch_bounds__(256) k_gi_target_roots(GiParams p, CacheGiConst q, uint32_t steps,
                                                        const CacheHit* __restrict__ hits,
                                                        uint32_t* __restrict__ counters, uint32_t capacity,
                                                        PathRoot* __restrict__ roots, float* __restrict__ tx,
                                                        float* __restrict__ tt)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.n_train) return;
    const uint32_t per = steps ? q.n_train / steps : 0u;
    const uint32_t key = i < per * steps ? (i % steps) * per + i / steps : i;
    const uint32_t n_hits = min(counters[CC_QUERIES], capacity);
    if (i == 0) counters[CC_TRAIN_ROOTS] = n_hits ? q.n_train : 0u;
    if (n_hits == 0) {
#pragma unroll
        for (int k = 0; k < 9; k++) tx[9ull * key + k] = 0.0f;
        tt[3ull * key] = tt[3ull * key + 1] = tt[3ull * key + 2] = 0.0f;
        return;
    }
    uint32_t ctr[4] = {i, 0x7fffffffu, p.frame, 0x5eedu};
    philox(ctr, (uint32_t)p.seed ^ 0xA5A5A5A5u, (uint32_t)(p.seed >> 32));
    const uint32_t lo = (uint32_t)((uint64_t)i * n_hits / q.n_train);
    const uint32_t hi = (uint32_t)((uint64_t)(i + 1) * n_hits / q.n_train);
    const uint32_t pick = hi > lo ? lo + ctr[0] % (hi - lo) : min(lo, n_hits - 1u);
    const CacheHit h = hits[pick];
    PathRoot rt;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        rt.o[k] = xadd(h.p[k], xmul(h.n[k], p.offset));
        rt.n[k] = h.n[k];
        rt.a[k] = 1.0f;
    }
    rt.key = key;
    roots[i] = rt;
    cache_input(q, h.p, h.n, h.w, tx + 9ull * key);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

namespace {

struct PathBufs
{
    PathRoot* roots;
    Ray *rb, *rs, *root_rays;
    RayHit *hb, *hs, *root_hits;
    PathState* st;
    float* acc;
    uint64_t max_paths;
};

// carves aligned regions out of one scratch allocation
struct Carver
{
    char* base;
    size_t off = 0;
    template <class T> T* take(uint64_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T* p = base ? (T*)(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
};

void carve_paths(Carver& cv, PathBufs& b, uint64_t max_roots, uint64_t max_paths)
{
    b.roots = cv.take<PathRoot>(max_roots);
    b.root_rays = cv.take<Ray>(max_roots);
    b.root_hits = cv.take<RayHit>(max_roots);
    b.acc = cv.take<float>(max_roots * 3);
    b.rb = cv.take<Ray>(max_paths);
    b.rs = cv.take<Ray>(max_paths);
    b.hb = cv.take<RayHit>(max_paths);
    b.hs = cv.take<RayHit>(max_paths);
    b.st = cv.take<PathState>(max_paths);
    b.max_paths = max_paths;
}

uint32_t chunk_samples(uint32_t spp, uint64_t max_roots)
{
    const uint64_t cap = std::max<uint64_t>(1, kMaxPathsPerChunk / std::max<uint64_t>(max_roots, 1));
    return (uint32_t)std::min<uint64_t>(std::max(spp, 1u), cap);
}

uint32_t trace_grid(tgx_ctx* c)
{
    static int per_sm = 0;
    if (!per_sm) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_queue, 128, 0) != cudaSuccess || per_sm < 1)
            per_sm = 1;
    }
    return (uint32_t)(c->num_sms * per_sm);
}

uint32_t stride_grid(tgx_ctx* c, uint64_t items, uint32_t block)
{
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((items + block - 1) / block, (uint64_t)c->num_sms * 16));
}

// The frame's traversal work counters (DDA steps, rays) sit after the 32
// first words of the frame's counters, which every GI call zeroes.
__host__ __device__ inline unsigned long long* trace_work(uint32_t* counters)
{
    return reinterpret_cast<unsigned long long*>(counters + 32);
}

// queue = &counters[CC_QUEUE] of the frame's counters
tgx_status trace_lists(tgx_ctx* c, const SvoDev& s, const Ray* ra, RayHit* ha, uint32_t mul_a, const Ray* rb,
                       RayHit* hb, uint32_t mul_b, const uint32_t* n_dev, uint32_t max_steps, uint32_t* queue,
                       uint32_t* exhausted)
{
    TGX_CUDA(cudaMemsetAsync(queue, 0, 4, c->stream));
    TGX_LAUNCH(c, TR_GI_TRACE, trace_grid(c), 128, 0, k_trace_queue, s, ra, ha, mul_a, rb, hb, mul_b, n_dev, max_steps,
               c->trace_steps_per_round, queue, exhausted, trace_work(queue - CC_QUEUE));
    return TGX_OK;
}

// spp paths of p.bounces bounces from every root, then out[key] per root.
tgx_status run_paths(tgx_ctx* c, const SvoDev& s, const tgx_material* luts, const GiParams& p, const PathBufs& b,
                     const uint32_t* n_dev, uint32_t max_roots, uint32_t spp, uint32_t* queue, uint32_t* exhausted,
                     float* out)
{
    const uint32_t cs = chunk_samples(spp, max_roots);
    const uint32_t rg = stride_grid(c, max_roots, 256);
    if (spp == 0 || p.bounces == 0) {   // direct term only
        TGX_LAUNCH(c, TR_GI, rg, 256, 0, k_gi_emit, b.roots, n_dev, 0u, 0u, p, b.rb, b.st, b.root_rays);
        TGX_TRY(trace_lists(c, s, nullptr, nullptr, 0u, b.root_rays, b.root_hits, 1u, n_dev, p.max_steps, queue, exhausted));
        TGX_LAUNCH(c, TR_GI, rg, 256, 0, k_gi_finish, b.roots, n_dev, 0u, p, b.hs, b.st, b.root_hits, b.acc, true, true,
                   spp, out);
        return TGX_OK;
    }
    const uint32_t eg = stride_grid(c, (uint64_t)max_roots * cs + max_roots, 256);
    for (uint32_t s0 = 0; s0 < spp; s0 += cs) {
        const uint32_t n = std::min(cs, spp - s0);
        const bool first = s0 == 0, last = s0 + n >= spp;
        TGX_LAUNCH(c, TR_GI, eg, 256, 0, k_gi_emit, b.roots, n_dev, n, s0, p, b.rb, b.st, first ? b.root_rays : nullptr);
        TGX_TRY(trace_lists(c, s, b.rb, b.hb, n, b.root_rays, b.root_hits, first ? 1u : 0u, n_dev, p.max_steps, queue,
                            exhausted));
        for (uint32_t k = 0; k < p.bounces; k++) {
            TGX_LAUNCH(c, TR_GI, eg, 256, 0, k_gi_shade, s, luts, b.roots, n_dev, n, s0, k, p, b.rb, b.hb, b.rs, b.hs,
                       b.st);
            TGX_TRY(trace_lists(c, s, b.rb, b.hb, k + 1 < p.bounces ? n : 0u, b.rs, b.hs, n, n_dev, p.max_steps, queue,
                                exhausted));
        }
        TGX_LAUNCH(c, TR_GI, rg, 256, 0, k_gi_finish, b.roots, n_dev, n, p, b.hs, b.st, b.root_hits, b.acc, first, last,
                   spp, out);
    }
    return TGX_OK;
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
    const uint64_t n_pix = (uint64_t)view->width * view->height;
    const uint64_t max_paths = n_pix * chunk_samples(p.spp, n_pix);
    PathBufs b;
    Carver size{nullptr};
    size.take<uint32_t>(64);
    carve_paths(size, b, n_pix, max_paths);
    TGX_TRY(devbuf_reserve(c->gi_scratch, size.off + 256));
    Carver cv{(char*)c->gi_scratch.ptr};
    uint32_t* counters = cv.take<uint32_t>(64);
    carve_paths(cv, b, n_pix, max_paths);
    TGX_TRY(devbuf_reserve(c->svo_counters, 4 * 4 + 64));
    uint32_t* exhausted = (uint32_t*)c->svo_counters.ptr + 8;
    TGX_CUDA(cudaMemsetAsync(counters, 0, 64 * 4, c->stream));
    const dim3 grid((view->width + 15) / 16, (view->height + 7) / 8);
    TGX_LAUNCH(c, TR_GI, grid, 128, 0, k_gi_roots, sc->d_objects, sc->d_cluster_pointers, sc->d_c2o, sc->d_material,
               sc->d_luts, *view, p, (const unsigned long long*)d_visbuf, d_rgb, b.roots, &counters[CC_ROOTS]);
    return run_paths(c, svo_dev(svo), sc->d_luts, p, b, &counters[CC_ROOTS], (uint32_t)n_pix, p.spp,
                     &counters[CC_QUEUE], exhausted, d_rgb);
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
    if (!(cp->primary_weight >= 0.0f && cp->primary_weight <= 1.0f)) {
        tgx_set_error("tgx_gi_render_cached: primary_weight must be in [0, 1]");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    q.primary_weight = cp->primary_weight;
    if (!(cp->primary_variance_scale >= 0.0f)) {
        tgx_set_error("tgx_gi_render_cached: primary_variance_scale must be >= 0");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    q.primary_variance_scale = cp->primary_variance_scale > 0.0f ? cp->primary_variance_scale : 0.5f;
    q.n_train_primary = cp->n_train_primary;
    const bool primary = q.primary_weight > 0.0f || (q.n_train_primary && cp->train_steps);
    tgx_cache* pnet = nullptr;
    if (primary) TGX_TRY(cache_primary(c, cache, &pnet));
    const bool train = q.n_train && cp->train_steps;
    const uint64_t n_pix = (uint64_t)view->width * view->height;
    const uint64_t capacity = n_pix * p.spp;
    if (capacity > 0x7fffffffull) { tgx_set_error("tgx_gi_render_cached: too many queries"); return TGX_ERR_CAPACITY; }
    const uint32_t cs = chunk_samples(p.spp, n_pix);
    const uint32_t cs_t = train ? chunk_samples(q.train_spp, q.n_train) : 1u;
    const uint64_t max_roots = std::max<uint64_t>(n_pix, q.n_train);
    const uint64_t max_paths = std::max<uint64_t>(n_pix * cs, (uint64_t)q.n_train * cs_t);

    const uint64_t n_prim = primary ? n_pix : 0;
    // the blend needs more than one sample per pixel
    const bool blend = q.primary_weight > 0.0f && p.spp > 1;
    auto layout = [&](Carver& cv, uint32_t*& counters, PathBufs& b, int32_t*& qidx, float*& qx, float*& qrgb,
                      CacheHit*& hits, float*& tx, float*& tt, float*& pqx, float*& pqrgb, float*& pmean,
                      float2*& pstat, float*& ptx, float*& ptt) {
        counters = cv.take<uint32_t>(64);
        carve_paths(cv, b, max_roots, max_paths);
        qidx = cv.take<int32_t>(capacity);
        qx = cv.take<float>(capacity * 9);
        qrgb = cv.take<float>(capacity * 3);
        hits = cv.take<CacheHit>(capacity);
        tx = cv.take<float>((uint64_t)q.n_train * 9);
        tt = cv.take<float>((uint64_t)q.n_train * 3);
        pqx = cv.take<float>(n_prim * 9);
        pqrgb = cv.take<float>(n_prim * 3);
        pmean = cv.take<float>(n_prim * 3);
        pstat = cv.take<float2>(blend ? n_pix : 0);   // per pixel of the view
        ptx = cv.take<float>((uint64_t)(primary ? q.n_train_primary : 0u) * 9);
        ptt = cv.take<float>((uint64_t)(primary ? q.n_train_primary : 0u) * 3);
    };
    uint32_t* counters; PathBufs b; int32_t* qidx; CacheHit* hits;
    float *qx, *qrgb, *tx, *tt, *pqx, *pqrgb, *pmean, *ptx, *ptt;
    float2* pstat;
    Carver size{nullptr};
    layout(size, counters, b, qidx, qx, qrgb, hits, tx, tt, pqx, pqrgb, pmean, pstat, ptx, ptt);
    TGX_TRY(devbuf_reserve(c->gi_scratch, size.off + 256));
    Carver cv{(char*)c->gi_scratch.ptr};
    layout(cv, counters, b, qidx, qx, qrgb, hits, tx, tt, pqx, pqrgb, pmean, pstat, ptx, ptt);
    TGX_TRY(devbuf_reserve(c->svo_counters, 4 * 4 + 64));
    uint32_t* exhausted = (uint32_t*)c->svo_counters.ptr + 8;
    TGX_CUDA(cudaMemsetAsync(counters, 0, 64 * 4, c->stream));
    const SvoDev s = svo_dev(svo);

    // primary hits, then the first bounce of every (pixel, sample) in chunks
    const dim3 grid((view->width + 15) / 16, (view->height + 7) / 8);
    TGX_LAUNCH(c, TR_GI, grid, 128, 0, k_gi_roots, sc->d_objects, sc->d_cluster_pointers, sc->d_c2o, sc->d_material,
               sc->d_luts, *view, p, (const unsigned long long*)d_visbuf, d_rgb, b.roots, &counters[CC_ROOTS]);
    const uint32_t eg = stride_grid(c, n_pix * cs + n_pix, 256);
    for (uint32_t s0 = 0; s0 < p.spp; s0 += cs) {
        const uint32_t n = std::min(cs, p.spp - s0);
        const bool first = s0 == 0;
        TGX_LAUNCH(c, TR_GI, eg, 256, 0, k_gi_emit, b.roots, &counters[CC_ROOTS], n, s0, p, b.rb, (PathState*)nullptr,
                   first ? b.root_rays : nullptr);
        TGX_TRY(trace_lists(c, s, b.rb, b.hb, n, b.root_rays, b.root_hits, first ? 1u : 0u, &counters[CC_ROOTS],
                            p.max_steps, &counters[CC_QUEUE], exhausted));
        TGX_LAUNCH(c, TR_GI, eg, 256, 0, k_gi_query_shade, s, sc->d_luts, q, &counters[CC_ROOTS], n, s0, p.spp, b.rb,
                   b.hb, qidx, qx, hits, counters, (uint32_t)capacity);
    }
    // inference over all potential queries: slots past the hit count are never read
    TGX_TRY(cache_infer_counted(c, cache, &counters[CC_QUERIES], (uint32_t)capacity, qx, qrgb));
    if (primary) {
        TGX_LAUNCH(c, TR_GI, stride_grid(c, n_pix, 256), 256, 0, k_gi_primary_queries, b.roots, &counters[CC_ROOTS], p,
                   q, view->camera[0], view->camera[1], view->camera[2], pqx);
        if (q.primary_weight > 0.0f)
            TGX_TRY(cache_infer_counted(c, pnet, &counters[CC_ROOTS], (uint32_t)n_pix, pqx, pqrgb));
    }
    // pixels without geometry keep NaN statistics (all bytes 0xff)
    if (blend) TGX_CUDA(cudaMemsetAsync(pstat, 0xff, n_pix * sizeof(float2), c->stream));
    TGX_LAUNCH(c, TR_GI, stride_grid(c, n_pix, 256), 256, 0, k_gi_cache_resolve, b.roots, &counters[CC_ROOTS], p,
               b.root_hits, qidx, qrgb, hits, q.primary_weight > 0.0f ? pqrgb : nullptr, q.primary_weight,
               primary ? pmean : nullptr, blend ? pstat : nullptr, d_rgb);
    if (blend)
        TGX_LAUNCH(c, TR_GI, stride_grid(c, n_pix, 256), 256, 0, k_gi_cache_blend, b.roots, &counters[CC_ROOTS], p,
                   b.root_hits, pmean, pqrgb, pstat, view->width, view->height, q.primary_weight,
                   q.primary_variance_scale, d_rgb);
    const bool train_primary = primary && q.n_train_primary && cp->train_steps;
    if (train_primary)
        TGX_LAUNCH(c, TR_GI, (q.n_train_primary + 255) / 256, 256, 0, k_gi_primary_batch, p, q, &counters[CC_ROOTS], pqx,
                   pmean, ptx, ptt);
    if (train) {
        TGX_LAUNCH(c, TR_GI, (q.n_train + 255) / 256, 256, 0, k_gi_target_roots, p, q, cp->train_steps, hits,
                   counters, (uint32_t)capacity, b.roots, tx, tt);
        GiParams pp = p;
        pp.bounces = p.bounces - 1;
        pp.frame = p.frame | 0x800000u;   // decorrelated from the pixel streams
        TGX_TRY(run_paths(c, s, sc->d_luts, pp, b, &counters[CC_TRAIN_ROOTS], q.n_train, q.train_spp,
                          &counters[CC_QUEUE], exhausted, tt));
    }
    // the two networks' Adam steps, side by side in shared launches
    const uint32_t per = train ? q.n_train / cp->train_steps : 0u;
    const uint32_t pper = train_primary ? q.n_train_primary / cp->train_steps : 0u;
    for (uint32_t k = 0; k < cp->train_steps && (per || pper); k++) {
        tgx_cache* nets[2];
        uint32_t ns[2];
        const float *xs[2], *ts[2];
        uint32_t m = 0;
        if (per) { nets[m] = cache; ns[m] = per; xs[m] = tx + 9ull * per * k; ts[m] = tt + 3ull * per * k; m++; }
        if (pper) { nets[m] = pnet; ns[m] = pper; xs[m] = ptx + 9ull * pper * k; ts[m] = ptt + 3ull * pper * k; m++; }
        TGX_TRY(cache_train_pair(c, nets, ns, xs, ts, m, cp->lr));
    }
    return TGX_OK;
}

extern "C" tgx_status tgx_gi_get_work(tgx_ctx* c, tgx_gi_work* out)
{
    if (!c || !out) return TGX_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    if (!c->gi_scratch.ptr) return TGX_OK;
    unsigned long long h[2];
    TGX_CUDA(cudaMemcpyAsync(h, trace_work((uint32_t*)c->gi_scratch.ptr), sizeof(h), cudaMemcpyDeviceToHost,
                             c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    out->dda_steps = h[0];
    out->rays = h[1];
    return TGX_OK;
}
