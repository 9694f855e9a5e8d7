// vis.cu -- visibility-buffer pass.
//
// Replaces tg's instanced cluster-box raster (visibility.vert:19-26 with
// cluster_functions.inc:1-38), its fragment-shader DDA (visibility.frag:22-207)
// and the clear pass (clear.comp:15-21) with a binned compute pass:
//
//   1. k_vis_cluster_setup  one thread per (view, cluster pointer): drops
//      clusters outside the frustum or beyond the far plane (bounding
//      sphere, then box corners) and empty clusters, computes a conservative
//      screen-tile rectangle and a lower bound of the packed depth, and
//      appends a 32-byte record.
//   2. k_vis_count          per record: the ws2ms matrix and the camera
//      position in cluster space exactly as the shader does (one thread per
//      record), and its counts per (tile, depth bucket) (a half-warp per record).
//   3. k_vis_prefix         per tile: offsets of its 16 depth buckets; per
//                           256 tiles: their sum and class histogram.
//   4. k_vis_scan           one CTA: bases of the 256-tile groups and the
//      k_vis_finalize       cursors of the launch order (heaviest class
//                           first); then per group: tile offsets and order.
//                           Up to 512 groups, k_vis_finalize_direct does both:
//                           each CTA reads all groups' sums and histograms.
//   5. k_vis_bin_fill       a half-warp per record: writes it, with its cluster's
//                           64-byte bitmask, as a 96-byte entry into each of its
//                           (tile, bucket) bins, so every tile's entries are
//                           contiguous and run near to far.
//   6. k_vis_tiles          one CTA per tile (heaviest first), one thread per
//      pixel: batches of the tile's entries arrive by one cp.async.bulk each
//      on an mbarrier; every pixel skips entries whose depth bound cannot beat
//      its word and rejects clear misses with a conservative reciprocal slab
//      test; the surviving (pixel, cluster) pairs are compacted by warp ballot
//      and run the shader's exact ray/box test and DDA on full warps, keeping
//      each pixel's minimum packed depth|pointer|voxel word (shared
//      atomicMin); every pixel is written once (fused clear).
//      k_vis_tiles_queue is the persistent form over many jobs' tiles.
//
// Every pair evaluates the same binary32 operations in the same order as the
// CPU oracle's transcription of visibility.frag, so the buffer is bit-exact.

#include "tgx_internal.cuh"

#include <climits>
#include <cmath>
#include <mutex>
#include <vector>

namespace {

constexpr uint32_t kCluster = 8;
constexpr uint32_t kMaxDdaSteps = 64;      // the 8^3 DDA needs at most 22
constexpr uint32_t kMaxBuckets = 32;       // depth buckets per tile at the finest setting (half an octave each)

struct alignas(16) VisRecord
{
    float    ox, oy, oz;        // camera position in cluster space (visibility.frag:66)
    uint32_t cluster_idx;
    uint32_t cluster_pointer;
    uint32_t object_idx;
    uint32_t d24_lb;            // lower bound of the 24-bit depth field any pixel can get from it
    uint32_t view;
};
static_assert(sizeof(VisRecord) == 32, "record layout");

enum Counter { C_RECORDS = 0, C_ENTRIES = 1, C_DDA_OVERRUN = 2, C_OVERFLOW = 3, C_TILE_QUEUE = 4, C_NONEMPTY = 5,
               C_COUNT = 8 };

// One binned (tile, cluster) entry as the tile kernel stages it: the record's
// fields the DDA needs and the cluster's 64-byte bitmask, so a batch of a
// tile's entries is one contiguous bulk copy.
struct alignas(16) TileEntry
{
    float    ox, oy, oz;        // camera position in cluster space
    uint32_t cluster_pointer;
    uint32_t object_idx;
    uint32_t d24_lb;
    uint32_t pad[2];
    uint32_t bits[16];
};
static_assert(sizeof(TileEntry) == 96, "entry layout");
constexpr uint32_t kEntryWords = sizeof(TileEntry) / 4;
// work counters of the tile kernel's counting variant (tgx_vis_work, same order)
enum Work { W_PAIRS = 0, W_DEPTH_SKIPS, W_DIR_SETUPS, W_SLAB_MISSES, W_SURE_HITS, W_EXACT_TESTS, W_DDAS, W_DDA_STEPS,
            W_HITS, W_BATCHES, W_COUNT };
constexpr uint32_t kOrderClasses = 32;     // tiles are launched heaviest class (log2 of bin count) first

// bucket of a depth key: one per power of two of the 24-bit depth, keys < 512 share bucket 0
// Depth buckets of a tile's entries: key = the 24-bit depth field's lower
// bound.  Keys below 512 share the first bucket; above, every half octave of
// the key is a fine bucket (0..31), and a frame uses 32 >> bshift buckets
// (bshift 0, 1 or 2: 32, 16 or 8 buckets, i.e. half, one or two octaves each).
__device__ __forceinline__ uint32_t depth_bucket(uint32_t key, uint32_t bshift)
{
    if (key < 512u) return 0u;
    const uint32_t l = 31u - (uint32_t)__clz(key);   // 9..23
    const uint32_t fine = 2u * (l - 8u) + ((key >> (l - 1u)) & 1u);
    return fine >> bshift;
}
// the smallest key of bucket b
__device__ __forceinline__ uint32_t bucket_lo(uint32_t b, uint32_t bshift)
{
    const uint32_t f = b << bshift;
    return f == 0u ? 0u : (f & 1u) ? (3u << ((f >> 1) + 7u)) : (1u << ((f >> 1) + 8u));
}

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred)
{
    const uint32_t mask = __ballot_sync(0xffffffffu, pred);
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if (mask) {
        const int leader = __ffs(mask) - 1;
        if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------------------
// 1. per-cluster setup
// ---------------------------------------------------------------------------

// kPacked: the scene's per-pointer table gives each pointer's object and
// whether its cluster is empty (one load beside the pointer's own, instead of
// the chain pointer -> owner -> bitmask); without it (the entry point that
// allocates nothing) the owner and the bitmask are read.
template <bool kPacked>
__global__ void __launch_bounds__(256, 4) k_vis_cluster_setup(
    const tgx_object* __restrict__ objects, const uint32_t* __restrict__ cluster_pointers,
    const uint32_t* __restrict__ c2o, const uint32_t* __restrict__ bits, const uint32_t* __restrict__ cp_obj,
    uint32_t n_cp, const ViewConst* __restrict__ views, uint32_t n_views, VisRecord* __restrict__ records,
    uint2* __restrict__ rects, uint32_t record_capacity, uint32_t* __restrict__ counters,
    uint32_t* __restrict__ zero, uint32_t n_zero, tgx_dev_status* __restrict__ status)
{
    pdl_wait();
    pdl_trigger();
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // the (tile, bucket) counts start at zero; k_vis_count runs after this kernel
    for (uint64_t i = gid; i < n_zero; i += (uint64_t)gridDim.x * blockDim.x) zero[i] = 0u;
    const uint32_t v = (uint32_t)(gid / n_cp);
    const uint32_t cp = (uint32_t)(gid % n_cp);
    bool keep = false;
    VisRecord rec = {};
    uint32_t tx0 = 0, ty0 = 0, tx1 = 0, ty1 = 0;
    if (v < n_views) {
        const ViewConst& vc = views[v];
        const uint32_t ci = cluster_pointers[cp];
        const uint32_t po = kPacked ? cp_obj[cp] : 0u;
        if (!kPacked || !(po >> 31)) {   // bit 31: the cluster has no set voxel
            bool oi_cull = false;
            const uint32_t oi = kPacked ? po : c2o[ci];
            const tgx_object& od = objects[oi];
            const uint32_t nx = od.n_cluster_pointers_per_dim[0], ny = od.n_cluster_pointers_per_dim[1];
            const uint32_t rel = cp - od.first_cluster_pointer;
            const uint32_t rx = rel % nx, ry = (rel / nx) % ny, rz = rel / (nx * ny);
            const float offx = (float)(rx * kCluster), offy = (float)(ry * kCluster), offz = (float)(rz * kCluster);
            const float half = xmul((float)kCluster, 0.5f);
            const float ohx = xmul(half, (float)od.n_cluster_pointers_per_dim[0]);
            const float ohy = xmul(half, (float)od.n_cluster_pointers_per_dim[1]);
            const float ohz = xmul(half, (float)od.n_cluster_pointers_per_dim[2]);
            // the box's corner 0 relative to the camera and its three edges (8 voxels
            // along each rotated axis); corner k = base + (k&1) ex + (k&2) ey + (k&4) ez.
            // Rounding differs from a per-corner transform by ulps, far inside the
            // cull's slack (0.05 + 1e-5 |p|) and the rectangle's 2-pixel margin.
            float base[3], ex[3], ey[3], ez[3];
            {
                const float lx = offx - ohx, ly = offy - ohy, lz = offz - ohz;
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    const float r0 = od.rotation[r], r1 = od.rotation[4 + r], r2 = od.rotation[8 + r];
                    base[r] = r0 * lx + r1 * ly + r2 * lz + od.translation[r] - vc.cam[r];
                    ex[r] = 8.0f * r0; ey[r] = 8.0f * r1; ez[r] = 8.0f * r2;
                }
            }

            // ---- bounding-sphere cull against the side planes and the far plane ----
            {
                float q[3];
#pragma unroll
                for (int r = 0; r < 3; r++) q[r] = base[r] + 0.5f * (ex[r] + ey[r] + ez[r]);
                const float rad = 6.9283f + 0.05f + 1e-5f * (fabsf(q[0]) + fabsf(q[1]) + fabsf(q[2]));
                const float dist = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                bool out = dist - rad > vc.far_plane * 1.0001f;
#pragma unroll
                for (int k = 0; k < 4; k++)
                    out |= vc.planes[3 * k] * q[0] + vc.planes[3 * k + 1] * q[1] + vc.planes[3 * k + 2] * q[2] < -rad;
                if (out) oi_cull = true;
            }

            if (!kPacked && !oi_cull) {
                // a cluster without set bits never writes (its DDA finds nothing)
                const uint4* w = reinterpret_cast<const uint4*>(bits + (uint64_t)ci * 16u);
                const uint4 a = w[0], b = w[1], c = w[2], d = w[3];
                oi_cull = !(a.x | a.y | a.z | a.w | b.x | b.y | b.z | b.w | c.x | c.y | c.z | c.w | d.x | d.y | d.z | d.w);
            }
            if (!oi_cull) {
            // ---- culling and conservative screen rectangle (never exact-critical: widened) ----
            float fxmin = 1e30f, fxmax = -1e30f, fymin = 1e30f, fymax = -1e30f;
            bool full = false, any_front = false;
            bool inside0 = false, inside1 = false, inside2 = false, inside3 = false;
            float cxw = 0.0f, cyw = 0.0f, czw = 0.0f;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float p[3];
#pragma unroll
                for (int r = 0; r < 3; r++)
                    p[r] = base[r] + ((k & 1) ? ex[r] : 0.0f) + ((k & 2) ? ey[r] : 0.0f) + ((k & 4) ? ez[r] : 0.0f);
                cxw += p[0]; cyw += p[1]; czw += p[2];
                const float depth = p[0] * vc.fwd[0] + p[1] * vc.fwd[1] + p[2] * vc.fwd[2];
                if (depth > -0.5f) any_front = true;
                const float slack = -(0.05f + 1e-5f * (fabsf(p[0]) + fabsf(p[1]) + fabsf(p[2])));
                inside0 |= vc.planes[0] * p[0] + vc.planes[1] * p[1] + vc.planes[2] * p[2] > slack;
                inside1 |= vc.planes[3] * p[0] + vc.planes[4] * p[1] + vc.planes[5] * p[2] > slack;
                inside2 |= vc.planes[6] * p[0] + vc.planes[7] * p[1] + vc.planes[8] * p[2] > slack;
                inside3 |= vc.planes[9] * p[0] + vc.planes[10] * p[1] + vc.planes[11] * p[2] > slack;
                const float s = vc.inv_basis[0] * p[0] + vc.inv_basis[1] * p[1] + vc.inv_basis[2] * p[2];
                if (depth < 0.5f || s <= 0.0f) { full = true; continue; }
                const float fa = (vc.inv_basis[3] * p[0] + vc.inv_basis[4] * p[1] + vc.inv_basis[5] * p[2]) / s;
                const float fb = (vc.inv_basis[6] * p[0] + vc.inv_basis[7] * p[1] + vc.inv_basis[8] * p[2]) / s;
                fxmin = fminf(fxmin, fa); fxmax = fmaxf(fxmax, fa);
                fymin = fminf(fymin, fb); fymax = fmaxf(fymax, fb);
            }
            // lower bound of the distance from the camera to any point of the box
            const float cdist = sqrtf(cxw * cxw + cyw * cyw + czw * czw) * 0.125f;
            const float lb = fmaxf(0.0f, cdist * (1.0f - 1e-5f) - 6.9283f - 0.01f);
            const float lbq = lb / vc.far_plane;
            if (any_front && inside0 && inside1 && inside2 && inside3 && lbq <= 1.0001f) {
                const float W = (float)vc.width, H = (float)vc.height;
                float x0, x1, y0, y1;
                if (full) {
                    x0 = 0.0f; y0 = 0.0f; x1 = W - 1.0f; y1 = H - 1.0f;
                } else {
                    const float m = 2.0f;   // pixels of slack for the float projection
                    x0 = fxmin * W - 0.5f - m; x1 = fxmax * W - 0.5f + m;
                    y0 = (1.0f - fymax) * H - 0.5f - m; y1 = (1.0f - fymin) * H - 0.5f + m;
                }
                if (!(x1 < 0.0f || y1 < 0.0f || x0 > W - 1.0f || y0 > H - 1.0f)) {
                    const int ix0 = max(0, (int)floorf(x0)), iy0 = max(0, (int)floorf(y0));
                    const int ix1 = min((int)vc.width - 1, (int)ceilf(x1));
                    const int iy1 = min((int)vc.height - 1, (int)ceilf(y1));
                    if (ix0 <= ix1 && iy0 <= iy1) {
                        keep = true;
                        tx0 = (uint32_t)ix0 / vc.tile_w; ty0 = (uint32_t)iy0 / vc.tile_h;
                        tx1 = (uint32_t)ix1 / vc.tile_w; ty1 = (uint32_t)iy1 / vc.tile_h;
                    }
                }
            }
            if (keep) {
                // the exact cluster-space origin is computed by k_vis_count
                rec.cluster_idx = ci;
                rec.cluster_pointer = cp;
                rec.object_idx = oi;
                const float k24 = fminf(lbq, 1.0f) * 16777215.0f;
                rec.d24_lb = k24 >= 2.0f ? (uint32_t)k24 - 1u : 0u;
                rec.view = v;
            }
            }
        }
    }
    const uint32_t slot = warp_append(&counters[C_RECORDS], keep);
    if (!keep) return;
    if (slot >= record_capacity) {
        dev_error(status, TGX_ERR_CAPACITY, 1, slot);
        return;
    }
    records[slot] = rec;
    rects[slot] = make_uint2(tx0 | (ty0 << 16), tx1 | (ty1 << 16));
}

// ---------------------------------------------------------------------------
// 2. per record: the exact ws2ms and ray origin (visibility.frag:57-66), one
//    thread per record; then its per-(tile, bucket) counts, a half-warp per
//    record with the lanes over its tiles.  The two loops write different
//    fields and buffers; the cull kept apart runs at high occupancy.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_vis_count(VisRecord* __restrict__ records, const uint2* __restrict__ rects,
                                                  const uint32_t* __restrict__ counters, uint32_t record_capacity,
                                                  const tgx_object* __restrict__ objects,
                                                  const ViewConst* __restrict__ views,
                                                  uint32_t* __restrict__ bucket_cnt, uint32_t n_tiles,
                                                  uint32_t bshift)
{
    pdl_wait();
    pdl_trigger();
    const uint32_t n = min(counters[C_RECORDS], record_capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        VisRecord& rec = records[i];
        const tgx_object& od = objects[rec.object_idx];
        const ViewConst& vc = views[rec.view];
        const uint32_t nx = od.n_cluster_pointers_per_dim[0], ny = od.n_cluster_pointers_per_dim[1];
        const uint32_t rel = rec.cluster_pointer - od.first_cluster_pointer;
        const float offx = (float)((rel % nx) * kCluster), offy = (float)(((rel / nx) % ny) * kCluster);
        const float offz = (float)((rel / (nx * ny)) * kCluster);
        const float half = xmul((float)kCluster, 0.5f);
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
        float o[3];
        dm4_mulv4(ws2ms, vc.cam[0], vc.cam[1], vc.cam[2], 1.0f, o);
        rec.ox = o[0]; rec.oy = o[1]; rec.oz = o[2];
    }
    const uint32_t lane = threadIdx.x & 15u;   // a half-warp per record: records span ~17 tiles on average
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 4; i < n; i += (gridDim.x * blockDim.x) >> 4) {
        const uint2 r = rects[i];
        const uint32_t view = records[i].view;
        const ViewConst& vc = views[view];
        const uint32_t b = depth_bucket(records[i].d24_lb, bshift);
        const uint32_t tx0 = r.x & 0xffffu, ty0 = r.x >> 16, tx1 = r.y & 0xffffu, ty1 = r.y >> 16;
        const uint32_t w = tx1 - tx0 + 1, cnt = w * (ty1 - ty0 + 1);
        for (uint32_t k = lane; k < cnt; k += 16) {
            const uint32_t t = vc.tile_base + (ty0 + k / w) * vc.tiles_x + tx0 + k % w;
            atomicAdd(&bucket_cnt[b * n_tiles + t], 1u);
        }
    }
}

// ---------------------------------------------------------------------------
// 3. per-tile bucket offsets (one thread per tile, bucket-major = coalesced),
//    and per CTA of 256 tiles: the sum of the tile totals and the histogram
//    of tile classes (cta_aux = [n_ctas sums][n_ctas x kOrderClasses])
// ---------------------------------------------------------------------------

constexpr uint32_t kScanTiles = 256;   // tiles per CTA of the prefix and finalize kernels

__device__ __forceinline__ uint32_t tile_class(uint32_t total) { return total ? 32u - __clz(total) : 0u; }

template <uint32_t kBuckets>
__global__ void __launch_bounds__(kScanTiles) k_vis_prefix(uint32_t* __restrict__ bucket_cnt,
                                                          uint32_t* __restrict__ bucket_off,
                                                          uint32_t* __restrict__ tile_total, uint32_t n_tiles,
                                                          uint32_t* __restrict__ cta_aux)
{
    __shared__ uint32_t cls[kOrderClasses];
    __shared__ uint32_t wsum[kScanTiles / 32];
    if (threadIdx.x < kOrderClasses) cls[threadIdx.x] = 0;
    pdl_wait();
    pdl_trigger();
    __syncthreads();
    const uint32_t t = blockIdx.x * kScanTiles + threadIdx.x;
    uint32_t run = 0;
    if (t < n_tiles) {
        uint32_t c[kBuckets];   // all loads first: the cursor reset below must not wait on them one by one
#pragma unroll
        for (uint32_t b = 0; b < kBuckets; b++) c[b] = bucket_cnt[b * n_tiles + t];
#pragma unroll
        for (uint32_t b = 0; b < kBuckets; b++) {
            bucket_off[b * n_tiles + t] = run;
            bucket_cnt[b * n_tiles + t] = 0;   // becomes the fill cursor
            run += c[b];
        }
        tile_total[t] = run;
        atomicAdd(&cls[tile_class(run)], 1u);
    }
    uint32_t sum = run;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31u) == 0) wsum[threadIdx.x >> 5] = sum;
    __syncthreads();
    const uint32_t n_ctas = (n_tiles + kScanTiles - 1) / kScanTiles;
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
#pragma unroll
        for (uint32_t w = 0; w < kScanTiles / 32; w++) tot += wsum[w];
        cta_aux[blockIdx.x] = tot;
    }
    if (threadIdx.x < kOrderClasses) cta_aux[n_ctas + blockIdx.x * kOrderClasses + threadIdx.x] = cls[threadIdx.x];
}

// ---------------------------------------------------------------------------
// 4. one CTA: exclusive scan of the per-CTA sums (-> CTA bases) and, per
//    tile class (heaviest first), the exclusive scan over CTAs of the class
//    counts (-> per-(CTA, class) cursors of the launch order)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(1024) k_vis_scan(uint32_t* __restrict__ cta_aux, uint32_t n_tiles,
                                                   uint32_t* __restrict__ tile_off, uint32_t bin_capacity,
                                                   uint32_t* __restrict__ counters)
{
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t cls_tot[kOrderClasses];
    __shared__ uint32_t cls_base[kOrderClasses];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t n_ctas = (n_tiles + kScanTiles - 1) / kScanTiles;
    uint32_t* cls_cnt = cta_aux + n_ctas;
    pdl_wait();
    pdl_trigger();
    // CTA bases
    uint32_t carry = 0;
    for (uint32_t base = 0; base < n_ctas; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t x = i < n_ctas ? cta_aux[i] : 0u;
        uint32_t incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t w = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if ((int)lane >= o) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        if (i < n_ctas) cta_aux[i] = carry + (wid ? warp_sums[wid - 1] : 0u) + incl - x;
        carry += warp_sums[31];
        __syncthreads();
    }
    // class totals (warp c sums class c over the CTAs)
    uint32_t tot = 0;
#pragma unroll 4
    for (uint32_t b = lane; b < n_ctas; b += 32) tot += cls_cnt[b * kOrderClasses + wid];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
    if (lane == 0) cls_tot[wid] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
        tile_off[n_tiles] = carry;
        counters[C_ENTRIES] = carry;
        counters[C_OVERFLOW] = carry > bin_capacity ? 1u : 0u;
        counters[C_NONEMPTY] = n_tiles - cls_tot[0];   // class 0: the tiles without entries
        uint32_t run = 0;   // heaviest class first
        for (int c = (int)kOrderClasses - 1; c >= 0; c--) {
            cls_base[c] = run;
            run += cls_tot[c];
        }
    }
    __syncthreads();
    // per-(CTA, class) cursors: warp c scans class c over the CTAs
    uint32_t run = cls_base[wid];
    for (uint32_t b0 = 0; b0 < n_ctas; b0 += 128) {   // four chunks of 32 CTAs: loads first
        uint32_t x[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t b = b0 + 32u * j + lane;
            x[j] = b < n_ctas ? cls_cnt[b * kOrderClasses + wid] : 0u;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t b = b0 + 32u * j + lane;
            uint32_t incl = x[j];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl += y;
            }
            if (b < n_ctas) cls_cnt[b * kOrderClasses + wid] = run + incl - x[j];
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

// ---------------------------------------------------------------------------
// 4b. per CTA of 256 tiles: tile offsets (CTA base + scan of the totals) and
//     each tile's place in the launch order
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kScanTiles) k_vis_finalize(const uint32_t* __restrict__ tile_total, uint32_t n_tiles,
                                                            const uint32_t* __restrict__ cta_aux,
                                                            uint32_t* __restrict__ tile_off,
                                                            uint4* __restrict__ slot_info)
{
    __shared__ uint32_t cur[kOrderClasses];
    __shared__ uint32_t wsum[kScanTiles / 32];
    const uint32_t n_ctas = (n_tiles + kScanTiles - 1) / kScanTiles;
    pdl_wait();
    pdl_trigger();
    if (threadIdx.x < kOrderClasses) cur[threadIdx.x] = cta_aux[n_ctas + blockIdx.x * kOrderClasses + threadIdx.x];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t t = blockIdx.x * kScanTiles + threadIdx.x;
    const bool valid = t < n_tiles;
    const uint32_t x = valid ? tile_total[t] : 0u;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += y;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    uint32_t before = cta_aux[blockIdx.x];
    for (uint32_t w = 0; w < wid; w++) before += wsum[w];
    if (valid) {
        const uint32_t off = before + incl - x;
        tile_off[t] = off;
        slot_info[atomicAdd(&cur[tile_class(x)], 1u)] = make_uint4(t, off, x, 0u);
    }
}

// ---------------------------------------------------------------------------
// 4'. frames of at most kDirectGroups groups skip the one-CTA scan: every
//     CTA of the finalize derives its own group base and class cursors from
//     all groups' sums and class histograms (read from L2; 127 x 33 words at
//     1080p), then places its tiles as k_vis_finalize does.  Same offsets,
//     order and counters as k_vis_scan + k_vis_finalize.
// ---------------------------------------------------------------------------

constexpr uint32_t kDirectGroups = 512;

__global__ void __launch_bounds__(kScanTiles) k_vis_finalize_direct(const uint32_t* __restrict__ tile_total,
                                                                   uint32_t n_tiles,
                                                                   const uint32_t* __restrict__ cta_aux,
                                                                   uint32_t* __restrict__ tile_off,
                                                                   uint4* __restrict__ slot_info,
                                                                   uint32_t bin_capacity,
                                                                   uint32_t* __restrict__ counters)
{
    constexpr uint32_t kWarps = kScanTiles / 32;
    __shared__ uint32_t cur[kOrderClasses];
    __shared__ uint32_t part_tot[kWarps][kOrderClasses], part_pre[kWarps][kOrderClasses];
    __shared__ uint32_t red_pre[kWarps], red_all[kWarps], wsum[kWarps];
    const uint32_t n_ctas = (n_tiles + kScanTiles - 1) / kScanTiles;
    const uint32_t g = blockIdx.x, lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    pdl_wait();
    pdl_trigger();
    // this group's base (the sums of the groups before it) and the frame's total
    uint32_t pre = 0, all = 0;
    for (uint32_t i = threadIdx.x; i < n_ctas; i += kScanTiles) {
        const uint32_t v = cta_aux[i];
        all += v;
        pre += i < g ? v : 0u;
    }
    // per class (lane): its count over all groups and over the groups before this one
    const uint32_t* cls_cnt = cta_aux + n_ctas;
    uint32_t ct = 0, cp = 0;
    for (uint32_t b = wid; b < n_ctas; b += kWarps) {
        const uint32_t v = cls_cnt[b * kOrderClasses + lane];
        ct += v;
        cp += b < g ? v : 0u;
    }
    part_tot[wid][lane] = ct;
    part_pre[wid][lane] = cp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pre += __shfl_xor_sync(0xffffffffu, pre, o);
        all += __shfl_xor_sync(0xffffffffu, all, o);
    }
    if (lane == 0) { red_pre[wid] = pre; red_all[wid] = all; }
    // the tiles' totals, scanned within each warp
    const uint32_t t = g * kScanTiles + threadIdx.x;
    const bool valid = t < n_tiles;
    const uint32_t x = valid ? tile_total[t] : 0u;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += y;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {   // class bases, heaviest class first, plus this group's share before it
        uint32_t tot = 0, before = 0;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; w++) { tot += part_tot[w][lane]; before += part_pre[w][lane]; }
        uint32_t suffix = tot;   // classes lane .. 31
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_down_sync(0xffffffffu, suffix, o);
            if (lane + o < 32) suffix += y;
        }
        cur[lane] = suffix - tot + before;
        if (g == 0 && lane == 0) counters[C_NONEMPTY] = n_tiles - tot;   // class 0: the tiles without entries
    }
    __syncthreads();
    uint32_t base = 0, total = 0;
#pragma unroll
    for (uint32_t w = 0; w < kWarps; w++) { base += red_pre[w]; total += red_all[w]; }
    if (g == 0 && threadIdx.x == 0) {
        tile_off[n_tiles] = total;
        counters[C_ENTRIES] = total;
        counters[C_OVERFLOW] = total > bin_capacity ? 1u : 0u;
    }
    for (uint32_t w = 0; w < wid; w++) base += wsum[w];
    if (valid) {
        const uint32_t off = base + incl - x;
        tile_off[t] = off;
        slot_info[atomicAdd(&cur[tile_class(x)], 1u)] = make_uint4(t, off, x, 0u);
    }
}

// ---------------------------------------------------------------------------
// 5. bin fill: a half-warp per record; its lanes take the record's tiles'
//    slots (16 at a time), then 12 lanes write the 96-byte entry into each
//    slot with 8-byte stores
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_vis_bin_fill(const VisRecord* __restrict__ records,
                                                     const uint2* __restrict__ rects,
                                                     const uint32_t* __restrict__ counters,
                                                     const ViewConst* __restrict__ views,
                                                     const uint32_t* __restrict__ tile_off,
                                                     const uint32_t* __restrict__ bucket_off,
                                                     uint32_t* __restrict__ cursor, TileEntry* __restrict__ entries,
                                                     const uint32_t* __restrict__ bits,
                                                     uint32_t n_tiles, uint32_t bin_capacity, uint32_t bshift,
                                                     tgx_dev_status* __restrict__ status)
{
    pdl_wait();
    pdl_trigger();
    if (counters[C_OVERFLOW]) return;   // the tile kernel scans all records instead
    const uint32_t lane = threadIdx.x & 15u;
    const uint32_t src0 = threadIdx.x & 16u;   // this half-warp's first lane in the warp
    const uint32_t n = counters[C_RECORDS];
    uint2* const ew = reinterpret_cast<uint2*>(entries);
    const uint32_t stride = (gridDim.x * blockDim.x) >> 4;
    // every half-warp runs the same number of iterations, so the shuffles see full warps
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t it = 0; it < rounds; it++) {
        const uint32_t i = ((blockIdx.x * blockDim.x + threadIdx.x) >> 4) + it * stride;
        const bool have = i < n;
        // entry words 2 lane, 2 lane + 1: ox oy | oz pointer | object lb | 0 0 | bitmask (16 words)
        uint2 word = make_uint2(0u, 0u);
        uint32_t cnt = 0, w = 1, tx0 = 0, ty0 = 0, b = 0, tile_base = 0, tiles_x = 0;
        if (have) {
            const uint32_t* rw = reinterpret_cast<const uint32_t*>(records + i);
            if (lane == 0) word = make_uint2(rw[0], rw[1]);
            else if (lane == 1) word = make_uint2(rw[2], rw[4]);
            else if (lane == 2) word = make_uint2(rw[5], rw[6]);
            else if (lane >= 4 && lane < 12) {
                const uint2* bw = reinterpret_cast<const uint2*>(bits + (uint64_t)rw[3] * 16u);
                word = bw[lane - 4];
            }
            const uint2 r = rects[i];
            const VisRecord& rec = records[i];
            const ViewConst& vc = views[rec.view];
            b = depth_bucket(rec.d24_lb, bshift);
            tx0 = r.x & 0xffffu; ty0 = r.x >> 16;
            const uint32_t tx1 = r.y & 0xffffu, ty1 = r.y >> 16;
            w = tx1 - tx0 + 1;
            cnt = w * (ty1 - ty0 + 1);
            tile_base = vc.tile_base;
            tiles_x = vc.tiles_x;
        }
        // the longer record of the warp's two sets the trip count
        const uint32_t cnt_max = max(cnt, __shfl_xor_sync(0xffffffffu, cnt, 16));
        for (uint32_t k0 = 0; k0 < cnt_max; k0 += 16u) {
            uint32_t pos = 0xffffffffu;
            const uint32_t k = k0 + lane;
            if (k < cnt) {
                const uint32_t t = tile_base + (ty0 + k / w) * tiles_x + tx0 + k % w;
                pos = tile_off[t] + bucket_off[b * n_tiles + t] + atomicAdd(&cursor[b * n_tiles + t], 1u);
                if (pos >= bin_capacity) { dev_error(status, TGX_ERR_DEVICE_FAULT, 3, pos); pos = 0xffffffffu; }
            }
            for (uint32_t q = 0; q < 16u; q++) {
                const uint32_t pq = __shfl_sync(0xffffffffu, pos, src0 + q);
                if (pq != 0xffffffffu && lane < 12u) ew[(uint64_t)pq * 12u + lane] = word;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// 6. per-tile ray/cluster evaluation
// ---------------------------------------------------------------------------

// gmax(gmax(q0, q1), q2) of the near-plane quotients q_i = (p_i - o_i) / d_i
// (p_i = lo_i for d_i > 0, hi_i for d_i < 0; F32_MIN when d_i == 0), each an
// exactly rounded division, as the slab test and the voxel entry of
// visibility.frag compute them.  The maximum is located first with the
// correctly rounded reciprocals r_i (RN(n * RN(1/d)) is within 2^-23 + 2^-24
// relative of the exact quotient); when the largest approximation beats the
// next by more than 4e-6 of their magnitudes, only that axis is divided,
// since its exact quotient is then surely the largest and the maximum of
// distinct values does not depend on the comparison order.  Otherwise (near
// ties, values near underflow or overflow) all three are divided.
__device__ __forceinline__ float max_near_quot(float ox, float oy, float oz, float dx, float dy, float dz, float rx,
                                               float ry, float rz, float lox, float loy, float loz, float hix,
                                               float hiy, float hiz)
{
    // an axis counts when d > 0 or d < 0 (not for 0 or NaN), as in the shader's test
    const bool hx = dx > 0.0f || dx < 0.0f, hy = dy > 0.0f || dy < 0.0f, hz = dz > 0.0f || dz < 0.0f;
    const float nx = dx > 0.0f ? xsub(lox, ox) : xsub(hix, ox);
    const float ny = dy > 0.0f ? xsub(loy, oy) : xsub(hiy, oy);
    const float nz = dz > 0.0f ? xsub(loz, oz) : xsub(hiz, oz);
    const float ninf = __int_as_float(0xff800000);
    const float ax = hx ? xmul(nx, rx) : ninf;
    const float ay = hy ? xmul(ny, ry) : ninf;
    const float az = hz ? xmul(nz, rz) : ninf;
    // the largest approximation and the next one
    float top, next, num, den;
    if (ax >= ay && ax >= az) { top = ax; next = fmaxf(ay, az); num = nx; den = dx; }
    else if (ay >= az)        { top = ay; next = fmaxf(ax, az); num = ny; den = dy; }
    else                      { top = az; next = fmaxf(ax, ay); num = nz; den = dz; }
    const bool normal_top = fabsf(top) <= 1e30f && (top == 0.0f || fabsf(top) >= 1e-30f);
    const bool normal_next = next == ninf || (fabsf(next) <= 1e30f && (next == 0.0f || fabsf(next) >= 1e-30f));
    const bool no_nan = ax == ax && ay == ay && az == az;
    if (no_nan && normal_top && normal_next && (next == ninf || next < top - 4e-6f * (fabsf(top) + fabsf(next))))
        return xdiv(num, den);
    const float qx = hx ? xdiv(nx, dx) : F32_MIN_TG;
    const float qy = hy ? xdiv(ny, dy) : F32_MIN_TG;
    const float qz = hz ? xdiv(nz, dz) : F32_MIN_TG;
    return gmax(gmax(qx, qy), qz);
}

// One (pixel, cluster) fragment of visibility.frag:78-207 given the cluster-space
// ray (o, d), the correctly rounded reciprocals (ix, iy, iz) of its non-zero
// direction components and the cluster's 16 bit words.  Returns the packed
// word or ~0.  The DDA's per-axis steps 1/|d| are |ix| etc. exactly: a
// correctly rounded 1/(-d) is the negated 1/d.  The first voxel is tested
// before the DDA's start distances are computed: a hit there never reads them.
// 2^-k when f = 2^k with 2^-k a normal float, else 0.  For such f,
// RN(v * 2^-k) equals RN(v / f) for every v: both round the same exact real
// once (zeros, infinities and subnormal results included; a NaN stays a NaN).
__device__ __forceinline__ float pow2_reciprocal(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = b >> 23;   // sign 0 and biased exponent
    return (b & 0x7fffffu) == 0u && e >= 1u && e <= 253u ? __uint_as_float((254u - e) << 23) : 0.0f;
}

template <bool kCount = false>
__device__ __forceinline__ unsigned long long vis_pair(float ox, float oy, float oz, float dx, float dy, float dz,
                                                       float ix, float iy, float iz, bool sure_hit,
                                                       const uint32_t* __restrict__ w, uint32_t cluster_pointer,
                                                       float far_plane, float far_rcp, uint32_t* overrun,
                                                       uint32_t* work = nullptr)
{
    float enter;
    if (sure_hit) {
        // the box test surely passes: only the entry distance is needed, and of
        // each axis only the near-plane quotient can be ray_aabb's minimum
        enter = max_near_quot(ox, oy, oz, dx, dy, dz, ix, iy, iz, 0.0f, 0.0f, 0.0f, 8.0f, 8.0f, 8.0f);
    } else {
        float exit_;
        if (!ray_aabb(ox, oy, oz, dx, dy, dz, 0.0f, 0.0f, 0.0f, 8.0f, 8.0f, 8.0f, enter, exit_)) return ULLONG_MAX;
        // a ray parallel to a slab it does not cross is never rasterised
        if ((dx == 0.0f && (ox < 0.0f || ox > 8.0f)) || (dy == 0.0f && (oy < 0.0f || oy > 8.0f)) ||
            (dz == 0.0f && (oz < 0.0f || oz > 8.0f)))
            return ULLONG_MAX;
    }
    if (kCount) work[W_DDAS]++;
    const bool ent = enter > 0.0f;
    const float hx = ent ? xadd(ox, xmul(enter, dx)) : ox;
    const float hy = ent ? xadd(oy, xmul(enter, dy)) : oy;
    const float hz = ent ? xadd(oz, xmul(enter, dz)) : oz;
    int x = (int)gmin(gmax(floorf(hx), 0.0f), 7.0f);
    int y = (int)gmin(gmax(floorf(hy), 0.0f), 7.0f);
    int z = (int)gmin(gmax(floorf(hz), 0.0f), 7.0f);
    uint32_t rvi = 64u * (uint32_t)z + 8u * (uint32_t)y + (uint32_t)x;
    if (kCount) work[W_DDA_STEPS]++;
    bool hit = (w[rvi >> 5] >> (rvi & 31u)) & 1u;
    if (!hit) {
        int sx = 0, sy = 0, sz = 0;
        float tmx = F32_MAX_TG, tmy = F32_MAX_TG, tmz = F32_MAX_TG;
        float tdx = F32_MAX_TG, tdy = F32_MAX_TG, tdz = F32_MAX_TG;
        if (dx > 0.0f) { sx = 1; tmx = xadd(enter, xdiv(xsub((float)(x + 1), hx), dx)); tdx = ix; }
        else if (dx < 0.0f) { sx = -1; tmx = xadd(enter, xdiv(xsub(hx, (float)x), -dx)); tdx = -ix; }
        if (dy > 0.0f) { sy = 1; tmy = xadd(enter, xdiv(xsub((float)(y + 1), hy), dy)); tdy = iy; }
        else if (dy < 0.0f) { sy = -1; tmy = xadd(enter, xdiv(xsub(hy, (float)y), -dy)); tdy = -iy; }
        if (dz > 0.0f) { sz = 1; tmz = xadd(enter, xdiv(xsub((float)(z + 1), hz), dz)); tdz = iz; }
        else if (dz < 0.0f) { sz = -1; tmz = xadd(enter, xdiv(xsub(hz, (float)z), -dz)); tdz = -iz; }
        for (uint32_t step = 1;; step++) {
            if (step >= kMaxDdaSteps) {
                atomicAdd(overrun, 1u);
                return ULLONG_MAX;
            }
            if (tmx < tmy) {
                if (tmx < tmz) { tmx = xadd(tmx, tdx); x += sx; if (x < 0 || x >= 8) return ULLONG_MAX; }
                else           { tmz = xadd(tmz, tdz); z += sz; if (z < 0 || z >= 8) return ULLONG_MAX; }
            } else {
                if (tmy < tmz) { tmy = xadd(tmy, tdy); y += sy; if (y < 0 || y >= 8) return ULLONG_MAX; }
                else           { tmz = xadd(tmz, tdz); z += sz; if (z < 0 || z >= 8) return ULLONG_MAX; }
            }
            rvi = 64u * (uint32_t)z + 8u * (uint32_t)y + (uint32_t)x;
            if (kCount) work[W_DDA_STEPS]++;
            if ((w[rvi >> 5] >> (rvi & 31u)) & 1u) break;
        }
    }
    if (kCount) work[W_HITS]++;
    // entry distance of the voxel box (visibility.frag:155): only the near-plane
    // quotient of each axis can be the maximum, since (vmin-o)/d <= (vmax-o)/d for d>0
    const float fx0 = (float)x, fy0 = (float)y, fz0 = (float)z;
    const float ve = max_near_quot(ox, oy, oz, dx, dy, dz, ix, iy, iz, fx0, fy0, fz0, (float)(x + 1), (float)(y + 1),
                                   (float)(z + 1));
    // a power-of-two far plane (far_rcp != 0) divides by one exact product
    const float depth = gmax(0.0f, far_rcp != 0.0f ? xmul(ve, far_rcp) : xdiv(ve, far_plane));
    if (!(depth <= 1.0f)) return ULLONG_MAX;
    const unsigned long long d24 = __float2uint_rz(xmul(depth, 16777215.0f));   // < 2^24
    return (d24 << 40) | ((unsigned long long)cluster_pointer << 9) | (unsigned long long)rvi;
}

// Conservative classification of the exact box test of vis_pair: kMiss or
// kHit only when the exact test surely gives that answer, else kUnsure.  Slab
// distances use a correctly rounded reciprocal (error < 2 ulp against the
// exact quotient of the same numerator); an answer is given only with a 1e-5
// relative margin.
enum SlabClass { kMiss = 0, kUnsure = 1, kHit = 2 };
__device__ __forceinline__ int slab_class(float ox, float oy, float oz, float dx, float dy, float dz, float ix,
                                          float iy, float iz)
{
    if (ox != ox || oy != oy || oz != oz) return kUnsure;   // NaN origin: the exact test decides
    float en = -3.0e38f, ex = 3.0e38f;
    if (dx == 0.0f) { if (ox < 0.0f || ox > 8.0f) return kMiss; }
    else { const float a = -ox * ix, b = (8.0f - ox) * ix; en = fmaxf(en, fminf(a, b)); ex = fminf(ex, fmaxf(a, b)); }
    if (dy == 0.0f) { if (oy < 0.0f || oy > 8.0f) return kMiss; }
    else { const float a = -oy * iy, b = (8.0f - oy) * iy; en = fmaxf(en, fminf(a, b)); ex = fminf(ex, fmaxf(a, b)); }
    if (dz == 0.0f) { if (oz < 0.0f || oz > 8.0f) return kMiss; }
    else { const float a = -oz * iz, b = (8.0f - oz) * iz; en = fmaxf(en, fminf(a, b)); ex = fminf(ex, fmaxf(a, b)); }
    if (!(fabsf(en) < 1e37f) || !(fabsf(ex) < 1e37f)) return kUnsure;
    const float tol = 1e-5f * (fabsf(en) + fabsf(ex)) + 1e-30f;
    if (ex < -tol || en > ex + 2.0f * tol) return kMiss;
    if (ex > tol && en < ex - 2.0f * tol) return kHit;
    return kUnsure;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// One job's tile inputs: a scene's records and bins for its views.
struct TileJob
{
    const VisRecord* records;
    const uint2* rects;
    const TileEntry* entries;
    const uint32_t* tile_off;
    const uint4* slot_info;      // per launch slot (heavy first): tile, first entry, entry count
    const ViewConst* views;
    const uint32_t* bits;
    const float* inv_rot;
    unsigned long long* const* outs;
    uint32_t* counters;
    uint32_t n_views, n_tiles;
    uint32_t first;              // the job's first item in a multi-job work queue
    unsigned long long* work;    // W_COUNT work counters (counting variant of the tile kernel only)
    uint32_t bshift;             // depth buckets: 32 >> bshift
    uint32_t batch;              // entries per staged batch (1..kBatch)
    uint32_t drain;              // live pairs a warp collects before its lanes run their DDAs (1..32)
    uint32_t extra_tx;           // bytes the first batch's barrier expects beyond its copies: 0, or 64
                                 // under TGX_FLAG_TEST_LOST_COPY (its wait then runs out)
    uint32_t interleave;         // k_vis_tiles: spread the tiles without entries evenly over the launch
                                 // (outputs in host memory), instead of launching them last
};

// Shared memory of a tile CTA (dynamic, tile_smem_bytes(threads)):
//   the mbarrier of the bulk copies, the tile's view and a gather count;
//   the staged batch: up to kBatch of the tile's 96-byte entries;
//   every pixel's best packed word so far (the pair lanes' atomicMin target);
//   per warp, a ring of kQueue live (pixel, entry) pairs waiting for a lane:
//   the pixel's cluster-space direction and reciprocals and the packed
//   lane | entry << 5 | sure_hit << 11.
constexpr uint32_t kBatch = 48;                      // entries per staged batch (k < 64 fits the packed word)
constexpr uint32_t kQueue = 64;                      // ring entries per warp (an entry adds at most 32)
constexpr uint32_t kQueueWords = 7 * kQueue;         // 6 float arrays + the packed word
constexpr uint32_t kSmBar = 0, kSmView = 8, kSmN = 12;
constexpr uint32_t kSmStage = 128;                   // 16-byte aligned bulk-copy target
constexpr uint32_t kSmBest = kSmStage + kBatch * sizeof(TileEntry);
__host__ __device__ constexpr uint32_t tile_smem_bytes(uint32_t threads)
{
    return kSmBest + 8u * threads + (threads / 32u) * kQueueWords * 4u;
}

struct TileSm
{
    unsigned char* p;
    __device__ __forceinline__ uint32_t bar() const { return smem_addr(p + kSmBar); }
    __device__ __forceinline__ uint32_t& view() const { return *(uint32_t*)(p + kSmView); }
    __device__ __forceinline__ uint32_t& n() const { return *(uint32_t*)(p + kSmN); }
    __device__ __forceinline__ TileEntry* stage() const { return (TileEntry*)(p + kSmStage); }
    __device__ __forceinline__ unsigned long long* best() const { return (unsigned long long*)(p + kSmBest); }
    __device__ __forceinline__ uint32_t* queue(uint32_t warp) const
    {
        return (uint32_t*)(p + kSmBest + 8u * blockDim.x) + warp * kQueueWords;
    }
};

__device__ __forceinline__ TileSm tile_sm()
{
    extern __shared__ __align__(128) unsigned char tile_dyn_smem[];
    return TileSm{tile_dyn_smem};
}

__device__ __forceinline__ void tile_smem_init(const TileSm& sm)
{
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(sm.bar()));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

// One bulk copy of n contiguous entries into the stage, completing on the
// CTA's mbarrier (expecting `extra` bytes more than it copies under the
// lost-copy test).  Thread 0 only.
__device__ __forceinline__ void stage_entries(const TileSm& sm, const TileEntry* src, uint32_t n, uint32_t extra)
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(sm.bar()), "r"(n * (uint32_t)sizeof(TileEntry) + extra) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(sm.stage())), "l"(src), "r"(n * (uint32_t)sizeof(TileEntry)), "r"(sm.bar())
                 : "memory");
}

// Tile `slot` (in the job's heavy-first order) of one job: every pixel's
// nearest packed word over the entries binned to the tile.  `phase` is the
// parity of the CTA's bulk-copy mbarrier, carried across tiles.  Returns
// false (the same in every thread) when a batch's copy did not complete in
// time: the status word then holds TGX_ERR_TIMEOUT, the CTA has issued no
// further copy, has waited once more (bounded) for the one in flight and has
// written its pixels' words so far; it must not stage another tile.
//
// The tile's entries (record fields and bitmask, contiguous and sorted near
// to far by depth bucket) arrive kBatch at a time by one cp.async.bulk; the
// first copy is issued before the pixels' rays are set up, so the two
// overlap.  Per batch every lane walks the entries for its own pixel: the
// depth skip, the cluster-space direction (once per object), and the
// conservative slab test.  The pairs that survive are compacted by warp
// ballot into the warp's ring; whenever it holds 32, all 32 lanes take one
// pair each and run the exact entry test and the voxel DDA (vis_pair),
// folding the result into the pixel's word with a shared-memory atomicMin.
// The ring is drained at the end of each batch.  The minimum over a pixel's
// pairs does not depend on the order they are evaluated in (every word is
// distinct), so the buffer is the same bits as one DDA per pair in order.
template <bool kCount = false>
__device__ __forceinline__ bool vis_tile(const TileJob& J, uint32_t slot, const TileSm& sm, uint32_t& phase,
                                         tgx_dev_status* __restrict__ status)
{
    uint32_t work[W_COUNT];
    if (kCount) {
#pragma unroll
        for (int i = 0; i < W_COUNT; i++) work[i] = 0u;
    }
    // the CTA's previous tile is done with the shared state (its generic reads of the stage
    // ordered before the bulk copy that overwrites it)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    const uint4 si = J.slot_info[slot];   // one load: the tile and its entry range
    const uint32_t tile = si.x;
    // bins overflowed this frame: gather every record whose tile rectangle holds the tile (slow, exact)
    const bool scan_all = J.counters[C_OVERFLOW] != 0u;
    const uint32_t begin = scan_all ? 0u : si.y;
    const uint32_t end = scan_all ? J.counters[C_RECORDS] : si.y + si.z;
    if (!scan_all && si.z == 0u) {
        // no entry: the tile is only cleared (no ray set-up, no barrier; the same in every thread)
        uint32_t v = 0;
        while (v + 1 < J.n_views && J.views[v + 1].tile_base <= tile) v++;
        const ViewConst& vc = J.views[v];
        const uint32_t lt = tile - vc.tile_base;
        const uint32_t px = (lt % vc.tiles_x) * vc.tile_w + threadIdx.x % vc.tile_w;
        const uint32_t py = (lt / vc.tiles_x) * vc.tile_h + threadIdx.x / vc.tile_w;
        if (px < vc.width && py < vc.height) J.outs[v][(size_t)py * vc.width + px] = ULLONG_MAX;
        return true;
    }
    if (threadIdx.x == 0) {
        if (!scan_all && end > begin) stage_entries(sm, J.entries + begin, min(J.batch, end - begin), J.extra_tx);
        uint32_t v = 0;
        while (v + 1 < J.n_views && J.views[v + 1].tile_base <= tile) v++;
        sm.view() = v;
    }
    sm.best()[threadIdx.x] = ULLONG_MAX;
    __syncthreads();
    const uint32_t view = sm.view();
    const ViewConst& vc = J.views[view];
    const uint32_t lt = tile - vc.tile_base;
    const uint32_t tx = lt % vc.tiles_x, ty = lt / vc.tiles_x;
    const uint32_t px = tx * vc.tile_w + threadIdx.x % vc.tile_w;
    const uint32_t py = ty * vc.tile_h + threadIdx.x / vc.tile_w;
    const bool valid = px < vc.width && py < vc.height;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t* const q = sm.queue(warp);
    float* const qf = (float*)q;
    const float far_plane = vc.far_plane, far_rcp = pow2_reciprocal(far_plane);
    const TileEntry* const E = sm.stage();
    const uint32_t drain = J.drain;

    // pixel ray in world space (visibility.frag:29-33,68; mix per GLSL 8.3)
    const float fx = xdiv(xadd((float)px, 0.5f), (float)vc.width);
    const float fy = xsub(1.0f, xdiv(xadd((float)py, 0.5f), (float)vc.height));
    float dws[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const float a = xadd(xmul(vc.bl[i], xsub(1.0f, fy)), xmul(vc.tl[i], fy));
        const float b = xadd(xmul(vc.br[i], xsub(1.0f, fy)), xmul(vc.tr[i], fy));
        dws[i] = xadd(xmul(a, xsub(1.0f, fx)), xmul(b, fx));
    }

    uint32_t best_d24 = 0xffffffu;
    uint32_t cur_obj = 0xffffffffu;
    float dx = 0.0f, dy = 0.0f, dz = 0.0f, ix = 0.0f, iy = 0.0f, iz = 0.0f;
    bool lost = false;      // a wait for a batch's copy ran out (the same in every lane of a warp)
    uint32_t qh = 0;        // the warp's ring: first pending entry (warp-uniform)
    for (uint32_t base = begin; base < end;) {
        uint32_t n;
        if (!scan_all) {
            n = min(J.batch, end - base);
            if (base != begin) {
                // the previous batch is fully consumed; after a lost copy nobody stages another
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                if (__syncthreads_or(lost)) break;
                if (threadIdx.x == 0) stage_entries(sm, J.entries + base, n, 0u);
            }
            base += n;
            lost = __any_sync(0xffffffffu, !mbar_wait_bounded(sm.bar(), phase));
            phase ^= 1u;
            if (lost) continue;
        } else {
            // keep the records of this view whose tile rectangle holds this tile, copied into the stage
            __syncthreads();
            if (threadIdx.x == 0) sm.n() = 0;
            __syncthreads();
            const uint32_t m = min(J.batch, end - base);
            for (uint32_t k = threadIdx.x; k < m; k += blockDim.x) {
                const uint32_t r = base + k;
                const uint2 qr = J.rects[r];
                if (J.records[r].view == view && tx >= (qr.x & 0xffffu) && tx <= (qr.y & 0xffffu) &&
                    ty >= (qr.x >> 16) && ty <= (qr.y >> 16)) {
                    const VisRecord& rec = J.records[r];
                    TileEntry& te = sm.stage()[atomicAdd(&sm.n(), 1u)];
                    te.ox = rec.ox; te.oy = rec.oy; te.oz = rec.oz;
                    te.cluster_pointer = rec.cluster_pointer;
                    te.object_idx = rec.object_idx;
                    te.d24_lb = rec.d24_lb;
#pragma unroll
                    for (int w = 0; w < 16; w++) te.bits[w] = J.bits[(uint64_t)rec.cluster_idx * 16u + w];
                }
            }
            base += m;
            __syncthreads();
            n = sm.n();
            if (n == 0) continue;
        }
        if (kCount && valid) work[W_BATCHES]++;
        // produce live pairs entry by entry; drain the ring 32 at a time, and what is left at the end
        uint32_t qn = 0;     // pending entries (warp-uniform)
        for (uint32_t k = 0;;) {
            if (k < n) {
                bool live = false, sure = false;
                if (valid) {
                    if (best_d24 < E[k].d24_lb) {   // cannot produce a smaller word
                        if (kCount) work[W_DEPTH_SKIPS]++;
                    } else {
                        if (kCount) work[W_PAIRS]++;
                        const uint32_t obj = E[k].object_idx;
                        if (obj != cur_obj) {
                            // normalize((ws2ms * v4(dir, 0)).xyz) (visibility.frag:69) with the
                            // object's shared linear part (see k_object_setup)
                            if (kCount) work[W_DIR_SETUPS]++;
                            cur_obj = obj;
                            const float* L = J.inv_rot + 9u * obj;
                            const float ux = xadd(xadd(xmul(dws[0], L[0]), xmul(dws[1], L[1])), xmul(dws[2], L[2]));
                            const float uy = xadd(xadd(xmul(dws[0], L[3]), xmul(dws[1], L[4])), xmul(dws[2], L[5]));
                            const float uz = xadd(xadd(xmul(dws[0], L[6]), xmul(dws[1], L[7])), xmul(dws[2], L[8]));
                            const float mag = xsqrt(xadd(xadd(xmul(ux, ux), xmul(uy, uy)), xmul(uz, uz)));
                            dx = xdiv(ux, mag); dy = xdiv(uy, mag); dz = xdiv(uz, mag);
                            ix = dx != 0.0f ? __frcp_rn(dx) : 0.0f;
                            iy = dy != 0.0f ? __frcp_rn(dy) : 0.0f;
                            iz = dz != 0.0f ? __frcp_rn(dz) : 0.0f;
                        }
                        const int sc = slab_class(E[k].ox, E[k].oy, E[k].oz, dx, dy, dz, ix, iy, iz);
                        live = sc != kMiss;
                        sure = sc == kHit;
                        if (kCount) work[sc == kMiss ? W_SLAB_MISSES : sc == kHit ? W_SURE_HITS : W_EXACT_TESTS]++;
                    }
                }
                const uint32_t m = __ballot_sync(0xffffffffu, live);
                if (live) {
                    const uint32_t e = (qh + qn + __popc(m & ((1u << lane) - 1u))) & (kQueue - 1u);
                    qf[0 * kQueue + e] = dx; qf[1 * kQueue + e] = dy; qf[2 * kQueue + e] = dz;
                    qf[3 * kQueue + e] = ix; qf[4 * kQueue + e] = iy; qf[5 * kQueue + e] = iz;
                    q[6 * kQueue + e] = lane | (k << 5) | ((uint32_t)sure << 11);
                }
                qn += __popc(m);
                k++;
                if (qn < drain && k < n) continue;
            }
            if (qn == 0u) break;   // k == n and nothing pending
            // one pair per lane: the exact test and the DDA; the word goes to its pixel
            const uint32_t take = min(qn, 32u);
            __syncwarp();
            if (lane < take) {
                const uint32_t e = (qh + lane) & (kQueue - 1u);
                const uint32_t pk = q[6 * kQueue + e];
                const TileEntry& te = E[(pk >> 5) & 63u];
                const unsigned long long w = vis_pair<kCount>(
                    te.ox, te.oy, te.oz, qf[0 * kQueue + e], qf[1 * kQueue + e], qf[2 * kQueue + e],
                    qf[3 * kQueue + e], qf[4 * kQueue + e], qf[5 * kQueue + e], (pk >> 11) != 0u, te.bits,
                    te.cluster_pointer, far_plane, far_rcp, &J.counters[C_DDA_OVERRUN], work);
                if (w != ULLONG_MAX) atomicMin(sm.best() + ((warp << 5) | (pk & 31u)), w);
            }
            qh = (qh + take) & (kQueue - 1u);
            qn -= take;
            __syncwarp();
            best_d24 = (uint32_t)(sm.best()[threadIdx.x] >> 40);
        }
        // every pixel already nearer than the rest of the (bucket-sorted) entries: the tile is done
        if (!scan_all && base < end) {
            const uint32_t lo = bucket_lo(depth_bucket(E[n - 1].d24_lb, J.bshift), J.bshift);
            if (__syncthreads_and(!valid || best_d24 < lo)) break;
        }
    }
    const unsigned long long best = sm.best()[threadIdx.x];
    if (__syncthreads_or(lost)) {
        // a batch's copy did not complete: report it, give the copy still in
        // flight one more bounded wait so it does not land after the CTA is
        // gone, and write the words found so far
        if (threadIdx.x == 0) {
            dev_error(status, TGX_ERR_TIMEOUT, 5, tile);
            mbar_wait_bounded(sm.bar(), phase ^ 1u);
        }
        __syncthreads();
        if (valid) J.outs[view][(size_t)py * vc.width + px] = best;
        return false;
    }
    if (valid) J.outs[view][(size_t)py * vc.width + px] = best;
    if (kCount) {
        // per warp: sum the lanes' counters, one 64-bit atomic each
#pragma unroll
        for (int i = 0; i < W_COUNT; i++) {
            unsigned long long v = work[i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0u && v) atomicAdd(&J.work[i], v);
        }
    }
    return true;
}

// Instantiated per block size (= tile pixels) so the register budget can be
// bounded for the occupancy each size needs.  One CTA per tile of one job.
// The slot (heavy-first order, the tiles without entries last) that CTA b of
// t takes.  With interleave, the n non-empty tiles keep their order but are
// spread over the launch, one every t / n CTAs, and the empty ones fill the
// CTAs between: CTA b is the c(b)-th non-empty one when c(b + 1) > c(b), with
// c(b) = floor(b n / t), else the (b - c(b))-th empty one.  Both maps are
// bijections of [0, t).
__device__ __forceinline__ uint32_t tile_slot(uint32_t b, uint32_t t, uint32_t n, bool interleave)
{
    if (!interleave || n >= t) return b;
    const uint32_t c0 = (uint32_t)((uint64_t)b * n / t), c1 = (uint32_t)((uint64_t)(b + 1) * n / t);
    return c1 > c0 ? c0 : n + (b - c0);
}

template <int kThreads, int kMinBlocks, bool kCount = false>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_vis_tiles(TileJob J, tgx_dev_status* __restrict__ status)
{
    const TileSm sm = tile_sm();
    tile_smem_init(sm);
    pdl_wait();
    uint32_t phase = 0;
    const uint32_t slot = J.interleave ? tile_slot(blockIdx.x, J.n_tiles, J.counters[C_NONEMPTY], true) : blockIdx.x;
    vis_tile<kCount>(J, slot, sm, phase, status);
}

// Persistent form over several jobs (scenes, each with its views): CTAs take
// tiles from one work queue in job order, each job's tiles heavy-first, until
// all jobs' tiles are done.
template <int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_vis_tiles_queue(const TileJob* __restrict__ jobs,
                                                                          uint32_t n_jobs, uint32_t total,
                                                                          uint32_t* __restrict__ queue,
                                                                          tgx_dev_status* __restrict__ status)
{
    const TileSm sm = tile_sm();
    __shared__ TileJob s_job;
    __shared__ uint32_t s_slot, s_jobidx;
    tile_smem_init(sm);
    if (threadIdx.x == 0) s_jobidx = 0xffffffffu;
    uint32_t phase = 0;
    for (;;) {
        __syncthreads();   // the previous tile is done with s_job
        if (threadIdx.x == 0) {
            const uint32_t item = atomicAdd(queue, 1u);
            s_slot = 0xffffffffu;
            if (item < total) {
                uint32_t lo = 0, hi = n_jobs - 1;   // the last job whose first item is <= item
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (jobs[mid].first <= item) lo = mid; else hi = mid - 1;
                }
                if (lo != s_jobidx) { s_job = jobs[lo]; s_jobidx = lo; }
                s_slot = item - s_job.first;
            }
        }
        __syncthreads();
        if (s_slot == 0xffffffffu) break;
        if (!vis_tile(s_job, s_slot, sm, phase, status)) break;   // its shared staging is not reusable
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static void make_view_const(const tgx_view& v, uint32_t tile_w, uint32_t tile_h, uint32_t tile_base, ViewConst& c)
{
    memset(&c, 0, sizeof(c));
    for (int i = 0; i < 3; i++) {
        c.cam[i] = v.camera[i];
        c.bl[i] = v.ray_bl[i]; c.br[i] = v.ray_br[i]; c.tr[i] = v.ray_tr[i]; c.tl[i] = v.ray_tl[i];
    }
    c.far_plane = v.far_plane;
    c.width = v.width;
    c.height = v.height;
    c.tile_w = tile_w;
    c.tile_h = tile_h;
    c.tiles_x = (v.width + tile_w - 1) / tile_w;
    c.tiles_y = (v.height + tile_h - 1) / tile_h;
    c.tile_base = tile_base;
    // affine corner-ray model d(fx, fy) = bl + fx (br - bl) + fy (tl - bl):
    // p = s * d  <=>  (s, s fx, s fy) = B^-1 p with B = [bl | br-bl | tl-bl]
    double B[3][3];
    for (int i = 0; i < 3; i++) {
        B[i][0] = v.ray_bl[i];
        B[i][1] = (double)v.ray_br[i] - v.ray_bl[i];
        B[i][2] = (double)v.ray_tl[i] - v.ray_bl[i];
    }
    const double det = B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) - B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
                       B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
    const double inv[9] = {
        (B[1][1] * B[2][2] - B[1][2] * B[2][1]) / det, (B[0][2] * B[2][1] - B[0][1] * B[2][2]) / det,
        (B[0][1] * B[1][2] - B[0][2] * B[1][1]) / det, (B[1][2] * B[2][0] - B[1][0] * B[2][2]) / det,
        (B[0][0] * B[2][2] - B[0][2] * B[2][0]) / det, (B[0][2] * B[1][0] - B[0][0] * B[1][2]) / det,
        (B[1][0] * B[2][1] - B[1][1] * B[2][0]) / det, (B[0][1] * B[2][0] - B[0][0] * B[2][1]) / det,
        (B[0][0] * B[1][1] - B[0][1] * B[1][0]) / det};
    for (int i = 0; i < 9; i++) c.inv_basis[i] = (float)inv[i];
    double f[3], fl = 0.0;
    for (int i = 0; i < 3; i++) {
        f[i] = 0.25 * ((double)v.ray_bl[i] + v.ray_br[i] + v.ray_tr[i] + v.ray_tl[i]);
        fl += f[i] * f[i];
    }
    fl = sqrt(fl);
    for (int i = 0; i < 3; i++) c.fwd[i] = (float)(f[i] / fl);
    // side planes through the camera, spanned by adjacent corner rays, normals pointing inward
    const float* cr[4] = {v.ray_bl, v.ray_br, v.ray_tr, v.ray_tl};
    for (int k = 0; k < 4; k++) {
        const float* a = cr[k];
        const float* b = cr[(k + 1) % 4];
        double n[3] = {(double)a[1] * b[2] - (double)a[2] * b[1], (double)a[2] * b[0] - (double)a[0] * b[2],
                       (double)a[0] * b[1] - (double)a[1] * b[0]};
        const double sgn = n[0] * f[0] + n[1] * f[1] + n[2] * f[2] < 0 ? -1.0 : 1.0;
        const double l = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int i = 0; i < 3; i++) c.planes[3 * k + i] = (float)(sgn * n[i] / l);
    }
}

static tgx_status check_views(const tgx_view* views, uint32_t n_views, uint32_t tile_w, uint32_t tile_h)
{
    if (!views || n_views == 0 || n_views > 65535) { tgx_set_error("views: NULL or count %u out of range", n_views); return TGX_ERR_INVALID_ARGUMENT; }
    for (uint32_t i = 0; i < n_views; i++) {
        const tgx_view& v = views[i];
        if (v.width == 0 || v.height == 0 || (v.width + tile_w - 1) / tile_w > 4095 || (v.height + tile_h - 1) / tile_h > 4095) {
            tgx_set_error("view %u: size %ux%u out of range", i, v.width, v.height);
            return TGX_ERR_INVALID_ARGUMENT;
        }
        if (!(v.far_plane > 0.0f)) { tgx_set_error("view %u: far plane must be > 0", i); return TGX_ERR_INVALID_ARGUMENT; }
    }
    return TGX_OK;
}

// Scratch of one visibility frame (context buffers, or a frame graph's own).
struct VisScratch
{
    VisRecord* records;
    uint2* rects;
    uint32_t rec_cap;
    uint32_t* counters;
    uint32_t* bucket_cnt;
    uint32_t* bucket_off;
    uint32_t* tile_total;
    uint32_t* cta_aux;
    uint32_t* tile_off;
    uint4* slot_info;
    TileEntry* entries;
    uint32_t bin_capacity;     // entries
};

// bytes of the tile-sized part of the scratch
// (the bucket arrays are sized for the finest setting, kMaxBuckets per tile)
static size_t vis_tile_bytes(uint32_t n_tiles)
{
    const uint32_t n_scan_ctas = (n_tiles + kScanTiles - 1) / kScanTiles;
    return (size_t)n_tiles * kMaxBuckets * 4 * 2 + (size_t)n_tiles * 4 + (size_t)n_scan_ctas * (1 + kOrderClasses) * 4;
}

// bytes of the tile offsets (n_tiles + 1 words, padded to 16 bytes) and the slot records
static size_t vis_off_bytes(uint32_t n_tiles)
{
    return (size_t)((n_tiles + 4u) & ~3u) * 4 + (size_t)n_tiles * sizeof(uint4);
}

static void vis_carve_tiles(VisScratch& w, uint32_t* tile_cnt, uint32_t* tile_off, uint32_t n_tiles)
{
    w.bucket_cnt = tile_cnt;
    w.bucket_off = w.bucket_cnt + (size_t)n_tiles * kMaxBuckets;
    w.tile_total = w.bucket_off + (size_t)n_tiles * kMaxBuckets;
    w.cta_aux = w.tile_total + n_tiles;
    w.tile_off = tile_off;
    w.slot_info = reinterpret_cast<uint4*>(w.tile_off + ((n_tiles + 4u) & ~3u));
}

enum VisPhase { VIS_ALL = 0, VIS_TO_SCAN = 1, VIS_FROM_BINS = 2, VIS_NO_TILES = 3 };

static TileJob tile_job(const tgx_ctx* c, const tgx_scene* s, const ViewConst* d_vc, unsigned long long* const* d_outs,
                        uint32_t n_views, uint32_t n_tiles, const VisScratch& w)
{
    TileJob J;
    J.bshift = c->vis_bshift;
    J.batch = c->vis_batch;
    J.drain = c->vis_drain;
    J.records = w.records;
    J.rects = w.rects;
    J.entries = w.entries;
    J.tile_off = w.tile_off;
    J.slot_info = w.slot_info;
    J.views = d_vc;
    J.bits = s->d_bits;
    J.inv_rot = s->d_inv_rot;
    J.outs = d_outs;
    J.counters = w.counters;
    J.n_views = n_views;
    J.n_tiles = n_tiles;
    J.first = 0;
    J.work = nullptr;
    J.extra_tx = 0;
    J.interleave = 0;
    return J;
}

// The launches of one frame (n_views views of scene s, view table d_vc / d_outs
// on the device): all of them, or the part up to the tile scan, or the rest.
static tgx_status vis_launch(tgx_ctx* c, const tgx_scene* s, const ViewConst* d_vc, unsigned long long* const* d_outs,
                             uint32_t n_views, uint32_t n_tiles, const VisScratch& w, int phase = VIS_ALL,
                             bool interleave = false)
{
    const uint64_t n_pairs = (uint64_t)s->n_cluster_pointers * n_views;
    const uint32_t n_scan_ctas = (n_tiles + kScanTiles - 1) / kScanTiles;
    const uint32_t warp_grid = (uint32_t)c->num_sms * 8;
    const uint32_t bshift = c->vis_bshift;
    if (phase != VIS_FROM_BINS) {
        TGX_CUDA(cudaMemsetAsync(w.counters, 0, C_COUNT * sizeof(uint32_t), c->stream));
        const uint32_t setup_blocks = (uint32_t)((n_pairs + 255) / 256);
        TGX_LAUNCH(c, TR_VIS_SETUP, setup_blocks, 256, 0, k_vis_cluster_setup<true>,
                   s->d_objects, s->d_cluster_pointers, s->d_c2o, s->d_bits, s->d_cp_obj, s->n_cluster_pointers,
                   d_vc, n_views, w.records, w.rects, w.rec_cap, w.counters, w.bucket_cnt,
                   n_tiles * (kMaxBuckets >> bshift), c->d_status);
        // each later pass is a programmatic dependent of the one before
        TGX_LAUNCH_PDL(c, TR_VIS_COUNT, warp_grid, 256, 0, k_vis_count, w.records, w.rects, w.counters, w.rec_cap,
                       s->d_objects, d_vc, w.bucket_cnt, n_tiles, bshift);
        if (bshift == 0)
            TGX_LAUNCH_PDL(c, TR_VIS_PREFIX, n_scan_ctas, kScanTiles, 0, k_vis_prefix<32>, w.bucket_cnt, w.bucket_off,
                           w.tile_total, n_tiles, w.cta_aux);
        else if (bshift == 1)
            TGX_LAUNCH_PDL(c, TR_VIS_PREFIX, n_scan_ctas, kScanTiles, 0, k_vis_prefix<16>, w.bucket_cnt, w.bucket_off,
                           w.tile_total, n_tiles, w.cta_aux);
        else
            TGX_LAUNCH_PDL(c, TR_VIS_PREFIX, n_scan_ctas, kScanTiles, 0, k_vis_prefix<8>, w.bucket_cnt, w.bucket_off,
                           w.tile_total, n_tiles, w.cta_aux);
        if (n_scan_ctas <= kDirectGroups) {
            TGX_LAUNCH_PDL(c, TR_VIS_SCAN, n_scan_ctas, kScanTiles, 0, k_vis_finalize_direct, w.tile_total, n_tiles,
                           w.cta_aux, w.tile_off, w.slot_info, w.bin_capacity, w.counters);
        } else {
            TGX_LAUNCH_PDL(c, TR_VIS_SCAN, 1, 1024, 0, k_vis_scan, w.cta_aux, n_tiles, w.tile_off, w.bin_capacity,
                           w.counters);
            TGX_LAUNCH_PDL(c, TR_VIS_SCAN, n_scan_ctas, kScanTiles, 0, k_vis_finalize, w.tile_total, n_tiles,
                           w.cta_aux, w.tile_off, w.slot_info);
        }
    }
    if (phase == VIS_TO_SCAN) return TGX_OK;
    TGX_LAUNCH_PDL(c, TR_VIS_BIN, warp_grid, 256, 0, k_vis_bin_fill,
                   w.records, w.rects, w.counters, d_vc, w.tile_off, w.bucket_off, w.bucket_cnt, w.entries,
                   s->d_bits, n_tiles, w.bin_capacity, bshift, c->d_status);
    if (phase == VIS_NO_TILES) return TGX_OK;
    TileJob J = tile_job(c, s, d_vc, d_outs, n_views, n_tiles, w);
    J.interleave = interleave ? 1u : 0u;
    if (c->flags & TGX_FLAG_TEST_LOST_COPY) J.extra_tx = 64u;
    const uint32_t threads = c->tile_w * c->tile_h, smem = tile_smem_bytes(threads);
    if (c->vis_count_work) {
        // the counting variant (tgx_vis_count_work): same results, plus the work counters
        TGX_TRY(devbuf_reserve(c->vis_work, W_COUNT * sizeof(unsigned long long)));
        J.work = (unsigned long long*)c->vis_work.ptr;
        TGX_CUDA(cudaMemsetAsync(J.work, 0, W_COUNT * sizeof(unsigned long long), c->stream));
        if (threads == 64) TGX_LAUNCH(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<64, 16, true>), J, c->d_status);
        else if (threads == 128) TGX_LAUNCH(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<128, 10, true>), J, c->d_status);
        else if (threads == 256) TGX_LAUNCH(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<256, 5, true>), J, c->d_status);
        else TGX_LAUNCH(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<512, 2, true>), J, c->d_status);
        return TGX_OK;
    }
    if (threads == 64) TGX_LAUNCH_PDL(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<64, 16>), J, c->d_status);
    else if (threads == 128) TGX_LAUNCH_PDL(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<128, 10>), J, c->d_status);
    else if (threads == 256) TGX_LAUNCH_PDL(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<256, 5>), J, c->d_status);
    else TGX_LAUNCH_PDL(c, TR_VIS_TILES, n_tiles, threads, smem, (k_vis_tiles<512, 2>), J, c->d_status);
    return TGX_OK;
}

// Once per context, with its device current: the persistent tile kernel's
// resident CTAs for the context's tile size (an occupancy query, so it is made
// outside any stream capture).
template <int kThreads, int kMinBlocks>
static uint32_t vis_queue_per_sm()
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vis_tiles_queue<kThreads, kMinBlocks>, kThreads,
                                                      tile_smem_bytes(kThreads)) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return (uint32_t)per_sm;
}

tgx_status vis_prepare_device(tgx_ctx* c)
{
    const uint32_t threads = c->tile_w * c->tile_h;
    const uint32_t per_sm = threads == 64 ? vis_queue_per_sm<64, 16>() : threads == 128 ? vis_queue_per_sm<128, 10>()
                          : threads == 256 ? vis_queue_per_sm<256, 5>() : vis_queue_per_sm<512, 2>();
    c->vis_tile_ctas = (uint32_t)c->num_sms * per_sm;
    return TGX_OK;
}

// The tile stage of several jobs as one persistent launch over a work queue
// (d_jobs: the jobs' TileJob records with their first queue items; d_queue
// zeroed here).
static tgx_status vis_launch_queue(tgx_ctx* c, const TileJob* d_jobs, uint32_t n_jobs, uint32_t total, uint32_t* d_queue)
{
    TGX_CUDA(cudaMemsetAsync(d_queue, 0, 4, c->stream));
    const uint32_t threads = c->tile_w * c->tile_h, smem = tile_smem_bytes(threads);
    const uint32_t grid = std::max(1u, std::min(c->vis_tile_ctas, total));
#define QUEUE_ARGS d_jobs, n_jobs, total, d_queue, c->d_status
    if (threads == 64) TGX_LAUNCH(c, TR_VIS_TILES, grid, threads, smem, (k_vis_tiles_queue<64, 16>), QUEUE_ARGS);
    else if (threads == 128) TGX_LAUNCH(c, TR_VIS_TILES, grid, threads, smem, (k_vis_tiles_queue<128, 10>), QUEUE_ARGS);
    else if (threads == 256) TGX_LAUNCH(c, TR_VIS_TILES, grid, threads, smem, (k_vis_tiles_queue<256, 5>), QUEUE_ARGS);
    else TGX_LAUNCH(c, TR_VIS_TILES, grid, threads, smem, (k_vis_tiles_queue<512, 2>), QUEUE_ARGS);
#undef QUEUE_ARGS
    return TGX_OK;
}

// host view table: ViewConst per view (tile bases) and the output pointer table
static std::vector<unsigned char> vis_view_table(tgx_ctx* c, const tgx_view* views, uint32_t n_views,
                                                 uint64_t* const* d_visbuf, uint32_t& n_tiles, size_t& ptr_off)
{
    std::vector<ViewConst> vcs(n_views);
    n_tiles = 0;
    for (uint32_t i = 0; i < n_views; i++) {
        make_view_const(views[i], c->tile_w, c->tile_h, n_tiles, vcs[i]);
        n_tiles += vcs[i].tiles_x * vcs[i].tiles_y;
    }
    const size_t vc_bytes = n_views * sizeof(ViewConst);
    ptr_off = (vc_bytes + 15) & ~(size_t)15;
    std::vector<unsigned char> stage(ptr_off + n_views * sizeof(void*));
    memcpy(stage.data(), vcs.data(), vc_bytes);
    memcpy(stage.data() + ptr_off, d_visbuf, n_views * sizeof(void*));
    return stage;
}

tgx_status vis_render_device(tgx_ctx* c, const tgx_scene* s, const tgx_view* views, uint32_t n_views,
                             uint64_t* const* d_visbuf, bool host_out)
{
    if (!c || !s || !d_visbuf) { tgx_set_error("tgx_vis_render: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    TGX_TRY(check_views(views, n_views, c->tile_w, c->tile_h));
    for (uint32_t i = 0; i < n_views; i++)
        if (!d_visbuf[i]) { tgx_set_error("tgx_vis_render: output %u is NULL", i); return TGX_ERR_INVALID_ARGUMENT; }
    TGX_CUDA(cudaSetDevice(c->device));

    // view constants + output pointer table, copied from pageable memory (staged by the driver, no sync)
    uint32_t n_tiles = 0;
    size_t ptr_off = 0;
    const std::vector<unsigned char> stage = vis_view_table(c, views, n_views, d_visbuf, n_tiles, ptr_off);
    TGX_TRY(devbuf_reserve(c->vis_views, stage.size()));
    TGX_CUDA(cudaMemcpyAsync(c->vis_views.ptr, stage.data(), stage.size(), cudaMemcpyHostToDevice, c->stream));
    const ViewConst* d_vc = (const ViewConst*)c->vis_views.ptr;
    unsigned long long* const* d_outs = (unsigned long long* const*)((char*)c->vis_views.ptr + ptr_off);

    // bin capacity: grown from earlier frames' totals (read back without waiting); a frame
    // that still overflows is rendered correctly by the tile kernel's record scan
    // Bin capacity.  Grown from earlier frames' totals, read back without
    // waiting.  A frame that could outgrow what is known (the first one, one
    // with more tiles or (view, cluster) pairs than before, or the one after an
    // overflow) is sized exactly instead: the host reads this frame's total
    // after the tile scan, once.  A frame that still overflows is rendered
    // correctly, but slowly, by the tile kernel's record scan.
    const uint64_t n_pairs = (uint64_t)s->n_cluster_pointers * n_views;
    if (n_pairs > 0xffffffffull) { tgx_set_error("too many (view, cluster) pairs"); return TGX_ERR_CAPACITY; }
    VisScratch w;
    bool exact = false;
    constexpr size_t kEntry = sizeof(TileEntry);
    if (c->flags & TGX_FLAG_MIN_BIN_CAPACITY) {
        TGX_TRY(devbuf_reserve(c->vis_bins, 64 * kEntry));
        w.bin_capacity = 64;
    } else {
        exact = c->vis_last_tiles == 0 || n_tiles > c->vis_last_tiles || n_pairs > c->vis_last_pairs;
        if (c->vis_done && cudaEventQuery(c->vis_done) == cudaSuccess) {
            const uint32_t* hc = (const uint32_t*)c->h_vis_counters;
            if (hc[C_OVERFLOW]) exact = true;
            if ((size_t)hc[C_ENTRIES] * 2 > c->vis_bins.bytes / kEntry)
                TGX_TRY(devbuf_reserve(c->vis_bins, (size_t)hc[C_ENTRIES] * 2 * kEntry));
        }
        cudaGetLastError();
        TGX_TRY(devbuf_reserve(c->vis_bins, std::max<size_t>((size_t)n_tiles * 16, (size_t)1 << 18) * kEntry));
        w.bin_capacity = (uint32_t)std::min<size_t>(c->vis_bins.bytes / kEntry, 0xffffffffu);
    }
    w.rec_cap = (uint32_t)n_pairs;
    TGX_TRY(devbuf_reserve(c->vis_records, (size_t)w.rec_cap * (sizeof(VisRecord) + sizeof(uint2))));
    TGX_TRY(devbuf_reserve(c->vis_counters, C_COUNT * sizeof(uint32_t)));
    TGX_TRY(devbuf_reserve(c->vis_tile_cnt, vis_tile_bytes(n_tiles)));
    TGX_TRY(devbuf_reserve(c->vis_tile_off, vis_off_bytes(n_tiles)));
    w.records = (VisRecord*)c->vis_records.ptr;
    w.rects = (uint2*)(w.records + w.rec_cap);
    w.counters = (uint32_t*)c->vis_counters.ptr;
    w.entries = (TileEntry*)c->vis_bins.ptr;
    vis_carve_tiles(w, (uint32_t*)c->vis_tile_cnt.ptr, (uint32_t*)c->vis_tile_off.ptr, n_tiles);
    if (!exact) {
        TGX_TRY(vis_launch(c, s, d_vc, d_outs, n_views, n_tiles, w, VIS_ALL, host_out));
    } else {
        TGX_TRY(vis_launch(c, s, d_vc, d_outs, n_views, n_tiles, w, VIS_TO_SCAN, host_out));
        TGX_CUDA(cudaMemcpyAsync(c->h_vis_counters, w.counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
        TGX_CUDA(cudaStreamSynchronize(c->stream));
        const uint32_t entries = ((const uint32_t*)c->h_vis_counters)[C_ENTRIES];
        if (entries > w.bin_capacity) {
            TGX_TRY(devbuf_reserve(c->vis_bins, (size_t)entries * kEntry));
            w.entries = (TileEntry*)c->vis_bins.ptr;
            w.bin_capacity = (uint32_t)std::min<size_t>(c->vis_bins.bytes / kEntry, 0xffffffffu);
            if (entries <= w.bin_capacity) TGX_CUDA(cudaMemsetAsync(w.counters + C_OVERFLOW, 0, 4, c->stream));
        }
        TGX_TRY(vis_launch(c, s, d_vc, d_outs, n_views, n_tiles, w, VIS_FROM_BINS, host_out));
    }
    c->vis_last_tiles = n_tiles;
    c->vis_last_pairs = n_pairs;
    // counters of this frame to pinned memory, read by the next call without waiting
    TGX_CUDA(cudaMemcpyAsync(c->h_vis_counters, w.counters, C_COUNT * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    if (!c->vis_done) TGX_CUDA(cudaEventCreateWithFlags(&c->vis_done, cudaEventDisableTiming));
    TGX_CUDA(cudaEventRecord(c->vis_done, c->stream));
    return TGX_OK;
}

// ---------------------------------------------------------------------------
// batched frames: the visibility passes of many jobs captured as one CUDA graph
// ---------------------------------------------------------------------------

struct tgx_frame_graph
{
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void* d_mem = nullptr;                       // view tables, then the shared scratch
    struct Job
    {
        const tgx_scene* scene;
        std::vector<tgx_view> views;             // resolutions fixed at capture
        std::vector<uint64_t*> outs;
        size_t table_off, ptr_off;
        uint32_t n_tiles;
        uint64_t rec_cap, bin_cap;               // this job's own scratch
        size_t scratch_off;
    };
    std::vector<Job> jobs;
    uint32_t kernels = 0;
};

static void frame_graph_free(tgx_frame_graph* g)
{
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaFree(g->d_mem);
    delete g;
}

extern "C" tgx_status tgx_frame_graph_create(tgx_ctx* c, const tgx_vis_job* jobs, uint32_t n_jobs,
                                             tgx_frame_graph** out)
{
    if (!c || !jobs || !n_jobs || !out) { tgx_set_error("tgx_frame_graph_create: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    TGX_CUDA(cudaSetDevice(c->device));
    tgx_frame_graph* g = new (std::nothrow) tgx_frame_graph();
    if (!g) return TGX_ERR_OUT_OF_MEMORY;
    auto fail = [&](tgx_status st) { cudaStreamSynchronize(c->stream); frame_graph_free(g); return st; };
    // sizes, and one uncaptured frame per job to size its bins
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t table_bytes = 0, scratch_bytes = 0;
    uint32_t total_tiles = 0;
    std::vector<std::vector<unsigned char>> tables(n_jobs);
    auto job_bytes = [&](const tgx_frame_graph::Job& job) {
        return al((size_t)job.rec_cap * (sizeof(VisRecord) + sizeof(uint2))) + 256 + al(vis_tile_bytes(job.n_tiles)) +
               al(vis_off_bytes(job.n_tiles)) + al((size_t)job.bin_cap * sizeof(TileEntry));
    };
    for (uint32_t j = 0; j < n_jobs; j++) {
        const tgx_vis_job& jb = jobs[j];
        if (!jb.scene || !jb.views || !jb.d_visbuf || !jb.n_views) {
            tgx_set_error("tgx_frame_graph_create: job %u has a NULL member or no views", j);
            return fail(TGX_ERR_INVALID_ARGUMENT);
        }
        tgx_status st = vis_render_device(c, jb.scene, jb.views, jb.n_views, jb.d_visbuf);
        if (st != TGX_OK) return fail(st);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) { tgx_set_error("tgx_frame_graph_create: frame failed"); return fail(TGX_ERR_CUDA); }
        const uint32_t entries = ((const uint32_t*)c->h_vis_counters)[C_ENTRIES];
        tgx_frame_graph::Job job;
        job.scene = jb.scene;
        job.views.assign(jb.views, jb.views + jb.n_views);
        job.outs.assign(jb.d_visbuf, jb.d_visbuf + jb.n_views);
        tables[j] = vis_view_table(c, jb.views, jb.n_views, jb.d_visbuf, job.n_tiles, job.ptr_off);
        job.table_off = table_bytes;
        table_bytes += al(tables[j].size());
        job.rec_cap = (uint64_t)jb.scene->n_cluster_pointers * jb.n_views;
        job.bin_cap = std::max<uint64_t>(1u << 14, std::max<uint64_t>((uint64_t)job.n_tiles * 4, (uint64_t)entries * 3 / 2));
        if (job.rec_cap > 0xffffffffull || job.bin_cap > 0xffffffffull || (uint64_t)total_tiles + job.n_tiles > 0xffffffffull) {
            tgx_set_error("tgx_frame_graph_create: job %u has too many (view, cluster) pairs or tiles", j);
            return fail(TGX_ERR_CAPACITY);
        }
        total_tiles += job.n_tiles;
        job.scratch_off = scratch_bytes;
        scratch_bytes += job_bytes(job);
        g->jobs.push_back(std::move(job));
    }
    const size_t jobs_off = table_bytes + scratch_bytes;
    const size_t total = jobs_off + al((size_t)n_jobs * sizeof(TileJob)) + 256;
    if (cudaMalloc(&g->d_mem, total) != cudaSuccess) {
        cudaGetLastError();
        tgx_set_error("tgx_frame_graph_create: out of device memory (%zu bytes)", total);
        return fail(TGX_ERR_OUT_OF_MEMORY);
    }
    char* base = (char*)g->d_mem;
    for (uint32_t j = 0; j < n_jobs; j++)
        if (cudaMemcpy(base + g->jobs[j].table_off, tables[j].data(), tables[j].size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            tgx_set_error("tgx_frame_graph_create: view table upload failed");
            return fail(TGX_ERR_CUDA);
        }
    // each job's own scratch, so the jobs' sorting passes can run side by side
    std::vector<VisScratch> ws(n_jobs);
    std::vector<TileJob> tjobs(n_jobs);
    for (uint32_t j = 0; j < n_jobs; j++) {
        const tgx_frame_graph::Job& job = g->jobs[j];
        VisScratch& w = ws[j];
        char* p = base + table_bytes + job.scratch_off;
        w.records = (VisRecord*)p;
        w.rec_cap = (uint32_t)job.rec_cap;
        w.rects = (uint2*)(w.records + job.rec_cap);
        p += al((size_t)job.rec_cap * (sizeof(VisRecord) + sizeof(uint2)));
        w.counters = (uint32_t*)p;
        p += 256;
        uint32_t* tile_cnt = (uint32_t*)p;
        p += al(vis_tile_bytes(job.n_tiles));
        uint32_t* tile_off = (uint32_t*)p;
        p += al(vis_off_bytes(job.n_tiles));
        w.entries = (TileEntry*)p;
        w.bin_capacity = (uint32_t)job.bin_cap;
        vis_carve_tiles(w, tile_cnt, tile_off, job.n_tiles);
        const ViewConst* d_vc = (const ViewConst*)(base + job.table_off);
        unsigned long long* const* d_outs = (unsigned long long* const*)(base + job.table_off + job.ptr_off);
        tjobs[j] = tile_job(c, job.scene, d_vc, d_outs, (uint32_t)job.views.size(), job.n_tiles, w);
        tjobs[j].first = j ? tjobs[j - 1].first + g->jobs[j - 1].n_tiles : 0u;
    }
    TileJob* d_jobs = (TileJob*)(base + jobs_off);
    uint32_t* d_queue = (uint32_t*)(base + jobs_off + al((size_t)n_jobs * sizeof(TileJob)));
    if (cudaMemcpy(d_jobs, tjobs.data(), n_jobs * sizeof(TileJob), cudaMemcpyHostToDevice) != cudaSuccess) {
        tgx_set_error("tgx_frame_graph_create: job table upload failed");
        return fail(TGX_ERR_CUDA);
    }
    // side streams and events for the fork and join inside the capture
    const uint32_t n_side = std::min<uint32_t>(n_jobs, 8u);
    std::vector<cudaStream_t> side(n_side, nullptr);
    std::vector<cudaEvent_t> done(n_jobs, nullptr);
    cudaEvent_t fork = nullptr;
    auto release = [&]() {
        for (cudaStream_t q : side) if (q) cudaStreamDestroy(q);
        for (cudaEvent_t e : done) if (e) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
    };
    bool ok = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) == cudaSuccess;
    for (uint32_t k = 0; k < n_side && ok; k++) ok = cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking) == cudaSuccess;
    for (uint32_t j = 0; j < n_jobs && ok; j++) ok = cudaEventCreateWithFlags(&done[j], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        release();
        tgx_set_error("tgx_frame_graph_create: stream or event creation failed");
        return fail(TGX_ERR_CUDA);
    }
    // capture (no trace events inside the graph): every job's passes up to the
    // bins on its side stream, then one persistent tile launch over all jobs
    const bool tracing = c->trace.enabled;
    c->trace.enabled = false;
    const uint64_t launches0 = c->launches;
    cudaStream_t main_stream = c->stream;
    if (cudaStreamBeginCapture(main_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        c->trace.enabled = tracing;
        release();
        tgx_set_error("tgx_frame_graph_create: stream capture refused (%s)", cudaGetErrorString(cudaGetLastError()));
        return fail(TGX_ERR_CUDA);
    }
    tgx_status st = TGX_OK;
    if (n_jobs == 1) {
        // one job: its passes and its own tile launch, no fork
        const tgx_frame_graph::Job& job = g->jobs[0];
        const ViewConst* d_vc = (const ViewConst*)(base + job.table_off);
        unsigned long long* const* d_outs = (unsigned long long* const*)(base + job.table_off + job.ptr_off);
        st = vis_launch(c, job.scene, d_vc, d_outs, (uint32_t)job.views.size(), job.n_tiles, ws[0], VIS_ALL);
        goto captured;
    }
    if (cudaEventRecord(fork, main_stream) != cudaSuccess) st = TGX_ERR_CUDA;
    for (uint32_t k = 0; k < n_side && st == TGX_OK; k++)
        if (cudaStreamWaitEvent(side[k], fork, 0) != cudaSuccess) st = TGX_ERR_CUDA;
    for (uint32_t j = 0; j < n_jobs && st == TGX_OK; j++) {
        const tgx_frame_graph::Job& job = g->jobs[j];
        c->stream = side[j % n_side];
        const ViewConst* d_vc = (const ViewConst*)(base + job.table_off);
        unsigned long long* const* d_outs = (unsigned long long* const*)(base + job.table_off + job.ptr_off);
        st = vis_launch(c, job.scene, d_vc, d_outs, (uint32_t)job.views.size(), job.n_tiles, ws[j], VIS_NO_TILES);
        if (st == TGX_OK && cudaEventRecord(done[j], c->stream) != cudaSuccess) st = TGX_ERR_CUDA;
    }
    c->stream = main_stream;
    for (uint32_t j = 0; j < n_jobs && st == TGX_OK; j++)
        if (cudaStreamWaitEvent(main_stream, done[j], 0) != cudaSuccess) st = TGX_ERR_CUDA;
    if (st == TGX_OK) st = vis_launch_queue(c, d_jobs, n_jobs, total_tiles, d_queue);
captured:
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &g->graph);
    release();
    c->trace.enabled = tracing;
    g->kernels = (uint32_t)(c->launches - launches0);
    c->launches = launches0;
    if (st != TGX_OK) return fail(st);
    if (ce != cudaSuccess || cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) {
        tgx_set_error("tgx_frame_graph_create: graph capture failed (%s)", cudaGetErrorString(cudaGetLastError()));
        return fail(TGX_ERR_CUDA);
    }
    *out = g;
    return TGX_OK;
}

extern "C" tgx_status tgx_frame_graph_launch(tgx_ctx* c, tgx_frame_graph* g)
{
    if (!c || !g) return TGX_ERR_INVALID_ARGUMENT;
    TGX_CUDA(cudaGraphLaunch(g->exec, c->stream));
    c->launches += g->kernels;
    return TGX_OK;
}

extern "C" tgx_status tgx_frame_graph_set_views(tgx_ctx* c, tgx_frame_graph* g, uint32_t job, const tgx_view* views)
{
    if (!c || !g || !views || job >= g->jobs.size()) return TGX_ERR_INVALID_ARGUMENT;
    tgx_frame_graph::Job& jb = g->jobs[job];
    const uint32_t n = (uint32_t)jb.views.size();
    for (uint32_t i = 0; i < n; i++)
        if (views[i].width != jb.views[i].width || views[i].height != jb.views[i].height) {
            tgx_set_error("tgx_frame_graph_set_views: view %u changes its resolution", i);
            return TGX_ERR_INVALID_ARGUMENT;
        }
    TGX_TRY(check_views(views, n, c->tile_w, c->tile_h));
    uint32_t n_tiles = 0;
    size_t ptr_off = 0;
    const std::vector<unsigned char> t = vis_view_table(c, views, n, jb.outs.data(), n_tiles, ptr_off);
    // the pinned-free staging copy is ordered on the stream before the next launch
    TGX_CUDA(cudaMemcpyAsync((char*)g->d_mem + jb.table_off, t.data(), t.size(), cudaMemcpyHostToDevice, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    jb.views.assign(views, views + n);
    return TGX_OK;
}

extern "C" uint32_t tgx_frame_graph_kernels(const tgx_frame_graph* g) { return g ? g->kernels : 0u; }

extern "C" void tgx_frame_graph_destroy(tgx_ctx* c, tgx_frame_graph* g)
{
    if (c) cudaStreamSynchronize(c->stream);
    frame_graph_free(g);
}

extern "C" tgx_status tgx_vis_render(tgx_ctx* c, const tgx_scene* s, const tgx_view* views, uint32_t n_views,
                                     uint64_t* const* d_visbuf)
{
    return vis_render_device(c, s, views, n_views, d_visbuf);
}

// The device address of pinned (page-locked, mapped) host memory, or null for
// any other pointer.  The tile kernel stores each pixel once, so it can write
// a pinned host buffer directly over the CPU-GPU link, hidden under its own
// work, instead of through a device buffer and a copy.
static uint64_t* mapped_host(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost && a.devicePointer ? (uint64_t*)a.devicePointer : nullptr;
}

// whether some output of a host-buffer render is written in host memory directly
static bool any_mapped(const std::vector<bool>& staged)
{
    for (bool st : staged)
        if (!st) return true;
    return false;
}

// Output pointers of a host-buffer render: pinned buffers directly, the rest
// in `stage` (device memory, `staged` entries) for a copy afterwards.
static tgx_status host_outputs(tgx_ctx* c, const tgx_view* views, uint32_t n_views, uint64_t* const* h_visbuf,
                               DevBuf& stage, std::vector<uint64_t*>& dptr, std::vector<bool>& staged, const char* who)
{
    size_t total = 0;
    std::vector<size_t> offs(n_views);
    dptr.assign(n_views, nullptr);
    staged.assign(n_views, false);
    for (uint32_t i = 0; i < n_views; i++) {
        if (!h_visbuf[i]) { tgx_set_error("%s: output %u is NULL", who, i); return TGX_ERR_INVALID_ARGUMENT; }
        dptr[i] = mapped_host(h_visbuf[i]);
        if (dptr[i]) continue;
        staged[i] = true;
        offs[i] = total;
        total += (size_t)views[i].width * views[i].height;
    }
    if (total) TGX_TRY(devbuf_reserve(stage, total * 8));
    for (uint32_t i = 0; i < n_views; i++)
        if (staged[i]) dptr[i] = (uint64_t*)stage.ptr + offs[i];
    return TGX_OK;
}

extern "C" tgx_status tgx_vis_render_host(tgx_ctx* c, const tgx_scene* s, const tgx_view* views, uint32_t n_views,
                                          uint64_t* const* h_visbuf)
{
    if (!c || !s || !h_visbuf) { tgx_set_error("tgx_vis_render_host: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    TGX_TRY(check_views(views, n_views, c->tile_w, c->tile_h));
    TGX_CUDA(cudaSetDevice(c->device));
    std::vector<uint64_t*> dptr;
    std::vector<bool> staged;
    TGX_TRY(host_outputs(c, views, n_views, h_visbuf, c->host_stage, dptr, staged, "tgx_vis_render_host"));
    TGX_TRY(vis_render_device(c, s, views, n_views, dptr.data(), any_mapped(staged)));
    for (uint32_t i = 0; i < n_views; i++)
        if (staged[i])
            TGX_CUDA(cudaMemcpyAsync(h_visbuf[i], dptr[i], (size_t)views[i].width * views[i].height * 8,
                                     cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

// Pinned host buffers are written by the render itself.  Other buffers go
// through two device copies that alternate between frames: frame k renders
// into copy k % 2 on the context stream once frame k-2's copy out of it is
// done (an event wait on the device, not the host), then the copy stream
// takes it to the host while frame k+1 renders into the other copy.
extern "C" tgx_status tgx_vis_render_host_async(tgx_ctx* c, const tgx_scene* s, const tgx_view* views,
                                                uint32_t n_views, uint64_t* const* h_visbuf)
{
    if (!c || !s || !h_visbuf) {
        tgx_set_error("tgx_vis_render_host_async: NULL argument");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    TGX_TRY(check_views(views, n_views, c->tile_w, c->tile_h));
    TGX_CUDA(cudaSetDevice(c->device));
    if (!c->copy_stream) {
        TGX_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; i++) {
            TGX_CUDA(cudaEventCreateWithFlags(&c->host_rendered[i], cudaEventDisableTiming));
            TGX_CUDA(cudaEventCreateWithFlags(&c->host_copied[i], cudaEventDisableTiming));
        }
    }
    const uint32_t slot = (uint32_t)(c->host_issued & 1u);
    // the copy two frames back reads this slot: the render waits for it on the device
    TGX_CUDA(cudaStreamWaitEvent(c->stream, c->host_copied[slot], 0));
    std::vector<uint64_t*> dptr;
    std::vector<bool> staged;
    TGX_TRY(host_outputs(c, views, n_views, h_visbuf, c->host_slot[slot], dptr, staged, "tgx_vis_render_host_async"));
    TGX_TRY(vis_render_device(c, s, views, n_views, dptr.data(), any_mapped(staged)));
    TGX_CUDA(cudaEventRecord(c->host_rendered[slot], c->stream));
    TGX_CUDA(cudaStreamWaitEvent(c->copy_stream, c->host_rendered[slot], 0));
    for (uint32_t i = 0; i < n_views; i++)
        if (staged[i])
            TGX_CUDA(cudaMemcpyAsync(h_visbuf[i], dptr[i], (size_t)views[i].width * views[i].height * 8,
                                     cudaMemcpyDeviceToHost, c->copy_stream));
    // marks the frame done: after its copies, or after its render when it wrote the host directly
    TGX_CUDA(cudaEventRecord(c->host_copied[slot], c->copy_stream));
    c->host_issued++;
    return TGX_OK;
}

extern "C" tgx_status tgx_vis_host_wait(tgx_ctx* c, uint32_t max_in_flight)
{
    if (!c) { tgx_set_error("tgx_vis_host_wait: NULL context"); return TGX_ERR_INVALID_ARGUMENT; }
    while (c->host_issued - c->host_done > max_in_flight) {
        // copies complete in issue order; the slot's event is that of its latest frame
        TGX_CUDA(cudaEventSynchronize(c->host_copied[c->host_done & 1u]));
        c->host_done++;
    }
    return TGX_OK;
}

extern "C" tgx_status tgx_vis_get_stats(tgx_ctx* c, tgx_vis_stats* out)
{
    if (!c || !out) return TGX_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    if (!c->vis_counters.ptr) return TGX_OK;
    uint32_t h[C_COUNT];
    TGX_CUDA(cudaMemcpyAsync(c->h_counter, c->vis_counters.ptr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    memcpy(h, c->h_counter, sizeof(h));
    out->visible_clusters = h[C_RECORDS];
    out->bin_entries = h[C_ENTRIES];
    out->dda_overruns = h[C_DDA_OVERRUN];
    out->tiles = c->vis_last_tiles;
    return TGX_OK;
}

extern "C" tgx_status tgx_set_vis_tuning(tgx_ctx* c, uint32_t depth_buckets, uint32_t batch, uint32_t drain)
{
    if (!c) return TGX_ERR_INVALID_ARGUMENT;
    const uint32_t nb = depth_buckets ? depth_buckets : 16u, bt = batch ? batch : kBatch, dr = drain ? drain : 32u;
    if ((nb != 8 && nb != 16 && nb != 32) || bt > kBatch || dr > 32) {
        tgx_set_error("tgx_set_vis_tuning: depth buckets %u (8, 16 or 32), batch %u (1..%u), drain %u (1..32)", nb, bt,
                      kBatch, dr);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    c->vis_bshift = nb == 32 ? 0u : nb == 16 ? 1u : 2u;
    c->vis_batch = bt;
    c->vis_drain = dr;
    return TGX_OK;
}

extern "C" tgx_status tgx_vis_count_work(tgx_ctx* c, int enable)
{
    if (!c) return TGX_ERR_INVALID_ARGUMENT;
    c->vis_count_work = enable != 0;
    return TGX_OK;
}

extern "C" tgx_status tgx_vis_get_work(tgx_ctx* c, tgx_vis_work* out)
{
    if (!c || !out) return TGX_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    if (!c->vis_work.ptr) return TGX_OK;
    static_assert(sizeof(tgx_vis_work) == W_COUNT * sizeof(uint64_t), "tgx_vis_work layout");
    TGX_CUDA(cudaMemcpyAsync(out, c->vis_work.ptr, sizeof(*out), cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

// ---------------------------------------------------------------------------
// Visibility render without any allocation (tgx_vis_render_noalloc).
//
// For callers that cannot allocate device memory at all: code running under an
// allocator they do not own (a host application with a fixed memory budget, or
// a plugin whose host forbids cudaMalloc), or code that must not trigger the
// implicit device synchronisation a cudaMalloc/cudaFree can cause.  All the
// scratch of the pass lives in one file-scope device array of fixed size,
// created when the library is loaded on a device and kept until the process
// exits.  The caller passes the scene arrays and the output buffer, both in
// device memory.
// ---------------------------------------------------------------------------

namespace {

constexpr uint32_t kNaMaxObjects = 65536;
constexpr uint32_t kNaMaxClusterPointers = 1u << 19;
constexpr uint32_t kNaMaxTiles = 32768;      // 16x16 tiles: up to 3840x2160
constexpr uint32_t kNaBins = 1u << 18;       // (tile, cluster) entries; more take the exact record-scan path
constexpr uint32_t kNaTile = 16;

constexpr size_t na_align(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kNaCounters = 0;
constexpr size_t kNaStatus = kNaCounters + 256;
constexpr size_t kNaViews = kNaStatus + 256;
constexpr size_t kNaInvRot = kNaViews + na_align(sizeof(ViewConst) + 16);
constexpr size_t kNaRecords = kNaInvRot + na_align((size_t)kNaMaxObjects * 9 * 4);
constexpr size_t kNaRects = kNaRecords + na_align((size_t)kNaMaxClusterPointers * sizeof(VisRecord));
constexpr size_t kNaBucketCnt = kNaRects + na_align((size_t)kNaMaxClusterPointers * 8);
constexpr uint32_t kNaBuckets = 16;          // depth buckets per tile (bucket shift 1)
constexpr size_t kNaBucketOff = kNaBucketCnt + na_align((size_t)kNaMaxTiles * kNaBuckets * 4);
constexpr size_t kNaTileTotal = kNaBucketOff + na_align((size_t)kNaMaxTiles * kNaBuckets * 4);
constexpr size_t kNaScanAux = kNaTileTotal + na_align((size_t)kNaMaxTiles * 4);
constexpr size_t kNaTileOff = kNaScanAux + na_align(((size_t)kNaMaxTiles / kScanTiles + 1) * (1 + kOrderClasses) * 4);
constexpr size_t kNaSlotInfo = kNaTileOff + na_align(((size_t)kNaMaxTiles + 4) * 4);
constexpr size_t kNaBinsOff = kNaSlotInfo + na_align((size_t)kNaMaxTiles * 16);
constexpr size_t kNaBytes = kNaBinsOff + na_align((size_t)kNaBins * sizeof(TileEntry));   // about 51 MiB

// The scratch.  In host code this name is only a host-side stand-in: its
// device address is taken with cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_vis_noalloc_scratch[kNaBytes];

// The call's set-up on the device, so that no host buffer is read after the
// call returns: the first CTA writes the view constants and the output
// pointer (both passed by value) and zeroes the counters and the status
// word; every thread writes one object's 3x3 of inverse(rotation), as
// k_object_setup computes it at upload.
__global__ void __launch_bounds__(128) k_vis_noalloc_setup(ViewConst vc, unsigned long long* visbuf,
                                                          ViewConst* __restrict__ d_vc,
                                                          unsigned long long** __restrict__ d_outs,
                                                          uint32_t* __restrict__ counters,
                                                          tgx_dev_status* __restrict__ status,
                                                          const tgx_object* __restrict__ objs, uint32_t n,
                                                          float* __restrict__ inv_rot)
{
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0) {
            *d_vc = vc;
            *d_outs = visbuf;
            status->code = 0u;
            status->where = 0u;
            status->detail = 0ull;
        }
        if (threadIdx.x < 64) counters[threadIdx.x] = 0u;
    }
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float rot[16], inv[16];
#pragma unroll
    for (int k = 0; k < 16; k++) rot[k] = objs[i].rotation[k];
    dm4_inverse(rot, inv);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) inv_rot[9 * i + 3 * r + c] = DM(inv, r, c);
}

constexpr int kNaMaxDevices = 64;
std::mutex g_na_mutex;
void* g_na_ptr[kNaMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per device.
tgx_status na_scratch(int device, unsigned char** out)
{
    if (device < 0 || device >= kNaMaxDevices) {
        tgx_set_error("tgx_vis_render_noalloc: device %d out of range", device);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_vis_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            tgx_set_error("tgx_vis_render_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return TGX_ERR_CUDA;
        }
        g_na_ptr[device] = p;
    }
    *out = (unsigned char*)g_na_ptr[device];
    return TGX_OK;
}

#define NA_LAUNCH(grid, block, kernel, ...)                                                        \
    do {                                                                                           \
        kernel<<<(grid), (block), 0, st>>>(__VA_ARGS__);                                           \
        const cudaError_t le_ = cudaGetLastError();                                                \
        if (le_ != cudaSuccess) {                                                                  \
            tgx_set_error("tgx_vis_render_noalloc: launch of %s failed: %s", #kernel,              \
                          cudaGetErrorString(le_));                                                \
            return TGX_ERR_CUDA;                                                                   \
        }                                                                                          \
    } while (0)

}  // namespace

extern "C" tgx_status tgx_vis_render_noalloc(void* stream, const tgx_object* d_objects, uint32_t n_objects,
                                             const uint32_t* d_cluster_pointers, uint32_t n_cluster_pointers,
                                             const uint32_t* d_cluster_idx_to_object_idx,
                                             const uint32_t* d_voxel_bits, const tgx_view* view, uint64_t* d_visbuf,
                                             tgx_device_error* out_error)
{
    if (!d_objects || !d_cluster_pointers || !d_cluster_idx_to_object_idx || !d_voxel_bits || !view || !d_visbuf) {
        tgx_set_error("tgx_vis_render_noalloc: NULL argument");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (n_objects == 0 || n_objects > kNaMaxObjects) {
        tgx_set_error("tgx_vis_render_noalloc: %u objects, the fixed scratch holds 1..%u", n_objects, kNaMaxObjects);
        return TGX_ERR_CAPACITY;
    }
    if (n_cluster_pointers == 0 || n_cluster_pointers > kNaMaxClusterPointers) {
        tgx_set_error("tgx_vis_render_noalloc: %u cluster pointers, the fixed scratch holds 1..%u", n_cluster_pointers,
                      kNaMaxClusterPointers);
        return TGX_ERR_CAPACITY;
    }
    TGX_TRY(check_views(view, 1, kNaTile, kNaTile));
    ViewConst vc;
    make_view_const(*view, kNaTile, kNaTile, 0, vc);
    const uint32_t n_tiles = vc.tiles_x * vc.tiles_y;
    if (n_tiles > kNaMaxTiles) {
        tgx_set_error("tgx_vis_render_noalloc: %ux%u needs %u tiles of 16x16, the fixed scratch holds %u", view->width,
                      view->height, n_tiles, kNaMaxTiles);
        return TGX_ERR_CAPACITY;
    }
    int device = 0;
    TGX_CUDA(cudaGetDevice(&device));
    unsigned char* base = nullptr;
    TGX_TRY(na_scratch(device, &base));
    cudaStream_t st = (cudaStream_t)stream;

    uint32_t* counters = (uint32_t*)(base + kNaCounters);
    tgx_dev_status* status = (tgx_dev_status*)(base + kNaStatus);
    ViewConst* d_vc = (ViewConst*)(base + kNaViews);
    unsigned long long** d_outs = (unsigned long long**)(base + kNaViews + ((sizeof(ViewConst) + 15) & ~(size_t)15));
    float* inv_rot = (float*)(base + kNaInvRot);
    VisRecord* records = (VisRecord*)(base + kNaRecords);
    uint2* rects = (uint2*)(base + kNaRects);
    uint32_t* bucket_cnt = (uint32_t*)(base + kNaBucketCnt);
    uint32_t* bucket_off = (uint32_t*)(base + kNaBucketOff);
    uint32_t* tile_total = (uint32_t*)(base + kNaTileTotal);
    uint32_t* cta_aux = (uint32_t*)(base + kNaScanAux);
    uint32_t* tile_off = (uint32_t*)(base + kNaTileOff);
    uint4* slot_info = (uint4*)(base + kNaSlotInfo);
    TileEntry* entries = (TileEntry*)(base + kNaBinsOff);

    int sms = 0;
    TGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const uint32_t warp_grid = (uint32_t)sms * 8;
    // what must start at zero (counters, status) is cleared by the set-up kernel;
    // everything else is written before it is read
    NA_LAUNCH((n_objects + 127) / 128, 128, k_vis_noalloc_setup, vc, (unsigned long long*)d_visbuf, d_vc, d_outs,
              counters, status, d_objects, n_objects, inv_rot);
    NA_LAUNCH((n_cluster_pointers + 255) / 256, 256, k_vis_cluster_setup<false>, d_objects, d_cluster_pointers,
              d_cluster_idx_to_object_idx, d_voxel_bits, (const uint32_t*)nullptr, n_cluster_pointers, d_vc, 1u,
              records, rects, kNaMaxClusterPointers, counters, bucket_cnt, n_tiles * kNaBuckets, status);
    NA_LAUNCH(warp_grid, 256, k_vis_count, records, rects, counters, kNaMaxClusterPointers, d_objects, d_vc, bucket_cnt,
              n_tiles, 1u);
    const uint32_t n_scan_ctas = (n_tiles + kScanTiles - 1) / kScanTiles;
    NA_LAUNCH(n_scan_ctas, kScanTiles, k_vis_prefix<kNaBuckets>, bucket_cnt, bucket_off, tile_total, n_tiles, cta_aux);
    if (n_scan_ctas <= kDirectGroups) {
        NA_LAUNCH(n_scan_ctas, kScanTiles, k_vis_finalize_direct, tile_total, n_tiles, cta_aux, tile_off, slot_info,
                  kNaBins, counters);
    } else {
        NA_LAUNCH(1, 1024, k_vis_scan, cta_aux, n_tiles, tile_off, kNaBins, counters);
        NA_LAUNCH(n_scan_ctas, kScanTiles, k_vis_finalize, tile_total, n_tiles, cta_aux, tile_off, slot_info);
    }
    NA_LAUNCH(warp_grid, 256, k_vis_bin_fill, records, rects, counters, d_vc, tile_off, bucket_off, bucket_cnt, entries,
              d_voxel_bits, n_tiles, kNaBins, 1u, status);
    TileJob J;
    J.records = records;
    J.rects = rects;
    J.entries = entries;
    J.tile_off = tile_off;
    J.slot_info = slot_info;
    J.views = d_vc;
    J.bits = d_voxel_bits;
    J.inv_rot = inv_rot;
    J.outs = d_outs;
    J.counters = counters;
    J.n_views = 1;
    J.n_tiles = n_tiles;
    J.first = 0;
    J.work = nullptr;
    J.extra_tx = 0;
    J.interleave = 0;
    J.bshift = 1;
    J.batch = kBatch;
    J.drain = 32;
    k_vis_tiles<256, 5><<<n_tiles, kNaTile * kNaTile, tile_smem_bytes(kNaTile * kNaTile), st>>>(J, status);
    if (const cudaError_t le = cudaGetLastError(); le != cudaSuccess) {
        tgx_set_error("tgx_vis_render_noalloc: launch of k_vis_tiles failed: %s", cudaGetErrorString(le));
        return TGX_ERR_CUDA;
    }
    if (out_error) {
        tgx_dev_status hs;
        TGX_CUDA(cudaMemcpyAsync(&hs, status, sizeof(hs), cudaMemcpyDeviceToHost, st));
        TGX_CUDA(cudaStreamSynchronize(st));
        out_error->code = hs.code;
        out_error->where = hs.where;
        out_error->detail = hs.detail;
        if (hs.code) return (tgx_status)hs.code;
    }
    return TGX_OK;
}
#undef NA_LAUNCH
