// svo.cu -- one-bit SVO build on the GPU.
//
// Replaces tg's recursive single-threaded CPU builder tg_svo_create
// (tg_sparse_voxel_octree.c:466-542) with four data-parallel passes that set
// exactly the same world voxels:
//
//   1. k_svo_candidates  one thread per cluster pointer: drops empty clusters
//      (:515-531), finds the 32^3 blocks its box can touch, and for each runs
//      the reference's OBB/AABB test (tg_physics.c:226-392) on every node on
//      the path from the root's children down to the block, with the node
//      boxes and ws2ms matrix of tg__construct_inner_node (:319-397).  A block
//      whose whole path passes becomes a (cluster, block) pair; the block is
//      marked in the dense block table.
//   2. k_svo_alloc       gives every marked block a slot in the block pool.
//   3. k_svo_voxelize    the pairs grouped by block (count, scan, place),
//      then one CTA per block, one warp per pair: the leaf voxelisation of
//      tg__construct_leaf_node (:102-317) -- corner lerp, [0,8)^3 test, bit
//      fetch -- into the block's image (and material grid) in shared
//      memory, written out whole and coalesced, with no global atomics.
//   4. k_svo_pyramid     bottom-up occupancy: one bit per non-empty block and
//      per non-empty node of every coarser level, and inside each block one
//      bit per non-empty 4^3 and 8^3 cell (the sub-block levels the
//      traversal steps through before single voxels).
//
// The node encoding of the reference (u16 relative child pointers, 64-entry
// leaf lists) is not kept; the voxel set is.  Side length 2^6 .. 2^14.

#include "svo_trace.cuh"

#include <algorithm>
#include <vector>



namespace {

constexpr uint32_t kBlockSide = 32;
constexpr uint32_t kBlockWords = 1024;
constexpr uint32_t kMark = 0xffffffffu;
constexpr uint32_t kWarpsPerVoxCta = 16;

struct SvoPair
{
    uint32_t cluster_pointer;
    uint32_t block;
};

enum SvoCounter { S_PAIRS = 0, S_MARKED = 1, S_SLOTS = 2, S_NONEMPTY = 3, S_FREED = 4, S_MOVED = 5, S_COUNT = 8 };

struct dv3 { float x, y, z; };

__device__ __forceinline__ void cluster_offsets(const tgx_object& od, uint32_t rel, float off[3], float ohe[3])
{
    const uint32_t nx = od.n_cluster_pointers_per_dim[0], ny = od.n_cluster_pointers_per_dim[1];
    off[0] = (float)((rel % nx) * 8u);
    off[1] = (float)(((rel / nx) % ny) * 8u);
    off[2] = (float)((rel / (nx * ny)) * 8u);
    const float h = 4.0f;   // (f32)(TG_N_PRIMITIVES_PER_CLUSTER_CUBE_ROOT / 2)
    ohe[0] = xmul((float)od.n_cluster_pointers_per_dim[0], h);
    ohe[1] = xmul((float)od.n_cluster_pointers_per_dim[1], h);
    ohe[2] = xmul((float)od.n_cluster_pointers_per_dim[2], h);
}

// tg_world_space_to_cluster_model_space (tg_sparse_voxel_octree.c:23-60)
__device__ __forceinline__ void svo_ws2ms(const tgx_object& od, uint32_t rel, float* out)
{
    float off[3], ohe[3], rot[16], m1[16], m2[16], m3[16], m4[16];
    cluster_offsets(od, rel, off, ohe);
#pragma unroll
    for (int k = 0; k < 16; k++) rot[k] = od.rotation[k];
    dm4_translate(-od.translation[0], -od.translation[1], -od.translation[2], m1);
    dm4_inverse(rot, m2);
    dm4_translate(ohe[0], ohe[1], ohe[2], m3);
    dm4_translate(-off[0], -off[1], -off[2], m4);
    dm4_mul(m4, m3, out);
    dm4_mul(out, m2, out);
    dm4_mul(out, m1, out);
}

// tg_cluster_model_space_to_world_space (tg_sparse_voxel_octree.c:62-100)
__device__ __forceinline__ void svo_cs2ws(const tgx_object& od, uint32_t rel, float* out)
{
    float off[3], ohe[3], rot[16], m1[16], m2[16], m4[16];
    cluster_offsets(od, rel, off, ohe);
#pragma unroll
    for (int k = 0; k < 16; k++) rot[k] = od.rotation[k];
    dm4_translate(off[0], off[1], off[2], m1);
    dm4_translate(-ohe[0], -ohe[1], -ohe[2], m2);
    dm4_translate(od.translation[0], od.translation[1], od.translation[2], m4);
    dm4_mul(m4, rot, out);
    dm4_mul(out, m2, out);
    dm4_mul(out, m1, out);
}

__device__ __forceinline__ dv3 mulv4p(const float* m, float x, float y, float z)
{
    float r[3];
    dm4_mulv4(m, x, y, z, 1.0f, r);
    return dv3{r[0], r[1], r[2]};
}

__device__ __forceinline__ float dot3(dv3 a, dv3 b) { return xadd(xadd(xmul(a.x, b.x), xmul(a.y, b.y)), xmul(a.z, b.z)); }
__device__ __forceinline__ float mag3(dv3 a) { return xsqrt(dot3(a, a)); }
__device__ __forceinline__ dv3 sub3(dv3 a, dv3 b) { return dv3{xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)}; }
__device__ __forceinline__ dv3 normalized3(dv3 a)
{
    const float m = mag3(a);
    return dv3{xdiv(a.x, m), xdiv(a.y, m), xdiv(a.z, m)};
}

// tg_intersect_aabb_obb_ignore_contact (tg_physics.c:226-392) with the AABB
// [0,8]^3 (the cluster) and the OBB given by its 8 corners (a block).
__device__ __forceinline__ bool aabb_obb(const dv3* c)
{
    const float mx = 8.0f;
    bool sep;
    sep = true;
#pragma unroll
    for (int i = 0; i < 8; i++) sep &= c[i].x <= 0.0f;
    if (sep) return false;
    sep = true;
#pragma unroll
    for (int i = 0; i < 8; i++) sep &= c[i].x >= mx;
    if (sep) return false;
    sep = true;
#pragma unroll
    for (int i = 0; i < 8; i++) sep &= c[i].y <= 0.0f;
    if (sep) return false;
    sep = true;
#pragma unroll
    for (int i = 0; i < 8; i++) sep &= c[i].y >= mx;
    if (sep) return false;
    sep = true;
#pragma unroll
    for (int i = 0; i < 8; i++) sep &= c[i].z <= 0.0f;
    if (sep) return false;
    sep = true;
#pragma unroll
    for (int i = 0; i < 8; i++) sep &= c[i].z >= mx;
    if (sep) return false;

    const dv3 nxp = normalized3(sub3(c[1], c[0]));
    const dv3 nyp = normalized3(sub3(c[2], c[0]));
    const dv3 nzp = normalized3(sub3(c[4], c[0]));
    const dv3 nrm[6] = {dv3{-nxp.x, -nxp.y, -nxp.z}, nxp, dv3{-nyp.x, -nyp.y, -nyp.z}, nyp,
                        dv3{-nzp.x, -nzp.y, -nzp.z}, nzp};
    const float l0 = mag3(c[0]);
    const float l1 = mag3(c[7]);
    const dv3 n0 = l0 == 0.0f ? dv3{0.0f, 0.0f, 0.0f} : dv3{xdiv(c[0].x, l0), xdiv(c[0].y, l0), xdiv(c[0].z, l0)};
    const dv3 n1 = l1 == 0.0f ? dv3{0.0f, 0.0f, 0.0f} : dv3{xdiv(c[7].x, l1), xdiv(c[7].y, l1), xdiv(c[7].z, l1)};
    float dist[6];
    dist[0] = xmul(l0, dot3(n0, nrm[0]));
    dist[1] = xmul(l1, dot3(n1, nrm[1]));
    dist[2] = xmul(l0, dot3(n0, nrm[2]));
    dist[3] = xmul(l1, dot3(n1, nrm[3]));
    dist[4] = xmul(l0, dot3(n0, nrm[4]));
    dist[5] = xmul(l1, dot3(n1, nrm[5]));
#pragma unroll
    for (int p = 0; p < 6; p++) {
        sep = true;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const dv3 pt = dv3{(k & 1) ? mx : 0.0f, (k & 2) ? mx : 0.0f, (k & 4) ? mx : 0.0f};
            sep &= xsub(dot3(nrm[p], pt), dist[p]) >= 0.0f;
        }
        if (sep) return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// 1. candidates
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(128) k_svo_candidates(
    const tgx_object* __restrict__ objects, const uint32_t* __restrict__ cluster_pointers,
    const uint32_t* __restrict__ c2o, const uint32_t* __restrict__ bits, uint32_t n_cp, float mnx, float mny,
    float mnz, uint32_t L, uint32_t B, uint32_t* __restrict__ table, SvoPair* __restrict__ pairs,
    uint32_t pair_capacity, uint32_t* __restrict__ counters, tgx_dev_status* __restrict__ status,
    const uint8_t* __restrict__ dirty /* null: every block; else only blocks marked dirty */)
{
    const uint32_t cp = blockIdx.x * blockDim.x + threadIdx.x;
    if (cp >= n_cp) return;
    const uint32_t ci = cluster_pointers[cp];
    const uint4* w = reinterpret_cast<const uint4*>(bits + (uint64_t)ci * 16u);
    const uint4 a = w[0], b = w[1], c = w[2], d = w[3];
    if (!(a.x | a.y | a.z | a.w | b.x | b.y | b.z | b.w | c.x | c.y | c.z | c.w | d.x | d.y | d.z | d.w)) return;
    const tgx_object& od = objects[c2o[ci]];
    const uint32_t rel = cp - od.first_cluster_pointer;

    // conservative world box of the cluster (only selects blocks to test)
    float off[3], ohe[3];
    cluster_offsets(od, rel, off, ohe);
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float lx = off[0] + ((k & 1) ? 8.0f : 0.0f) - ohe[0];
        const float ly = off[1] + ((k & 2) ? 8.0f : 0.0f) - ohe[1];
        const float lz = off[2] + ((k & 4) ? 8.0f : 0.0f) - ohe[2];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const float p = DM(od.rotation, r, 0) * lx + DM(od.rotation, r, 1) * ly + DM(od.rotation, r, 2) * lz +
                            od.translation[r];
            lo[r] = fminf(lo[r], p);
            hi[r] = fmaxf(hi[r], p);
        }
    }
    const float mn[3] = {mnx, mny, mnz};
    int b0[3], b1[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        const float slack = 0.5f + 1e-5f * fabsf(lo[r]) + 1e-5f * fabsf(hi[r]);
        b0[r] = (int)floorf((lo[r] - slack - mn[r]) / 32.0f);
        b1[r] = (int)floorf((hi[r] + slack - mn[r]) / 32.0f);
        b0[r] = max(b0[r], 0);
        b1[r] = min(b1[r], (int)B - 1);
        if (b0[r] > b1[r]) return;
    }
    float ws2ms[16];
    svo_ws2ms(od, rel, ws2ms);
    const float ext = (float)(1u << L);
    for (int bz = b0[2]; bz <= b1[2]; bz++)
        for (int by = b0[1]; by <= b1[1]; by++)
            for (int bx = b0[0]; bx <= b1[0]; bx++) {
                if (dirty && !dirty[((uint32_t)bz * B + (uint32_t)by) * B + (uint32_t)bx]) continue;
                // walk the reference's recursion from the root to this block
                dv3 pmin = dv3{mnx, mny, mnz};
                dv3 pmax = dv3{xadd(mnx, ext), xadd(mny, ext), xadd(mnz, ext)};
                bool pass = true;
                for (int lev = (int)L - 1; lev >= 5; lev--) {
                    const dv3 ce = dv3{xmul(xsub(pmax.x, pmin.x), 0.5f), xmul(xsub(pmax.y, pmin.y), 0.5f),
                                       xmul(xsub(pmax.z, pmin.z), 0.5f)};
                    const uint32_t sh = (uint32_t)lev - 5;
                    const uint32_t cx = ((uint32_t)bx >> sh) & 1u, cy = ((uint32_t)by >> sh) & 1u,
                                   cz = ((uint32_t)bz >> sh) & 1u;
                    const dv3 cmin = dv3{xadd(pmin.x, xmul((float)cx, ce.x)), xadd(pmin.y, xmul((float)cy, ce.y)),
                                         xadd(pmin.z, xmul((float)cz, ce.z))};
                    const dv3 cmax = dv3{xadd(cmin.x, ce.x), xadd(cmin.y, ce.y), xadd(cmin.z, ce.z)};
                    dv3 bc[8];
#pragma unroll
                    for (int k = 0; k < 8; k++)
                        bc[k] = mulv4p(ws2ms, (k & 1) ? cmax.x : cmin.x, (k & 2) ? cmax.y : cmin.y,
                                       (k & 4) ? cmax.z : cmin.z);
                    if (!aabb_obb(bc)) { pass = false; break; }
                    pmin = cmin;
                    pmax = cmax;
                }
                if (!pass) continue;
                const uint32_t blk = ((uint32_t)bz * B + (uint32_t)by) * B + (uint32_t)bx;
                const uint32_t slot = atomicAdd(&counters[S_PAIRS], 1u);
                if (slot < pair_capacity) pairs[slot] = SvoPair{cp, blk};
                else dev_error(status, TGX_ERR_CAPACITY, 11, slot);
                if (atomicCAS(&table[blk], 0u, kMark) == 0u) atomicAdd(&counters[S_MARKED], 1u);
            }
}

// ---------------------------------------------------------------------------
// 2. slot allocation
// ---------------------------------------------------------------------------

// Marked blocks take slots from the end of the free list first (free[n_free-1],
// free[n_free-2], ...), then fresh slots from `next_slot` on.
__global__ void __launch_bounds__(256) k_svo_alloc(uint32_t* __restrict__ table, uint64_t n_table,
                                                  uint32_t* __restrict__ counters, const uint32_t* __restrict__ free_list,
                                                  uint32_t n_free, uint32_t next_slot, uint32_t pool_blocks,
                                                  tgx_dev_status* __restrict__ status)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_table;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (table[i] == kMark) {
            const uint32_t s = atomicAdd(&counters[S_SLOTS], 1u);
            const uint32_t slot = s < n_free ? free_list[n_free - 1u - s] : next_slot + (s - n_free);
            if (slot < pool_blocks) table[i] = slot + 1u;
            else { table[i] = 0u; dev_error(status, TGX_ERR_CAPACITY, 12, s); }
        }
    }
}

// ---------------------------------------------------------------------------
// 3. voxelisation: one warp per (cluster, block) pair
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t trim_u32(float v) { return v > 0.0f ? (uint32_t)v : 0u; }

// max of a 16-bit code in place in shared memory (CAS on the containing word)
__device__ __forceinline__ void smem_max_u16(uint32_t* words, uint32_t idx, uint32_t val)
{
    uint32_t* base = words + (idx >> 1);
    const uint32_t shift = (idx & 1u) ? 16u : 0u;
    uint32_t old = *base;
    for (int guard = 0; guard < 1 << 20; guard++) {
        if (((old >> shift) & 0xffffu) >= val) return;
        const uint32_t nv = (old & ~(0xffffu << shift)) | (val << shift);
        const uint32_t prev = atomicCAS(base, old, nv);
        if (prev == old) return;
        old = prev;
    }
}

// 3a. pairs grouped by their block's slot: counts, one scan, placement
__global__ void __launch_bounds__(256) k_svo_pair_count(const SvoPair* __restrict__ pairs,
                                                       const uint32_t* __restrict__ counters, uint32_t pair_capacity,
                                                       const uint32_t* __restrict__ table, uint32_t* __restrict__ cnt)
{
    const uint32_t n = min(counters[S_PAIRS], pair_capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t tv = table[pairs[i].block];
        if (tv) atomicAdd(&cnt[tv - 1u], 1u);
    }
}

// exclusive scan of cnt[0, n) into off[0, n] (off[n] = total): one CTA, each
// thread a contiguous run
__global__ void __launch_bounds__(1024) k_svo_pair_scan(const uint32_t* __restrict__ cnt, uint32_t n,
                                                       uint32_t* __restrict__ off)
{
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x, per = (n + 1023u) / 1024u;
    const uint32_t b = min(n, t * per), e = min(n, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; i++) sum += cnt[i];
    part[t] = sum;
    __syncthreads();
    for (uint32_t o = 1; o < 1024u; o <<= 1) {
        const uint32_t v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = t ? part[t - 1u] : 0u;
    for (uint32_t i = b; i < e; i++) {
        off[i] = run;
        run += cnt[i];
    }
    if (t == 1023u) off[n] = part[1023];
}

__global__ void __launch_bounds__(256) k_svo_pair_fill(const SvoPair* __restrict__ pairs,
                                                      const uint32_t* __restrict__ counters, uint32_t pair_capacity,
                                                      const uint32_t* __restrict__ table, const uint32_t* __restrict__ off,
                                                      uint32_t* __restrict__ cursor, SvoPair* __restrict__ sorted)
{
    const uint32_t n = min(counters[S_PAIRS], pair_capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const SvoPair pr = pairs[i];
        const uint32_t tv = table[pr.block];
        if (tv) sorted[off[tv - 1u] + atomicAdd(&cursor[tv - 1u], 1u)] = pr;
    }
}

// 3b. voxelisation: one CTA per block slot.  Its warps take the block's
// (cluster, block) pairs; every set voxel goes into the CTA's shared image of
// the block (and the material codes' maximum into its shared material grid),
// then the block is written out whole, coalesced, with no global atomics.
// A pair's cluster-space transform and its voxel range in the block: the
// trimmed range of tg__construct_leaf_node (tg_sparse_voxel_octree.c:180-226).
struct PairBox
{
    dv3 pmin, pext;
    float cs2ws[16];
    uint32_t x0, y0, z0, x1, y1, z1;
    uint32_t ci, rel;
    const tgx_object* od;
};

__device__ __forceinline__ void pair_box(const tgx_object* __restrict__ objects,
                                         const uint32_t* __restrict__ cluster_pointers,
                                         const uint32_t* __restrict__ c2o, const SvoPair& pr, float mnx, float mny,
                                         float mnz, uint32_t B, PairBox& pb)
{
    const uint32_t cp = pr.cluster_pointer;
    pb.ci = cluster_pointers[cp];
    pb.od = &objects[c2o[pb.ci]];
    pb.rel = cp - pb.od->first_cluster_pointer;
    const uint32_t bx = pr.block % B, by = (pr.block / B) % B, bz = pr.block / (B * B);
    // block box: same values the recursion produces (exact powers of two)
    pb.pmin = dv3{xadd(mnx, (float)(bx * kBlockSide)), xadd(mny, (float)(by * kBlockSide)),
                  xadd(mnz, (float)(bz * kBlockSide))};
    const dv3 pmax = dv3{xadd(pb.pmin.x, 32.0f), xadd(pb.pmin.y, 32.0f), xadd(pb.pmin.z, 32.0f)};
    pb.pext = sub3(pmax, pb.pmin);
    svo_cs2ws(*pb.od, pb.rel, pb.cs2ws);
    dv3 cw[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
        cw[k] = mulv4p(pb.cs2ws, (k & 1) ? 8.0f : 0.0f, (k & 2) ? 8.0f : 0.0f, (k & 4) ? 8.0f : 0.0f);
    // :180-194 -- note corner 2 twice, corner 3 never
    auto vmin = [](dv3 p, dv3 q) { return dv3{p.x < q.x ? p.x : q.x, p.y < q.y ? p.y : q.y, p.z < q.z ? p.z : q.z}; };
    auto vmax = [](dv3 p, dv3 q) { return dv3{p.x > q.x ? p.x : q.x, p.y > q.y ? p.y : q.y, p.z > q.z ? p.z : q.z}; };
    const dv3 min_c = vmin(vmin(vmin(cw[0], cw[1]), vmin(cw[2], cw[2])), vmin(vmin(cw[4], cw[6]), vmin(cw[5], cw[7])));
    const dv3 max_c = vmax(vmax(vmax(cw[0], cw[1]), vmax(cw[2], cw[2])), vmax(vmax(cw[4], cw[6]), vmax(cw[5], cw[7])));
    const dv3 fmin_c = dv3{floorf(min_c.x), floorf(min_c.y), floorf(min_c.z)};
    const dv3 cmax_c = dv3{ceilf(max_c.x), ceilf(max_c.y), ceilf(max_c.z)};
    const dv3 tmin = vmax(pb.pmin, fmin_c);
    const dv3 tmax = vmin(pmax, cmax_c);
    pb.x0 = trim_u32(xsub(tmin.x, pb.pmin.x)); pb.y0 = trim_u32(xsub(tmin.y, pb.pmin.y)); pb.z0 = trim_u32(xsub(tmin.z, pb.pmin.z));
    pb.x1 = trim_u32(xsub(tmax.x, pb.pmin.x)); pb.y1 = trim_u32(xsub(tmax.y, pb.pmin.y)); pb.z1 = trim_u32(xsub(tmax.z, pb.pmin.z));
}

__device__ __forceinline__ uint32_t pair_voxels(const PairBox& b)
{
    return (b.x0 >= b.x1 || b.y0 >= b.y1 || b.z0 >= b.z1) ? 0u : (b.x1 - b.x0) * (b.y1 - b.y0) * (b.z1 - b.z0);
}

// One CTA per block slot.  The block's pairs are taken 32 at a time: their
// trimmed voxel counts are measured first (a lane per pair) and sorted by a
// warp bitonic sort, heaviest first; the warps then take pairs in that order
// from a shared counter, the next one whenever they finish one, so the CTA's
// final barrier waits little.  Within a pair, a lane takes a row (iy, iz) of
// the trimmed box: the reference's z- and y-lerps once per row, the x-lerp,
// the [0, 8)^3 test and the bit fetch per voxel, the cluster's bit words and
// material bytes from shared memory.  The block image and the material codes
// are merged with atomicOr / a 16-bit max in shared memory, so the order of
// the pairs changes no bit.
template <bool kMat>
__global__ void __launch_bounds__(32 * kWarpsPerVoxCta) k_svo_voxelize(
    const tgx_object* __restrict__ objects, const uint32_t* __restrict__ cluster_pointers,
    const uint32_t* __restrict__ c2o, const uint32_t* __restrict__ bits, const SvoPair* __restrict__ sorted,
    const uint32_t* __restrict__ off, uint32_t* __restrict__ pool, const uint8_t* __restrict__ material,
    uint16_t* __restrict__ mat_pool, float mnx, float mny, float mnz, uint32_t B)
{
    constexpr uint32_t kOrderCap = 32 * kWarpsPerVoxCta * 2;   // pairs ordered per round
    extern __shared__ __align__(16) uint32_t s_blk[];   // 1024 bit words, then 16384 words of u16 codes
    __shared__ uint32_t s_cw[kWarpsPerVoxCta][16];       // each warp's current cluster bits
    __shared__ uint4 s_cm[kMat ? kWarpsPerVoxCta : 1][32];  // and its 512 material bytes
    __shared__ uint16_t s_order[kOrderCap];              // per chunk of 32: pair offsets, heaviest first
    __shared__ uint32_t s_next;                          // the next entry of s_order to take
    uint32_t* img = s_blk;
    uint32_t* smat = s_blk + kBlockWords;
    const uint32_t slot = blockIdx.x;
    const uint32_t pb = off[slot], pe = off[slot + 1];
    if (pb == pe) return;
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t words = kBlockWords + (kMat ? 16384u : 0u);
    for (uint32_t k = threadIdx.x; k < words / 4u; k += blockDim.x)
        reinterpret_cast<uint4*>(s_blk)[k] = make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t r0 = pb; r0 < pe; r0 += kOrderCap) {
        const uint32_t np = min(kOrderCap, pe - r0);
        const uint32_t n_chunks = (np + 31u) / 32u;
        __syncthreads();   // the previous round's order is consumed (and the image is cleared)
        for (uint32_t ch = wid; ch < n_chunks; ch += kWarpsPerVoxCta) {
            const uint32_t i = ch * 32u + lane;
            // key: voxel count (pairs past the end sort last); value: pair offset in the round
            int32_t key = -1;
            uint32_t idx = i;
            if (i < np) {
                PairBox bx;
                pair_box(objects, cluster_pointers, c2o, sorted[r0 + i], mnx, mny, mnz, B, bx);
                key = (int32_t)pair_voxels(bx);
            }
            // ascending bitonic sort over the warp's 32 lanes
#pragma unroll
            for (uint32_t k = 2; k <= 32; k <<= 1) {
#pragma unroll
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    const int32_t ok = __shfl_xor_sync(0xffffffffu, key, j);
                    const uint32_t oi = __shfl_xor_sync(0xffffffffu, idx, j);
                    const bool lower = (lane & j) == 0u, asc = (lane & k) == 0u;
                    const bool take = (asc == lower) ? (ok < key) : (ok > key);
                    if (take) { key = ok; idx = oi; }
                }
            }
            // descending rank 31 - lane
            s_order[ch * 32u + (31u - lane)] = (uint16_t)(key >= 0 ? idx : 0xffffu);
        }
        if (threadIdx.x == 0) s_next = 0u;
        __syncthreads();
        // warps take the round's pairs heaviest first (each chunk of 32 is sorted), the
        // next one whenever they finish one, so the block's warps end close together
        for (;;) {
            uint32_t item = 0;
            if (lane == 0) item = atomicAdd(&s_next, 1u);
            item = __shfl_sync(0xffffffffu, item, 0);
            if (item >= n_chunks * 32u) break;
            {
                const uint32_t k = s_order[item];
                if (k == 0xffffu) continue;
                PairBox bx;
                pair_box(objects, cluster_pointers, c2o, sorted[r0 + k], mnx, mny, mnz, B, bx);
                const uint32_t total = pair_voxels(bx);
                if (total == 0u) continue;
                const uint32_t x0 = bx.x0, y0 = bx.y0, z0 = bx.z0;
                const uint32_t nx = bx.x1 - x0, ny = bx.y1 - y0;
                const dv3 pext = bx.pext;
                const uint32_t ci = bx.ci;
                const uint32_t lut = bx.od->lut_idx;
                float ws2cs[16];
                dm4_inverse(bx.cs2ws, ws2cs);
                const dv3 pmax = dv3{xadd(bx.pmin.x, 32.0f), xadd(bx.pmin.y, 32.0f), xadd(bx.pmin.z, 32.0f)};
                dv3 bc[8];
#pragma unroll
                for (int q = 0; q < 8; q++)
                    bc[q] = mulv4p(ws2cs, (q & 1) ? pmax.x : bx.pmin.x, (q & 2) ? pmax.y : bx.pmin.y,
                                   (q & 4) ? pmax.z : bx.pmin.z);
                // the block side is exactly 32 unless min is so large that min + extent rounds
                const bool p32 = pext.x == 32.0f && pext.y == 32.0f && pext.z == 32.0f;
                // the cluster's 16 bit words, one shared-memory lookup per voxel
                __syncwarp();
                if (lane < 16) s_cw[wid][lane] = bits[(uint64_t)ci * 16u + lane];
                if (kMat) s_cm[wid][lane] = reinterpret_cast<const uint4*>(material + (uint64_t)ci * 512u)[lane];
                __syncwarp();
                // a lane per row (iy, iz) of the trim box: the z- and y-lerps of
                // tg__construct_leaf_node depend on the row only, so they are evaluated
                // once per row and the x-lerp per voxel; the same operations on the same
                // values as per voxel.  row -> (iy, iz) without integer division: row <
                // 2^10 and ny <= 32, so (row + 0.5) / ny lies at least 0.5 / ny from an
                // integer while the float product's error stays far below that
                const uint32_t nz = bx.z1 - z0, rows = ny * nz;
                const float rny = 1.0f / (float)ny;
                for (uint32_t row = lane; row < rows; row += 32) {
                    const uint32_t q = (uint32_t)(((float)row + 0.5f) * rny);
                    const uint32_t iy = y0 + (row - q * ny), iz = z0 + q;
                    // (i + 0.5) / 32 is an exact scaling: the reciprocal multiply gives the same bits
                    const float tz = p32 ? xmul(xadd((float)iz, 0.5f), 0.03125f) : xdiv(xadd((float)iz, 0.5f), pext.z);
                    const float omtz = xsub(1.0f, tz);
                    const float ty = p32 ? xmul(xadd((float)iy, 0.5f), 0.03125f) : xdiv(xadd((float)iy, 0.5f), pext.y);
                    const float omty = xsub(1.0f, ty);
#define LZ(i, j, comp) xadd(xmul(omtz, bc[i].comp), xmul(tz, bc[j].comp))
                    const float pz0x = LZ(0, 4, x), pz0y = LZ(0, 4, y), pz0z = LZ(0, 4, z);
                    const float pz1x = LZ(1, 5, x), pz1y = LZ(1, 5, y), pz1z = LZ(1, 5, z);
                    const float pz2x = LZ(2, 6, x), pz2y = LZ(2, 6, y), pz2z = LZ(2, 6, z);
                    const float pz3x = LZ(3, 7, x), pz3y = LZ(3, 7, y), pz3z = LZ(3, 7, z);
#undef LZ
                    const float py0x = xadd(xmul(omty, pz0x), xmul(ty, pz2x));
                    const float py0y = xadd(xmul(omty, pz0y), xmul(ty, pz2y));
                    const float py0z = xadd(xmul(omty, pz0z), xmul(ty, pz2z));
                    const float py1x = xadd(xmul(omty, pz1x), xmul(ty, pz3x));
                    const float py1y = xadd(xmul(omty, pz1y), xmul(ty, pz3y));
                    const float py1z = xadd(xmul(omty, pz1z), xmul(ty, pz3z));
                    // the row's first voxel index (an exact small-integer float expression)
                    const float row_base = xadd(xmul(xmul(pext.x, pext.y), (float)iz), xmul(pext.x, (float)iy));
                    // with a 32-voxel side, tx = (ix + 0.5) / 32 is a multiple of 2^-6 below 1, so
                    // adding 1/32 per voxel is exact: the same bits as the product
                    float tx32 = xmul(xadd((float)x0, 0.5f), 0.03125f);
                    for (uint32_t ix = x0; ix < x0 + nx; ix++, tx32 = xadd(tx32, 0.03125f)) {
                        const float tx = p32 ? tx32 : xdiv(xadd((float)ix, 0.5f), pext.x);
                        const float omtx = xsub(1.0f, tx);
                        const float cx = xadd(xmul(omtx, py0x), xmul(tx, py1x));
                        const float cy = xadd(xmul(omtx, py0y), xmul(tx, py1y));
                        const float cz = xadd(xmul(omtx, py0z), xmul(tx, py1z));
                        // one test for the three components (a NaN passes, as in the per-axis form)
                        if (cx < 0.0f || cx >= 8.0f || cy < 0.0f || cy >= 8.0f || cz < 0.0f || cz >= 8.0f) continue;
                        const uint32_t rvi = 64u * (uint32_t)cz + 8u * (uint32_t)cy + (uint32_t)cx;
                        const uint32_t word = s_cw[wid][rvi >> 5];
                        if (word & (1u << (rvi & 31u))) {
                            const uint32_t bvi = (uint32_t)xadd(row_base, (float)ix);
                            atomicOr(&img[bvi >> 5], 1u << (bvi & 31u));
                            if (kMat)
                                smem_max_u16(smat, bvi,
                                             ((lut << 8) | reinterpret_cast<const uint8_t*>(s_cm[wid])[rvi]) + 1u);
                        }
                    }
                }
            }
        }
    }
    __syncthreads();
    uint4* dst = reinterpret_cast<uint4*>(pool + (uint64_t)slot * kBlockWords);
    for (uint32_t k = threadIdx.x; k < kBlockWords / 4u; k += blockDim.x) dst[k] = reinterpret_cast<const uint4*>(img)[k];
    if (kMat) {
        uint4* md = reinterpret_cast<uint4*>(mat_pool + (uint64_t)slot * 32768u);
        for (uint32_t k = threadIdx.x; k < 16384u / 4u; k += blockDim.x) md[k] = reinterpret_cast<const uint4*>(smat)[k];
    }
}

// ---------------------------------------------------------------------------
// 4. occupancy pyramid
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_svo_pyramid(const uint32_t* __restrict__ table, uint64_t n_table,
                                                    const uint32_t* __restrict__ pool, uint32_t* __restrict__ nonempty,
                                                    uint32_t* __restrict__ sub, uint32_t* __restrict__ occ,
                                                    const uint64_t* __restrict__ occ_off, uint32_t n_levels, uint32_t B,
                                                    uint32_t* __restrict__ counters)
{
    // one warp per table entry; lane y reads the 32 rows (y, z) of the block
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = warp; i < n_table; i += n_warps) {
        const uint32_t tv = table[i];
        if (tv == 0u) continue;
        const uint32_t* blk = pool + (uint64_t)(tv - 1u) * kBlockWords;
        uint32_t any = 0;
        uint32_t n4[8];   // per 4-voxel z-slab: which 4-voxel x-groups of row y hold a voxel
#pragma unroll
        for (int k = 0; k < 8; k++) n4[k] = 0;
#pragma unroll
        for (int z = 0; z < 32; z++) {
            const uint32_t row = blk[z * 32 + lane];
            any |= row;
            uint32_t f = 0;
#pragma unroll
            for (int gx = 0; gx < 8; gx++) f |= ((row >> (4 * gx)) & 15u) ? (1u << gx) : 0u;
            n4[z >> 2] |= f;
        }
        any = __any_sync(0xffffffffu, any != 0u);
        if (lane == 0) nonempty[tv - 1u] = any ? 1u : 0u;
        if (!any) continue;
        // 4^3 cells: bit ((cz * 8 + cy) * 8 + cx), cy = lane / 4
        uint32_t* sb = sub + (uint64_t)(tv - 1u) * 32u;
#pragma unroll
        for (int cz = 0; cz < 8; cz++) {
            uint32_t b = n4[cz];
            b |= __shfl_xor_sync(0xffffffffu, b, 1);
            b |= __shfl_xor_sync(0xffffffffu, b, 2);
            uint32_t w = (lane & 3u) == 0u ? b << (((lane >> 2) & 3u) * 8u) : 0u;
            w |= __shfl_xor_sync(0xffffffffu, w, 4);
            w |= __shfl_xor_sync(0xffffffffu, w, 8);
            if ((lane & 15u) == 0u) sb[cz * 2 + (lane >> 4)] = w;
        }
        // 8^3 cells: bit ((cz * 4 + cy) * 4 + cx), cy = lane / 8
        uint32_t w8[2] = {0u, 0u};
#pragma unroll
        for (int cz = 0; cz < 4; cz++) {
            const uint32_t b = n4[2 * cz] | n4[2 * cz + 1];
            uint32_t c3 = 0;
#pragma unroll
            for (int cx = 0; cx < 4; cx++) c3 |= ((b >> (2 * cx)) & 3u) ? (1u << cx) : 0u;
            c3 |= __shfl_xor_sync(0xffffffffu, c3, 1);
            c3 |= __shfl_xor_sync(0xffffffffu, c3, 2);
            c3 |= __shfl_xor_sync(0xffffffffu, c3, 4);
            if ((lane & 7u) == 0u) w8[cz >> 1] |= c3 << ((cz & 1) * 16 + (lane >> 3) * 4);
        }
#pragma unroll
        for (int k = 0; k < 2; k++) {
            w8[k] |= __shfl_xor_sync(0xffffffffu, w8[k], 8);
            w8[k] |= __shfl_xor_sync(0xffffffffu, w8[k], 16);
        }
        if (lane == 0) { sb[16] = w8[0]; sb[17] = w8[1]; }
        if (lane == 0) atomicAdd(&counters[S_NONEMPTY], 1u);
        const uint32_t bx = (uint32_t)(i % B), by = (uint32_t)((i / B) % B), bz = (uint32_t)(i / ((uint64_t)B * B));
        if (lane < n_levels) {
            const uint32_t s = lane, n = B >> s;
            const uint64_t idx = ((uint64_t)(bz >> s) * n + (by >> s)) * n + (bx >> s);
            atomicOr(&occ[occ_off[s] + (idx >> 5)], 1u << (idx & 31u));
        }
    }
}

// ---------------------------------------------------------------------------
// incremental update: blocks a moved object covered before or covers now
// ---------------------------------------------------------------------------

// Conservative world box of every non-empty cluster of one object -- the box
// k_svo_candidates selects blocks with -- marked into the dirty-block map.
__device__ void mark_object_blocks(const tgx_object& od, const uint32_t* __restrict__ cluster_pointers,
                                   const uint32_t* __restrict__ bits, const float mn[3], uint32_t B,
                                   uint8_t* __restrict__ dirty)
{
    const uint32_t n = od.n_cluster_pointers_per_dim[0] * od.n_cluster_pointers_per_dim[1] * od.n_cluster_pointers_per_dim[2];
    for (uint32_t rel = threadIdx.x; rel < n; rel += blockDim.x) {
        const uint32_t ci = cluster_pointers[od.first_cluster_pointer + rel];
        const uint4* w = reinterpret_cast<const uint4*>(bits + (uint64_t)ci * 16u);
        const uint4 a = w[0], b = w[1], c = w[2], d = w[3];
        if (!(a.x | a.y | a.z | a.w | b.x | b.y | b.z | b.w | c.x | c.y | c.z | c.w | d.x | d.y | d.z | d.w)) continue;
        float off[3], ohe[3];
        cluster_offsets(od, rel, off, ohe);
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const float lx = off[0] + ((k & 1) ? 8.0f : 0.0f) - ohe[0];
            const float ly = off[1] + ((k & 2) ? 8.0f : 0.0f) - ohe[1];
            const float lz = off[2] + ((k & 4) ? 8.0f : 0.0f) - ohe[2];
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const float p = DM(od.rotation, r, 0) * lx + DM(od.rotation, r, 1) * ly + DM(od.rotation, r, 2) * lz +
                                od.translation[r];
                lo[r] = fminf(lo[r], p);
                hi[r] = fmaxf(hi[r], p);
            }
        }
        int b0[3], b1[3];
        bool empty = false;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const float slack = 0.5f + 1e-5f * fabsf(lo[r]) + 1e-5f * fabsf(hi[r]);
            b0[r] = max((int)floorf((lo[r] - slack - mn[r]) / 32.0f), 0);
            b1[r] = min((int)floorf((hi[r] + slack - mn[r]) / 32.0f), (int)B - 1);
            empty |= b0[r] > b1[r];
        }
        if (empty) continue;
        for (int bz = b0[2]; bz <= b1[2]; bz++)
            for (int by = b0[1]; by <= b1[1]; by++)
                for (int bx = b0[0]; bx <= b1[0]; bx++) dirty[((uint32_t)bz * B + (uint32_t)by) * B + (uint32_t)bx] = 1;
    }
}

// One CTA per object: when the scene's record differs from the one the SVO
// was built from, the blocks its clusters touched before (old record) and
// touch now (new record) become dirty, and the stored record is replaced.
__global__ void __launch_bounds__(128) k_svo_mark_dirty(const tgx_object* __restrict__ cur, tgx_object* __restrict__ built,
                                                       const uint32_t* __restrict__ cluster_pointers,
                                                       const uint32_t* __restrict__ bits, float mnx, float mny,
                                                       float mnz, uint32_t B, uint8_t* __restrict__ dirty,
                                                       uint32_t* __restrict__ counters)
{
    const tgx_object now = cur[blockIdx.x], was = built[blockIdx.x];
    const uint32_t* a = reinterpret_cast<const uint32_t*>(&now);
    const uint32_t* b = reinterpret_cast<const uint32_t*>(&was);
    bool same = true;
#pragma unroll
    for (int k = 0; k < (int)(sizeof(tgx_object) / 4); k++) same &= a[k] == b[k];
    if (same) return;
    const float mn[3] = {mnx, mny, mnz};
    mark_object_blocks(was, cluster_pointers, bits, mn, B, dirty);
    mark_object_blocks(now, cluster_pointers, bits, mn, B, dirty);
    __syncthreads();
    if (threadIdx.x == 0) {
        built[blockIdx.x] = now;
        atomicAdd(&counters[S_MOVED], 1u);
    }
}

// One warp per dirty block that holds a slot: its voxel bits, sub-block masks,
// non-empty flag and materials are zeroed, the table entry is emptied and the
// slot goes on the free list.  k_svo_candidates re-marks the block if any
// cluster still reaches it.
__global__ void __launch_bounds__(256) k_svo_release_dirty(uint32_t* __restrict__ table, uint64_t n_table,
                                                          const uint8_t* __restrict__ dirty, uint32_t* __restrict__ pool,
                                                          uint32_t* __restrict__ sub, uint32_t* __restrict__ nonempty,
                                                          uint16_t* __restrict__ mat, uint32_t* __restrict__ free_tail,
                                                          uint32_t* __restrict__ counters)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = warp; i < n_table; i += n_warps) {
        if (!dirty[i]) continue;
        const uint32_t tv = table[i];
        if (tv == 0u) continue;
        const uint32_t slot = tv - 1u;
        uint4* blk = reinterpret_cast<uint4*>(pool + (uint64_t)slot * kBlockWords);
        for (uint32_t k = lane; k < kBlockWords / 4u; k += 32) blk[k] = make_uint4(0u, 0u, 0u, 0u);
        sub[(uint64_t)slot * 32u + lane] = 0u;
        if (mat) {
            uint4* m = reinterpret_cast<uint4*>(mat + (uint64_t)slot * 32768u);
            for (uint32_t k = lane; k < 32768u / 8u; k += 32) m[k] = make_uint4(0u, 0u, 0u, 0u);
        }
        if (lane == 0) {
            nonempty[slot] = 0u;
            table[i] = 0u;
            free_tail[atomicAdd(&counters[S_FREED], 1u)] = slot;
        }
    }
}

// Table entries still marked after an overflowed candidate pass go back to empty.
__global__ void __launch_bounds__(256) k_svo_unmark(uint32_t* __restrict__ table, uint64_t n_table)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_table; i += (uint64_t)gridDim.x * blockDim.x)
        if (table[i] == kMark) table[i] = 0u;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static void svo_free(tgx_svo* s)
{
    if (!s) return;
    cudaFree(s->d_table);
    cudaFree(s->d_pool);
    cudaFree(s->d_sub);
    cudaFree(s->d_occ);
    cudaFree(s->d_nonempty);
    cudaFree(s->d_mat);
    cudaFree(s->d_free);
    cudaFree(s->d_counters);
    cudaFree(s->d_objs);
    delete s;
}

static uint64_t svo_device_bytes(const tgx_svo* s)
{
    const uint64_t n_table = (uint64_t)s->B * s->B * s->B;
    return n_table * 4 + (uint64_t)s->pool_cap * (kBlockWords * 4 + 128 + 4 + 4 + (s->d_mat ? 65536 : 0)) +
           s->occ_words * 4 + (uint64_t)s->n_objects * sizeof(tgx_object);
}

// Per-slot arrays (pool, sub masks, non-empty flags, free list, materials)
// sized for `cap` slots; the first `keep` slots are carried over.  The rest
// of the small arrays start zero; pool and material slots are written whole
// by the voxeliser before anything reads them.
static tgx_status svo_resize_slots(tgx_ctx* c, tgx_svo* s, uint32_t cap, uint32_t keep, bool materials)
{
    struct Arr { void** p; uint64_t per_slot; };
    void* mat = s->d_mat;
    Arr arrs[5] = {{(void**)&s->d_pool, kBlockWords * 4}, {(void**)&s->d_sub, 128}, {(void**)&s->d_nonempty, 4},
                   {(void**)&s->d_free, 4}, {&mat, 65536}};
    const int n_arr = materials ? 5 : 4;
    void* fresh[5] = {};
    for (int a = 0; a < n_arr; a++)
        if (cudaMalloc(&fresh[a], (uint64_t)cap * arrs[a].per_slot) != cudaSuccess) {
            for (int k = 0; k < a; k++) cudaFree(fresh[k]);
            cudaGetLastError();
            tgx_set_error("tgx_svo: out of device memory for %u blocks", cap);
            return TGX_ERR_OUT_OF_MEMORY;
        }
    for (int a = 0; a < n_arr; a++) {
        const uint64_t kept = (uint64_t)keep * arrs[a].per_slot, total = (uint64_t)cap * arrs[a].per_slot;
        if (kept) TGX_CUDA(cudaMemcpyAsync(fresh[a], *arrs[a].p, kept, cudaMemcpyDeviceToDevice, c->stream));
        if (a != 0 && a != 4) TGX_CUDA(cudaMemsetAsync((char*)fresh[a] + kept, 0, total - kept, c->stream));
    }
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    for (int a = 0; a < n_arr; a++) {
        cudaFree(*arrs[a].p);
        *arrs[a].p = fresh[a];
    }
    s->d_mat = (uint16_t*)mat;
    s->pool_cap = cap;
    return TGX_OK;
}

// Candidate pass over every cluster pointer (only blocks marked in `dirty` when
// it is given), with the pair storage grown to the exact count and the pass
// rerun once when the first estimate was short.  Leaves the counters on the host.
static tgx_status svo_candidates(tgx_ctx* c, tgx_svo* s, const tgx_scene* sc, const uint8_t* dirty, uint64_t cap)
{
    const uint64_t n_table = (uint64_t)s->B * s->B * s->B;
    uint32_t* counters = s->d_counters;
    for (int attempt = 0; attempt < 2; attempt++) {
        TGX_TRY(devbuf_reserve(c->svo_pairs, cap * sizeof(SvoPair)));
        TGX_CUDA(cudaMemsetAsync(counters + S_PAIRS, 0, 2 * 4, c->stream));   // pairs, marks
        if (sc->n_cluster_pointers)
            TGX_LAUNCH(c, TR_SVO_CANDIDATES, (sc->n_cluster_pointers + 127) / 128, 128, 0, k_svo_candidates, sc->d_objects,
                       sc->d_cluster_pointers, sc->d_c2o, sc->d_bits, sc->n_cluster_pointers, s->mn[0], s->mn[1], s->mn[2],
                       s->L, s->B, s->d_table, (SvoPair*)c->svo_pairs.ptr, (uint32_t)cap, counters, c->d_status, dirty);
        if (cudaMemcpyAsync(c->h_counter, counters, S_COUNT * 4, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess) {
            tgx_set_error("tgx_svo: %s", cudaGetErrorString(cudaGetLastError()));
            return TGX_ERR_CUDA;
        }
        const uint32_t n_pairs = ((uint32_t*)c->h_counter)[S_PAIRS];
        if (n_pairs <= cap) return TGX_OK;
        // the capacity error recorded by the first attempt is expected; clear it and the marks it left
        TGX_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(tgx_dev_status), c->stream));
        const uint32_t grid = (uint32_t)std::min<uint64_t>((n_table + 255) / 256, (uint64_t)c->num_sms * 32);
        TGX_LAUNCH(c, TR_SVO_ALLOC, grid, 256, 0, k_svo_unmark, s->d_table, n_table);
        cap = (uint64_t)n_pairs + 1024;
    }
    tgx_set_error("tgx_svo: pair count grew between two identical passes");
    return TGX_ERR_CAPACITY;
}

// Slots for the marked blocks, voxelisation of the pairs, and the occupancy
// pyramid of the whole table (cleared first).
static tgx_status svo_fill(tgx_ctx* c, tgx_svo* s, const tgx_scene* sc, uint32_t n_free, uint32_t next_slot)
{
    const uint64_t n_table = (uint64_t)s->B * s->B * s->B;
    uint32_t* counters = s->d_counters;
    const uint32_t grid = (uint32_t)std::min<uint64_t>((n_table + 255) / 256, (uint64_t)c->num_sms * 32);
    TGX_CUDA(cudaMemsetAsync(counters + S_SLOTS, 0, 2 * 4, c->stream));   // slots, non-empty
    TGX_CUDA(cudaMemsetAsync(s->d_occ, 0, s->occ_words * 4, c->stream));
    TGX_LAUNCH(c, TR_SVO_ALLOC, grid, 256, 0, k_svo_alloc, s->d_table, n_table, counters, s->d_free, n_free, next_slot,
               s->pool_cap, c->d_status);
    // group the pairs by block slot: counts, offsets, placement
    const uint32_t cap = (uint32_t)(c->svo_pairs.bytes / sizeof(SvoPair));
    const uint64_t n_slots = s->pool_cap;
    const size_t sort_bytes = (size_t)(n_slots + 1) * 4 * 2 + (size_t)std::max<uint64_t>(s->n_pairs, 1) * sizeof(SvoPair) + 64;
    TGX_TRY(devbuf_reserve(c->svo_sort, sort_bytes));
    uint32_t* cnt = (uint32_t*)c->svo_sort.ptr;
    uint32_t* off = cnt + (n_slots + 1);
    SvoPair* sorted = (SvoPair*)(((uintptr_t)(off + n_slots + 1) + 15) & ~(uintptr_t)15);
    const uint32_t pgrid_pairs = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((s->n_pairs + 255) / 256, (uint64_t)c->num_sms * 16));
    TGX_CUDA(cudaMemsetAsync(cnt, 0, n_slots * 4, c->stream));
    TGX_LAUNCH(c, TR_SVO_VOXELIZE, pgrid_pairs, 256, 0, k_svo_pair_count, (const SvoPair*)c->svo_pairs.ptr, counters, cap,
               s->d_table, cnt);
    TGX_LAUNCH(c, TR_SVO_VOXELIZE, 1, 1024, 0, k_svo_pair_scan, cnt, (uint32_t)n_slots, off);
    TGX_CUDA(cudaMemsetAsync(cnt, 0, n_slots * 4, c->stream));
    TGX_LAUNCH(c, TR_SVO_VOXELIZE, pgrid_pairs, 256, 0, k_svo_pair_fill, (const SvoPair*)c->svo_pairs.ptr, counters, cap,
               s->d_table, off, cnt, sorted);
    // one CTA per slot: the block's image and material grid in shared memory
    static bool attr = false;
    if (!attr) {
        TGX_CUDA(cudaFuncSetAttribute(k_svo_voxelize<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (kBlockWords + 16384) * 4));
        attr = true;
    }
    if (s->d_mat)
        TGX_LAUNCH(c, TR_SVO_VOXELIZE, (uint32_t)n_slots, 32 * kWarpsPerVoxCta, (kBlockWords + 16384) * 4,
                   k_svo_voxelize<true>, sc->d_objects, sc->d_cluster_pointers, sc->d_c2o, sc->d_bits, sorted, off,
                   s->d_pool, sc->d_material, s->d_mat, s->mn[0], s->mn[1], s->mn[2], s->B);
    else
        TGX_LAUNCH(c, TR_SVO_VOXELIZE, (uint32_t)n_slots, 32 * kWarpsPerVoxCta, kBlockWords * 4, k_svo_voxelize<false>,
                   sc->d_objects, sc->d_cluster_pointers, sc->d_c2o, sc->d_bits, sorted, off, s->d_pool,
                   (const uint8_t*)nullptr, (uint16_t*)nullptr, s->mn[0], s->mn[1], s->mn[2], s->B);
    const uint32_t pgrid = (uint32_t)std::min<uint64_t>((n_table * 32 + 255) / 256, (uint64_t)c->num_sms * 32);
    TGX_LAUNCH(c, TR_SVO_PYRAMID, pgrid, 256, 0, k_svo_pyramid, s->d_table, n_table, s->d_pool, s->d_nonempty, s->d_sub,
               s->d_occ, (const uint64_t*)((char*)s->d_occ + svo_occ_off_bytes(s->occ_words)), s->n_levels, s->B, counters);
    return TGX_OK;
}

extern "C" tgx_status tgx_svo_build(tgx_ctx* c, const tgx_scene* sc, const float* mn, uint32_t L, tgx_svo** out)
{
    return tgx_svo_build_flags(c, sc, mn, L, 0u, out);
}

extern "C" tgx_status tgx_svo_build_flags(tgx_ctx* c, const tgx_scene* sc, const float* mn, uint32_t L, uint32_t flags,
                                          tgx_svo** out)
{
    if (flags & ~TGX_SVO_NO_MATERIALS) { tgx_set_error("tgx_svo_build: unknown flags %u", flags); return TGX_ERR_INVALID_ARGUMENT; }
    if (!c || !sc || !mn || !out) { tgx_set_error("tgx_svo_build: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    if (L < 6 || L > 14) { tgx_set_error("tgx_svo_build: extent_log2 %u outside 6..14", L); return TGX_ERR_INVALID_ARGUMENT; }
    for (int i = 0; i < 3; i++)
        if (!(fabsf(mn[i]) <= 16777216.0f) || mn[i] != floorf(mn[i])) {
            tgx_set_error("tgx_svo_build: min must be integral and |min| <= 2^24");
            return TGX_ERR_INVALID_ARGUMENT;
        }
    TGX_CUDA(cudaSetDevice(c->device));
    tgx_svo* s = new (std::nothrow) tgx_svo();
    if (!s) return TGX_ERR_OUT_OF_MEMORY;
    s->mn[0] = mn[0]; s->mn[1] = mn[1]; s->mn[2] = mn[2];
    s->L = L;
    s->B = 1u << (L - 5);
    s->n_objects = sc->n_objects;
    s->n_cluster_pointers = sc->n_cluster_pointers;
    const uint64_t n_table = (uint64_t)s->B * s->B * s->B;
    s->n_levels = L - 5 + 1;
    uint64_t occ_words = 0;
    for (uint32_t l = 0; l < s->n_levels; l++) {
        const uint64_t n = (uint64_t)(s->B >> l);
        s->occ_off[l] = occ_words;
        occ_words += (n * n * n + 31) / 32;
    }
    s->occ_words = occ_words;

    auto fail = [&](tgx_status st) { cudaStreamSynchronize(c->stream); svo_free(s); return st; };
    if (cudaMalloc(&s->d_table, n_table * 4) != cudaSuccess || cudaMalloc(&s->d_occ, occ_words * 4 + 128) != cudaSuccess ||
        cudaMalloc(&s->d_counters, S_COUNT * 4) != cudaSuccess ||
        cudaMalloc(&s->d_objs, std::max<uint64_t>(1, (uint64_t)sc->n_objects) * sizeof(tgx_object)) != cudaSuccess) {
        cudaGetLastError();
        tgx_set_error("tgx_svo_build: out of device memory for the block table");
        return fail(TGX_ERR_OUT_OF_MEMORY);
    }
    if (cudaMemsetAsync(s->d_table, 0, n_table * 4, c->stream) != cudaSuccess ||
        cudaMemsetAsync(s->d_counters, 0, S_COUNT * 4, c->stream) != cudaSuccess ||
        (sc->n_objects && cudaMemcpyAsync(s->d_objs, sc->d_objects, (uint64_t)sc->n_objects * sizeof(tgx_object),
                                          cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) ||
        cudaMemcpyAsync((char*)s->d_occ + svo_occ_off_bytes(occ_words), s->occ_off, sizeof(s->occ_off), cudaMemcpyHostToDevice,
                        c->stream) != cudaSuccess) {
        tgx_set_error("tgx_svo_build: memset failed");
        return fail(TGX_ERR_CUDA);
    }
    tgx_status st;
    // pair storage: start from a per-cluster estimate, retry once with the exact count
    if ((st = svo_candidates(c, s, sc, nullptr, std::max<uint64_t>(1024, (uint64_t)sc->n_cluster_pointers * 4))) != TGX_OK)
        return fail(st);
    const uint32_t* hc = (const uint32_t*)c->h_counter;
    s->n_pairs = hc[S_PAIRS];
    s->n_blocks = hc[S_MARKED];
    s->n_slots = s->n_blocks;
    const bool materials = sc->d_material && sc->d_luts && !(flags & TGX_SVO_NO_MATERIALS);
    if ((st = svo_resize_slots(c, s, std::max(s->n_blocks, 1u), 0, materials)) != TGX_OK) return fail(st);
    if ((st = svo_fill(c, s, sc, 0, 0)) != TGX_OK) return fail(st);
    s->device_bytes = svo_device_bytes(s);
    *out = s;
    return TGX_OK;
}

extern "C" tgx_status tgx_svo_update(tgx_ctx* c, tgx_svo* s, const tgx_scene* sc, uint32_t* out_n_moved)
{
    if (!c || !s || !sc) { tgx_set_error("tgx_svo_update: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    if (sc->n_objects != s->n_objects || sc->n_cluster_pointers != s->n_cluster_pointers) {
        tgx_set_error("tgx_svo_update: the scene has %u objects / %u cluster pointers, the SVO was built from %u / %u",
                      sc->n_objects, sc->n_cluster_pointers, s->n_objects, s->n_cluster_pointers);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (out_n_moved) *out_n_moved = 0;
    if (sc->n_objects == 0) return TGX_OK;
    TGX_CUDA(cudaSetDevice(c->device));
    const uint64_t n_table = (uint64_t)s->B * s->B * s->B;
    TGX_TRY(devbuf_reserve(c->svo_scratch, n_table));
    uint8_t* dirty = (uint8_t*)c->svo_scratch.ptr;
    uint32_t* counters = s->d_counters;
    TGX_CUDA(cudaMemsetAsync(dirty, 0, n_table, c->stream));
    TGX_CUDA(cudaMemsetAsync(counters + S_FREED, 0, 2 * 4, c->stream));   // freed, moved
    TGX_LAUNCH(c, TR_SVO_CANDIDATES, sc->n_objects, 128, 0, k_svo_mark_dirty, sc->d_objects, s->d_objs, sc->d_cluster_pointers,
               sc->d_bits, s->mn[0], s->mn[1], s->mn[2], s->B, dirty, counters);
    const uint32_t wgrid = (uint32_t)std::min<uint64_t>((n_table * 32 + 255) / 256, (uint64_t)c->num_sms * 32);
    TGX_LAUNCH(c, TR_SVO_ALLOC, wgrid, 256, 0, k_svo_release_dirty, s->d_table, n_table, dirty, s->d_pool, s->d_sub,
               s->d_nonempty, s->d_mat, s->d_free + s->n_free, counters);
    // pairs of the dirty blocks, into the pair storage the last build left (grown when short)
    TGX_TRY(svo_candidates(c, s, sc, dirty, std::max<uint64_t>(1024, c->svo_pairs.bytes / sizeof(SvoPair))));
    const uint32_t* hc = (const uint32_t*)c->h_counter;
    const uint32_t n_moved = hc[S_MOVED], n_freed = hc[S_FREED], n_marked = hc[S_MARKED];
    if (out_n_moved) *out_n_moved = n_moved;
    if (n_moved == 0) return TGX_OK;
    const uint32_t n_free = s->n_free + n_freed;
    const uint32_t fresh = n_marked > n_free ? n_marked - n_free : 0u;
    const uint32_t need = s->n_slots + fresh;
    if (need > s->pool_cap) TGX_TRY(svo_resize_slots(c, s, need + need / 4 + 64, s->n_slots, s->d_mat != nullptr));
    s->n_pairs = hc[S_PAIRS];
    TGX_TRY(svo_fill(c, s, sc, n_free, s->n_slots));
    s->n_free = n_free - (n_marked - fresh);
    s->n_slots = need;
    s->n_blocks = s->n_blocks - n_freed + n_marked;
    s->device_bytes = svo_device_bytes(s);
    return TGX_OK;
}

extern "C" void tgx_svo_destroy(tgx_ctx* c, tgx_svo* s)
{
    if (c) cudaStreamSynchronize(c->stream);
    svo_free(s);
}

extern "C" tgx_status tgx_svo_get_info(tgx_ctx* c, const tgx_svo* s, tgx_svo_info* out)
{
    if (!c || !s || !out) return TGX_ERR_INVALID_ARGUMENT;
    TGX_CUDA(cudaMemcpyAsync(c->h_counter, s->d_counters, S_COUNT * 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    out->min[0] = s->mn[0]; out->min[1] = s->mn[1]; out->min[2] = s->mn[2];
    out->extent_log2 = s->L;
    out->blocks_per_axis = s->B;
    out->n_blocks = s->n_blocks;
    out->n_nonempty_blocks = ((const uint32_t*)c->h_counter)[S_NONEMPTY];
    out->n_pairs = s->n_pairs;
    out->device_bytes = s->device_bytes;
    return TGX_OK;
}

extern "C" tgx_status tgx_svo_download(tgx_ctx* c, const tgx_svo* s, int32_t* out_xyz, uint32_t* out_words,
                                       uint32_t capacity, uint32_t* out_n)
{
    if (!c || !s || !out_n) return TGX_ERR_INVALID_ARGUMENT;
    const uint64_t n_table = (uint64_t)s->B * s->B * s->B;
    std::vector<uint32_t> table(n_table), nonempty(std::max(s->n_slots, 1u));
    TGX_CUDA(cudaMemcpyAsync(table.data(), s->d_table, n_table * 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaMemcpyAsync(nonempty.data(), s->d_nonempty, nonempty.size() * 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    uint32_t n = 0;
    for (uint64_t i = 0; i < n_table; i++) {
        const uint32_t tv = table[i];
        if (!tv || !nonempty[tv - 1]) continue;
        if (n < capacity) {
            if (out_xyz) {
                out_xyz[3 * n + 0] = (int32_t)(s->mn[0] + (float)((i % s->B) * kBlockSide));
                out_xyz[3 * n + 1] = (int32_t)(s->mn[1] + (float)(((i / s->B) % s->B) * kBlockSide));
                out_xyz[3 * n + 2] = (int32_t)(s->mn[2] + (float)((i / ((uint64_t)s->B * s->B)) * kBlockSide));
            }
            if (out_words)
                TGX_CUDA(cudaMemcpyAsync(out_words + (uint64_t)n * kBlockWords, s->d_pool + (uint64_t)(tv - 1) * kBlockWords,
                                         kBlockWords * 4, cudaMemcpyDeviceToHost, c->stream));
        }
        n++;
    }
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    *out_n = n;
    return TGX_OK;
}

namespace {

__global__ void __launch_bounds__(128) k_svo_trace(SvoDev s, uint32_t n, const float* __restrict__ o,
                                                  const float* __restrict__ d, uint32_t max_steps,
                                                  float* __restrict__ out_t, int32_t* __restrict__ out_voxel,
                                                  uint32_t* __restrict__ n_exhausted)
{
    __shared__ uint32_t occ_off[16];
    __shared__ LevelDesc lv[16];
    __shared__ uint8_t first_level[kFirstLevelSize];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 16; k++) occ_off[k] = s.occ_off[k];
    }
    __syncthreads();
    svo_level_tables(s.L, s.NL, s.B, s.occ, s.pool, s.sub, occ_off, lv, first_level);
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float oi[3] = {o[3 * i], o[3 * i + 1], o[3 * i + 2]};
    const float di[3] = {d[3 * i], d[3 * i + 1], d[3 * i + 2]};
    float t;
    int32_t c[3], ax;
    uint32_t steps;
    const int r = svo_trace(s, lv, first_level, oi, di, max_steps, t, c, ax, steps);
    if (r == 1) {
        out_t[i] = t;
        out_voxel[3 * i] = c[0] + (int32_t)s.mn[0];
        out_voxel[3 * i + 1] = c[1] + (int32_t)s.mn[1];
        out_voxel[3 * i + 2] = c[2] + (int32_t)s.mn[2];
    } else {
        out_t[i] = F32_MAX_TG;
        out_voxel[3 * i] = out_voxel[3 * i + 1] = out_voxel[3 * i + 2] = 0;
        if (r < 0) atomicAdd(n_exhausted, 1u);
    }
}

}  // namespace

extern "C" tgx_status tgx_svo_trace(tgx_ctx* c, const tgx_svo* s, uint32_t n, const float* d_o, const float* d_d,
                                    uint32_t max_steps, float* d_t, int32_t* d_voxel)
{
    if (!c || !s || (n && (!d_o || !d_d || !d_t || !d_voxel))) {
        tgx_set_error("tgx_svo_trace: NULL argument");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return TGX_OK;
    TGX_TRY(devbuf_reserve(c->svo_counters, S_COUNT * 4 + 64));
    uint32_t* exhausted = (uint32_t*)c->svo_counters.ptr + S_COUNT;
    TGX_LAUNCH(c, TR_SVO_TRACE, (n + 127) / 128, 128, 0, k_svo_trace, svo_dev(s), n, d_o, d_d, max_steps, d_t, d_voxel,
               exhausted);
    return TGX_OK;
}
