// tgx_internal.cuh -- shared internals of libtgx (not part of the C ABI).
#pragma once

#include "../../include/tgx.h"

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>

// ---------------------------------------------------------------------------
// Error plumbing
// ---------------------------------------------------------------------------

void tgx_set_error(const char* fmt, ...);

#define TGX_CUDA(call)                                                                                     \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess) {                                                                           \
            tgx_set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
            return e_ == cudaErrorMemoryAllocation ? TGX_ERR_OUT_OF_MEMORY : TGX_ERR_CUDA;                 \
        }                                                                                                  \
    } while (0)

#define TGX_CHECK_LAUNCH(ctx)                                                                              \
    do {                                                                                                   \
        cudaError_t e_ = cudaGetLastError();                                                               \
        if (e_ != cudaSuccess) {                                                                           \
            tgx_set_error("kernel launch failed: %s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__); \
            return TGX_ERR_CUDA;                                                                           \
        }                                                                                                  \
        (ctx)->launches++;                                                                                 \
    } while (0)

#define TGX_TRY(expr)                      \
    do {                                   \
        tgx_status s_ = (expr);            \
        if (s_ != TGX_OK) return s_;       \
    } while (0)

// Device status word: the first error wins.
struct tgx_dev_status
{
    uint32_t code;
    uint32_t where;
    unsigned long long detail;
};

__device__ __forceinline__ void dev_error(tgx_dev_status* st, uint32_t code, uint32_t where, unsigned long long detail)
{
    if (atomicCAS(&st->code, 0u, code) == 0u) {
        st->where = where;
        st->detail = detail;
    }
}

// Growable device buffer.
struct DevBuf
{
    void*  ptr = nullptr;
    size_t bytes = 0;
};

tgx_status devbuf_reserve(DevBuf& b, size_t bytes);
void       devbuf_free(DevBuf& b);

// ---------------------------------------------------------------------------
// Context and resources
// ---------------------------------------------------------------------------

// Kernel slots for tracing (tgx_trace_*).
enum TraceSlot
{
    TR_OBJECT_SETUP = 0,
    TR_VIS_SETUP,
    TR_VIS_COUNT,
    TR_VIS_PREFIX,
    TR_VIS_SCAN,
    TR_VIS_BIN,
    TR_VIS_TILES,
    TR_SVO_CANDIDATES,
    TR_SVO_ALLOC,
    TR_SVO_VOXELIZE,
    TR_SVO_PYRAMID,
    TR_SVO_TRACE,
    TR_GI,
    TR_GI_TRACE,
    TR_MLP,          // inference
    TR_MLP_FWD_BWD,
    TR_MLP_WGRAD,
    TR_MLP_ADAM,
    TR_COUNT
};

struct TraceState
{
    bool enabled = false;
    struct Pending { int slot; cudaEvent_t a, b; };
    Pending* pending = nullptr;
    size_t n_pending = 0, cap_pending = 0;
    cudaEvent_t* free_events = nullptr;
    size_t n_free = 0, cap_free = 0;
    double ms[TR_COUNT] = {};
    uint64_t launches[TR_COUNT] = {};
};

struct tgx_ctx
{
    TraceState trace;
    int            device = 0;
    cudaStream_t   stream = nullptr;
    bool           own_stream = false;
    uint32_t       tile_w = 16, tile_h = 16;
    uint32_t       flags = 0;
    uint64_t       launches = 0;
    int            num_sms = 0;
    tgx_dev_status* d_status = nullptr;

    // visibility scratch
    DevBuf vis_records;    // visible-cluster records
    DevBuf vis_counters;   // small counters
    DevBuf vis_tile_cnt;   // per-tile counts
    DevBuf vis_tile_off;   // per-tile offsets (exclusive scan), n_tiles+1
    DevBuf vis_bins;       // tile -> record indices
    DevBuf vis_views;      // device copies of the views
    DevBuf svo_counters;   // SVO build counters
    DevBuf svo_pairs;      // (cluster, block) voxelisation pairs
    DevBuf gi_scratch;     // learned-cache GI queries, hits, training batch
    DevBuf svo_scratch;    // SVO update: dirty-block marks
    DevBuf svo_sort;       // SVO build: pairs grouped by block slot, per-slot counts and offsets
    DevBuf vis_work;       // work counters of the tile kernel's counting variant
    uint64_t mem_budget = 0;           // bytes the context's scene stores may hold (0: no limit)
    uint64_t mem_scenes = 0;           // bytes its live scene stores hold
    uint32_t vis_tile_ctas = 0;        // resident CTAs of the persistent (batched-frame) tile kernel
    bool   vis_count_work = false;
    uint32_t vis_bshift = 1;           // depth buckets per tile: 32 >> vis_bshift
    uint32_t vis_batch = 48;           // entries per staged batch of the tile kernel
    uint32_t vis_drain = 32;           // live pairs a warp collects before running their DDAs
    uint32_t vis_last_tiles = 0;
    uint64_t vis_last_pairs = 0;
    void*  h_vis_counters = nullptr;   // pinned copy of the last frame's counters
    cudaEvent_t vis_done = nullptr;    // recorded after that copy
    DevBuf host_stage;     // pinned host staging (views)
    void*  h_pinned = nullptr;
    size_t h_pinned_bytes = 0;
    uint64_t* h_counter = nullptr;   // pinned u64 readback slot
    uint32_t trace_steps_per_round = 8;   // DDA steps a traversal lane runs between queue refills
    // pipelined host-buffer renders (tgx_vis_render_host_async): two device
    // copies of the buffers, the copy stream and per-copy events
    cudaStream_t copy_stream = nullptr;
    DevBuf host_slot[2];
    cudaEvent_t host_rendered[2] = {nullptr, nullptr};
    cudaEvent_t host_copied[2] = {nullptr, nullptr};
    uint64_t host_issued = 0, host_done = 0;
};

struct tgx_scene
{
    uint32_t    n_objects = 0, n_cluster_pointers = 0, n_clusters = 0, n_luts = 0;
    uint64_t    bytes = 0;                 // device bytes of the store, counted against the context's budget
    tgx_object* d_objects = nullptr;
    float*      d_inv_rot = nullptr;       // per object: 3x3 linear part of inverse(rotation), row-major
    uint32_t*   d_cluster_pointers = nullptr;
    uint32_t*   d_c2o = nullptr;
    uint32_t*   d_bits = nullptr;
    uint32_t*   d_cp_obj = nullptr;        // per cluster pointer: its object, bit 31 set when its cluster is empty
                                           // (built once: pointers, owners and bits never change after upload)
    uint8_t*    d_material = nullptr;
    tgx_material* d_luts = nullptr;
};

// One-bit SVO on the device (built by tgx_svo_build, svo.cu).
struct tgx_svo
{
    float     mn[3] = {0, 0, 0};
    uint32_t  L = 0;              // extent_log2
    uint32_t  B = 0;              // blocks per axis
    uint32_t  n_blocks = 0;       // live blocks: table entries that hold a slot
    uint32_t  n_slots = 0;        // slots handed out so far (live blocks + free slots)
    uint32_t  pool_cap = 0;       // slots the pool, sub, nonempty, material and free arrays hold
    uint32_t  n_free = 0;         // slots released by updates, d_free[0 .. n_free)
    uint32_t* d_free = nullptr;
    uint32_t* d_counters = nullptr;  // this SVO's build counters (pairs, marks, slots, non-empty, freed)
    tgx_object* d_objs = nullptr; // object records the SVO reflects (updates diff the scene against them)
    uint32_t  n_objects = 0, n_cluster_pointers = 0;
    uint32_t  n_pairs = 0;
    uint32_t* d_table = nullptr;  // B^3 entries: 0 = no block, else slot + 1
    uint32_t* d_pool = nullptr;   // pool_cap * 1024 words
    uint32_t* d_sub = nullptr;    // pool_cap * 32 words: 4^3-cell and 8^3-cell occupancy of each block
    uint32_t* d_occ = nullptr;    // occupancy pyramid, level 0 = blocks
    uint64_t  occ_words = 0;
    uint64_t  occ_off[10] = {};   // word offset of each level
    uint32_t  n_levels = 0;       // L - 5 + 1 levels (blocks .. root)
    uint32_t* d_nonempty = nullptr;  // per slot: 1 if any bit set
    uint16_t* d_mat = nullptr;    // pool_cap * 32768 material codes ((lut << 8 | byte) + 1, 0 = none) or null
    uint64_t  device_bytes = 0;
};

// ---------------------------------------------------------------------------
// Exact binary32 arithmetic: every parity-critical operation is spelled with
// a round-to-nearest intrinsic so no FMA contraction can change a result.
// ---------------------------------------------------------------------------

#define F32_MAX_TG 3.402823466e+38f       // TG_F32_MAX (common.inc:20)
#define F32_MIN_TG (-3.402823466e+38f)    // TG_F32_MIN (common.inc:21)

__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
// GLSL min/max semantics (GLSL 4.50 section 8.3)
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }

// Column-major 4x4 helpers in the operation order of tg's tgm_m4_* functions.
#define DM(m, r, c) ((m)[4 * (c) + (r)])

__device__ __forceinline__ void dm4_mul(const float* a, const float* b, float* out)
{
    float r[16];
#pragma unroll
    for (int c = 0; c < 4; c++)
#pragma unroll
        for (int row = 0; row < 4; row++)
            r[4 * c + row] = xadd(xadd(xadd(xmul(DM(a, row, 0), DM(b, 0, c)), xmul(DM(a, row, 1), DM(b, 1, c))),
                                       xmul(DM(a, row, 2), DM(b, 2, c))),
                                  xmul(DM(a, row, 3), DM(b, 3, c)));
#pragma unroll
    for (int i = 0; i < 16; i++) out[i] = r[i];
}

__device__ __forceinline__ void dm4_translate(float x, float y, float z, float* m)
{
#pragma unroll
    for (int i = 0; i < 16; i++) m[i] = 0.0f;
    m[0] = m[5] = m[10] = m[15] = 1.0f;
    m[12] = x; m[13] = y; m[14] = z;
}

// tgm_m4_inverse (tg_math.c:2185-2234), cofactor form.
__device__ __forceinline__ void dm4_inverse(const float* m, float* out)
{
#define E(r, c) DM(m, r, c)
#define MS(a, b, c, d) xsub(xmul(a, b), xmul(c, d))
    const float m2323 = MS(E(2,2), E(3,3), E(2,3), E(3,2));
    const float m1323 = MS(E(2,1), E(3,3), E(2,3), E(3,1));
    const float m1223 = MS(E(2,1), E(3,2), E(2,2), E(3,1));
    const float m0323 = MS(E(2,0), E(3,3), E(2,3), E(3,0));
    const float m0223 = MS(E(2,0), E(3,2), E(2,2), E(3,0));
    const float m0123 = MS(E(2,0), E(3,1), E(2,1), E(3,0));
    const float m2313 = MS(E(1,2), E(3,3), E(1,3), E(3,2));
    const float m1313 = MS(E(1,1), E(3,3), E(1,3), E(3,1));
    const float m1213 = MS(E(1,1), E(3,2), E(1,2), E(3,1));
    const float m2312 = MS(E(1,2), E(2,3), E(1,3), E(2,2));
    const float m1312 = MS(E(1,1), E(2,3), E(1,3), E(2,1));
    const float m1212 = MS(E(1,1), E(2,2), E(1,2), E(2,1));
    const float m0313 = MS(E(1,0), E(3,3), E(1,3), E(3,0));
    const float m0213 = MS(E(1,0), E(3,2), E(1,2), E(3,0));
    const float m0312 = MS(E(1,0), E(2,3), E(1,3), E(2,0));
    const float m0212 = MS(E(1,0), E(2,2), E(1,2), E(2,0));
    const float m0113 = MS(E(1,0), E(3,1), E(1,1), E(3,0));
    const float m0112 = MS(E(1,0), E(2,1), E(1,1), E(2,0));
    // (a*p - b*q + c*r) evaluated left to right
#define T3(a, p, b, q, c, r) xadd(xsub(xmul(a, p), xmul(b, q)), xmul(c, r))
    const float det = xdiv(1.0f,
        xsub(xadd(xsub(xmul(E(0,0), T3(E(1,1), m2323, E(1,2), m1323, E(1,3), m1223)),
                       xmul(E(0,1), T3(E(1,0), m2323, E(1,2), m0323, E(1,3), m0223))),
                  xmul(E(0,2), T3(E(1,0), m1323, E(1,1), m0323, E(1,3), m0123))),
             xmul(E(0,3), T3(E(1,0), m1223, E(1,1), m0223, E(1,2), m0123))));
    float r[16];
#define R(rr, cc) r[4 * (cc) + (rr)]
    R(0,0) = xmul(det,  T3(E(1,1), m2323, E(1,2), m1323, E(1,3), m1223));
    R(0,1) = xmul(det, -T3(E(0,1), m2323, E(0,2), m1323, E(0,3), m1223));
    R(0,2) = xmul(det,  T3(E(0,1), m2313, E(0,2), m1313, E(0,3), m1213));
    R(0,3) = xmul(det, -T3(E(0,1), m2312, E(0,2), m1312, E(0,3), m1212));
    R(1,0) = xmul(det, -T3(E(1,0), m2323, E(1,2), m0323, E(1,3), m0223));
    R(1,1) = xmul(det,  T3(E(0,0), m2323, E(0,2), m0323, E(0,3), m0223));
    R(1,2) = xmul(det, -T3(E(0,0), m2313, E(0,2), m0313, E(0,3), m0213));
    R(1,3) = xmul(det,  T3(E(0,0), m2312, E(0,2), m0312, E(0,3), m0212));
    R(2,0) = xmul(det,  T3(E(1,0), m1323, E(1,1), m0323, E(1,3), m0123));
    R(2,1) = xmul(det, -T3(E(0,0), m1323, E(0,1), m0323, E(0,3), m0123));
    R(2,2) = xmul(det,  T3(E(0,0), m1313, E(0,1), m0313, E(0,3), m0113));
    R(2,3) = xmul(det, -T3(E(0,0), m1312, E(0,1), m0312, E(0,3), m0112));
    R(3,0) = xmul(det, -T3(E(1,0), m1223, E(1,1), m0223, E(1,2), m0123));
    R(3,1) = xmul(det,  T3(E(0,0), m1223, E(0,1), m0223, E(0,2), m0123));
    R(3,2) = xmul(det, -T3(E(0,0), m1213, E(0,1), m0213, E(0,2), m0113));
    R(3,3) = xmul(det,  T3(E(0,0), m1212, E(0,1), m0212, E(0,2), m0112));
#undef R
#undef T3
#undef MS
#undef E
#pragma unroll
    for (int i = 0; i < 16; i++) out[i] = r[i];
}

// tgm_m4_mulv4 (tg_math.c:2428-2438): row = ((x*m0 + y*m1) + z*m2) + w*m3
__device__ __forceinline__ void dm4_mulv4(const float* m, float x, float y, float z, float w, float* out3)
{
#pragma unroll
    for (int row = 0; row < 3; row++)
        out3[row] = xadd(xadd(xadd(xmul(x, DM(m, row, 0)), xmul(y, DM(m, row, 1))), xmul(z, DM(m, row, 2))),
                         xmul(w, DM(m, row, 3)));
}

// collide.inc:3-24 (== tg_physics.c:394-406)
__device__ __forceinline__ bool ray_aabb(float ox, float oy, float oz, float dx, float dy, float dz,
                                         float mnx, float mny, float mnz, float mxx, float mxy, float mxz,
                                         float& enter, float& exit_)
{
    const float v0x = dx == 0.0f ? F32_MIN_TG : xdiv(xsub(mnx, ox), dx);
    const float v0y = dy == 0.0f ? F32_MIN_TG : xdiv(xsub(mny, oy), dy);
    const float v0z = dz == 0.0f ? F32_MIN_TG : xdiv(xsub(mnz, oz), dz);
    const float v1x = dx == 0.0f ? F32_MAX_TG : xdiv(xsub(mxx, ox), dx);
    const float v1y = dy == 0.0f ? F32_MAX_TG : xdiv(xsub(mxy, oy), dy);
    const float v1z = dz == 0.0f ? F32_MAX_TG : xdiv(xsub(mxz, oz), dz);
    const float nx = gmin(v0x, v1x), ny = gmin(v0y, v1y), nz = gmin(v0z, v1z);
    const float fx = gmax(v0x, v1x), fy = gmax(v0y, v1y), fz = gmax(v0z, v1z);
    enter = gmax(gmax(nx, ny), nz);
    exit_ = gmin(gmin(fx, fy), fz);
    return exit_ > 0.0f && enter <= exit_;
}

// Per-view constants uploaded with each render.
struct ViewConst
{
    float cam[3];
    float bl[3], br[3], tr[3], tl[3];
    float far_plane;
    uint32_t width, height;
    uint32_t tile_w, tile_h;   // tile size in pixels
    uint32_t tiles_x, tiles_y;
    uint32_t tile_base;        // first global tile index of this view
    // conservative projection: world offset p -> (s, s*fx, s*fy) = inv_basis * p
    float inv_basis[9];        // row-major
    float fwd[3];              // unit view axis
    float planes[12];          // inward unit normals of the 4 side planes of the frustum
};

void trace_begin(tgx_ctx* ctx, int slot);
void trace_end(tgx_ctx* ctx, int slot);
void trace_free(tgx_ctx* ctx);

// Launch a kernel on the context stream, optionally bracketed by trace events.
#define TGX_LAUNCH(ctx, slot, grid, block, smem, kernel, ...)                      \
    do {                                                                          \
        trace_begin((ctx), (slot));                                               \
        kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);          \
        cudaError_t le_ = cudaGetLastError();                                     \
        trace_end((ctx), (slot));                                                 \
        if (le_ != cudaSuccess) {                                                 \
            tgx_set_error("launch of %s failed: %s", #kernel, cudaGetErrorString(le_)); \
            return TGX_ERR_CUDA;                                                  \
        }                                                                         \
        (ctx)->launches++;                                                        \
    } while (0)

// The same launch as a programmatic dependent of the stream's previous
// kernel: its CTAs may be scheduled while that kernel drains, and each waits
// in pdl_wait() until the previous kernel has completed and its writes are
// visible.  Every kernel launched this way calls pdl_wait() before its first
// access to global memory that an earlier kernel of the stream touches.
#define TGX_LAUNCH_PDL(ctx, slot, grid, block, smem, kernel, ...)                  \
    do {                                                                          \
        trace_begin((ctx), (slot));                                               \
        cudaLaunchConfig_t cfg_ = {};                                             \
        cfg_.gridDim = dim3(grid);                                                \
        cfg_.blockDim = dim3(block);                                              \
        cfg_.dynamicSmemBytes = (smem);                                           \
        cfg_.stream = (ctx)->stream;                                              \
        cudaLaunchAttribute attr_[1];                                             \
        attr_[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;         \
        attr_[0].val.programmaticStreamSerializationAllowed = 1;                  \
        cfg_.attrs = attr_;                                                       \
        cfg_.numAttrs = 1;                                                        \
        cudaError_t le_ = cudaLaunchKernelEx(&cfg_, kernel, __VA_ARGS__);         \
        trace_end((ctx), (slot));                                                 \
        if (le_ != cudaSuccess) {                                                 \
            tgx_set_error("launch of %s failed: %s", #kernel, cudaGetErrorString(le_)); \
            return TGX_ERR_CUDA;                                                  \
        }                                                                         \
        (ctx)->launches++;                                                        \
    } while (0)

// griddepcontrol (PTX ISA 7.8, sm_90+): a kernel's wait for the kernel it
// depends on, and its signal that its dependents may be scheduled.  Both are
// no-ops in a kernel launched without the programmatic attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Bounded wait for phase `parity` of the mbarrier at shared address `bar`:
// true once the phase has completed, false when about `limit_ns` nanoseconds
// of the GPU's global timer went by first.  The timer is read only when the
// first test fails, so a wait that is already over costs one instruction.
constexpr unsigned long long kMbarWaitNs = 1000000000ull;   // one second
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity,
                                                  unsigned long long limit_ns = kMbarWaitNs)
{
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
    unsigned long long t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    for (;;) {
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > limit_ns) return false;
    }
}

// cache inference over min(max_n, *d_n) inputs (mlp.cu)
tgx_status cache_primary(tgx_ctx* c, tgx_cache* k, tgx_cache** out);
tgx_status cache_train_pair(tgx_ctx* c, tgx_cache* const* k, const uint32_t* n, const float* const* d_x,
                            const float* const* d_t, uint32_t n_nets, float lr);
tgx_status cache_infer_counted(tgx_ctx* c, tgx_cache* k, const uint32_t* d_n, uint32_t max_n, const float* d_x,
                               float* d_rgb);

tgx_status vis_prepare_device(tgx_ctx* c);
// cudaMalloc of one scene-store array, counted against the context's budget
cudaError_t scene_malloc(tgx_ctx* c, tgx_scene* s, void** p, size_t bytes);
// host_out: some outputs are pinned host memory the tile kernel writes directly
tgx_status vis_render_device(tgx_ctx* ctx, const tgx_scene* scene, const tgx_view* views, uint32_t n_views,
                             uint64_t* const* d_visbuf, bool host_out = false);
