// mlp.cu -- the learned radiance cache: a small MLP on the tensor cores.
//
// New functionality (the reference has no learned component).  The network
// and its loss are defined by the FP64 oracle (oracle/oracle_mlp.c):
//   9 inputs (position normalised to [0,1]^3, normal, direction) ->
//   216 sin/cos features (12 octaves of pi) -> 4 ReLU layers of 64 -> RGB,
//   no biases, relative L2 loss, Adam.
// Weights and activations are BF16, accumulation is FP32, master weights and
// Adam moments are FP32.  Inference and training run on tcgen05 (operands in
// shared memory, FP32 accumulators in TMEM).
//
// Kernels:
//   k_mlp_forward_tc inference: 128 queries per tile, one elected thread
//                   issues the MMAs of a layer (below).
//   k_mlp_train_tc  training: forward, relative-L2 output delta, backward and
//                   the weight gradients of 128-sample tiles in one kernel;
//                   gradients summed in TMEM over a CTA's tiles, then written
//                   to the CTA's slice of a partial buffer, its loss beside
//                   them.
//   k_mlp_adam      sums the slices in a fixed order (deterministic), then
//                   Adam on the FP32 master weights; refreshes the BF16
//                   image the kernels stage from; sums the CTAs' losses.
//   k_mlp_reduce    the same sums into the gradient and the loss, for
//                   tgx_cache_gradient.
// A training step's two launches are programmatic dependents of the kernel
// before them (the step's inputs, or the previous step's Adam), so each
// launch overlaps the previous kernel's drain.

#include "tgx_internal.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <vector>

namespace {

constexpr int NI = 9, NE = 216, NEP = 224, NH = 64, NO = 3;
constexpr int OFF_W0 = 0, OFF_W1 = OFF_W0 + NH * NE, OFF_W2 = OFF_W1 + NH * NH, OFF_W3 = OFF_W2 + NH * NH,
              OFF_W4 = OFF_W3 + NH * NH, N_PARAMS = OFF_W4 + NO * NH;

// BF16 weight image, row-major [out][in] per layer (row strides padded)
constexpr int S0 = 232;   // W0  [64][S0]   k < 216 real
constexpr int SH = 72;    // W1..W3 [64][SH]
// offsets in bf16 elements inside the packed image
constexpr int B_W0 = 0;
constexpr int B_W1 = B_W0 + NH * S0;
constexpr int B_W2 = B_W1 + NH * SH;
constexpr int B_W3 = B_W2 + NH * SH;
constexpr int B_W4 = B_W3 + NH * SH;         // [8][SH], rows >= 3 zero
constexpr int B_TOTAL = B_W4 + 8 * SH;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05, accumulators in TMEM)
// ---------------------------------------------------------------------------
//
// A CTA of 384 threads holds three independent groups of 4 warps that share
// the weights in shared memory.  Each group works through tiles of 128 queries:
// thread t of the group owns query t of its tile, which is row t of every
// GEMM and TMEM lane t.  While one group waits for its MMAs the others encode
// or drain their accumulators, so the tensor core and the CUDA cores overlap.
// A group's layer-0 feature tile (56 KB) also holds, in its first 16 KB, the
// A operand of layers 1-4, which is written only once layer 0's MMAs have
// completed; that is what leaves room for a third group.
// Operands use the canonical no-swizzle K-major layout: 8 x 8 BF16 core
// matrices (8 rows of 16 contiguous bytes), K-adjacent core matrices LBO
// bytes apart and row-group-adjacent ones SBO bytes apart.  Per layer one
// thread of the group issues tcgen05.mma (M = 128, N = 64 or 16, K = 16 per
// instruction) into the group's 64 TMEM columns and commits to the group's
// mbarrier; then each warp reads its 32 TMEM lanes with tcgen05.ld, applies
// ReLU and writes the next layer's A operand.

namespace tc {

constexpr int M = 128;                      // queries per tile
constexpr int KG0 = NEP / 8;                // 28 K core-matrix columns of layer 0
constexpr int KGH = NH / 8;                 // 8 of the hidden layers
constexpr int NG = 3;                       // query groups per CTA
constexpr int THREADS = 128 * NG;           // three groups of 128
// byte offsets in dynamic shared memory (all 1024-aligned)
constexpr int W0 = 0;                                   // [28 kg][8 ng][128 B]
constexpr int W1 = W0 + KG0 * 8 * 128;                  // [8 kg][8 ng][128 B] x 3
constexpr int W4 = W1 + 3 * KGH * 8 * 128;              // [8 kg][2 ng][128 B] (16 rows, 3 real)
constexpr int GROUP = W4 + KGH * 2 * 128;               // per group:
constexpr int A0 = 0;                                   //   [28 kg][16 mg][128 B] layer 0's A operand
constexpr int A1 = A0;                                  //   [8 kg][16 mg][128 B] layers 1-4's A operand, in
                                                        //   A0's first 16 KB: written only after layer 0's
                                                        //   MMAs completed, and A0 again only after layer 4's
constexpr int GROUP_BYTES = KG0 * 16 * 128;
constexpr int BAR = GROUP + NG * GROUP_BYTES;           // NG mbarriers, TMEM address
constexpr int SMEM = BAR + 64;
static_assert(SMEM <= 232448, "shared memory per CTA");
constexpr uint32_t TMEM_COLS = 256;                     // 64 per group, allocated as a power of two

// instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major
__host__ __device__ constexpr uint32_t idesc(uint32_t n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// shared-memory matrix descriptor, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(id), "r"(acc) : "memory");
}

__device__ __forceinline__ void commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

// bounded wait for mbarrier phase `parity` (about a second); false when the limit ran out
__device__ __forceinline__ bool wait(uint32_t bar, uint32_t parity) { return mbar_wait_bounded(bar, parity); }

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// barrier of the 128 threads of one group (ids 1 and 2)
__device__ __forceinline__ void group_sync(uint32_t g) { asm volatile("bar.sync %0, 128;" :: "r"(g + 1u) : "memory"); }
// the same barrier, returning whether any thread of the group passed pred = true
__device__ __forceinline__ bool group_sync_or(uint32_t g, bool pred)
{
    uint32_t r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, 128, p;\n selp.u32 %0, 1, 0, q;\n}"
                 : "=r"(r) : "r"((uint32_t)pred), "r"(g + 1u) : "memory");
    return r != 0;
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// row `row` of an A tile: the 8 BF16 values of core-matrix column kg
__device__ __forceinline__ void put8(unsigned char* a, int kg, int row, const float* v)
{
    uint4 q;
    q.x = pack_bf16(v[0], v[1]); q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]); q.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(a + kg * (16 * 128) + (row >> 3) * 128 + (row & 7) * 16) = q;
}

// copies rows [0, n_rows) of a BF16 image matrix ([row][stride], K real columns
// padded to kgs * 8) into the core-matrix layout [kg][row / 8][128 B]; rows up
// to pad_rows are zero
__device__ __forceinline__ void stage_weights(unsigned char* dst, const __nv_bfloat16* src, int stride, int n_rows,
                                              int pad_rows, int kgs)
{
    const int ngs = pad_rows / 8;
    for (int e = threadIdx.x; e < pad_rows * kgs; e += blockDim.x) {
        const int row = e % pad_rows, kg = e / pad_rows;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (row < n_rows) v = *reinterpret_cast<const uint4*>(src + (size_t)row * stride + kg * 8);
        *reinterpret_cast<uint4*>(dst + kg * (ngs * 128) + (row >> 3) * 128 + (row & 7) * 16) = v;
    }
}

// The 24 features of one input (sin, cos of 2^k pi x for k = 0..11) into core
// columns 3i .. 3i+2 of the A tile.  sincospif anchors octaves 0 and 6; the
// others follow by angle doubling (sin 2a = 2 sin a cos a, cos 2a =
// (cos a - sin a)(cos a + sin a)), whose error (a few ulp times 2^5) stays far
// below the BF16 rounding of the features.
__device__ __forceinline__ void encode_input(unsigned char* a, int i, int row, float x)
{
    float f[24];
#pragma unroll
    for (int half = 0; half < 2; half++) {
        float sv, cv;
        sincospif(half ? x * 64.0f : x, &sv, &cv);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            f[(half * 6 + k) * 2 + 0] = sv;
            f[(half * 6 + k) * 2 + 1] = cv;
            const float s2 = 2.0f * sv * cv, c2 = (cv - sv) * (cv + sv);
            sv = s2;
            cv = c2;
        }
    }
    put8(a, 3 * i + 0, row, f);
    put8(a, 3 * i + 1, row, f + 8);
    put8(a, 3 * i + 2, row, f + 16);
}

}  // namespace tc

__global__ void __launch_bounds__(tc::THREADS, 1) k_mlp_forward_tc(const __nv_bfloat16* __restrict__ wimg, uint32_t n,
                                                                  const uint32_t* __restrict__ n_dev,
                                                                  const float* __restrict__ x, float* __restrict__ y,
                                                                  tgx_dev_status* __restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    using namespace tc;
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t g = warp >> 2, gt = tid & 127u;         // group, thread (= tile row) in the group
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + BAR);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + BAR + 16);
    unsigned char* ga = sm + GROUP + g * GROUP_BYTES;
    if (n_dev) n = min(n, *n_dev);
    stage_weights(sm + W0, wimg + B_W0, S0, NH, NH, KG0);
    stage_weights(sm + W1 + 0 * KGH * 8 * 128, wimg + B_W1, SH, NH, NH, KGH);
    stage_weights(sm + W1 + 1 * KGH * 8 * 128, wimg + B_W2, SH, NH, NH, KGH);
    stage_weights(sm + W1 + 2 * KGH * 8 * 128, wimg + B_W3, SH, NH, NH, KGH);
    stage_weights(sm + W4, wimg + B_W4, SH, 8, 16, KGH);
    if (tid == 0) {
        for (int q = 0; q < NG; q++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&bars[q])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(saddr(tmem_slot)), "r"(TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot + g * 64u;                          // this group's 64 columns
    const uint32_t lanes = tmem + (((warp & 3u) * 32u) << 16);           // this warp's 32 lanes
    const uint32_t b = saddr(&bars[g]);
    uint32_t phase = 0;
    bool ok = true;
    const uint32_t tiles = (n + M - 1) / M;
    // this thread's query of the group's next tile, loaded one tile ahead so
    // its HBM latency hides behind the current tile's layers
    float xn[NI];
    {
        const uint32_t row = (blockIdx.x * NG + g) * M + gt;
#pragma unroll
        for (int i = 0; i < NI; i++) xn[i] = row < n ? __ldg(&x[(uint64_t)row * NI + i]) : 0.0f;
    }
    for (uint32_t tile = blockIdx.x * NG + g; tile < tiles && ok; tile += gridDim.x * NG) {
        const uint32_t row = tile * M + gt;
        float xc[NI];
#pragma unroll
        for (int i = 0; i < NI; i++) xc[i] = xn[i];
        {
            const uint32_t next = (tile + gridDim.x * NG) * M + gt;
#pragma unroll
            for (int i = 0; i < NI; i++) xn[i] = next < n ? __ldg(&x[(uint64_t)next * NI + i]) : 0.0f;
        }
#pragma unroll
        for (int i = 0; i < NI; i++) encode_input(ga + A0, i, (int)gt, xc[i]);
        {
            const float z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            put8(ga + A0, KG0 - 1, (int)gt, z);   // features 216..223
        }
        fence_async_smem();
        fence_before();
        group_sync(g);
        // five layers; the hidden ones write the next A operand into A1
        for (int l = 0; l < 5 && ok; l++) {
            if (gt == 0) {
                fence_after();
                const int kgs = l == 0 ? KG0 : KGH;
                const uint32_t a_base = saddr(ga + (l == 0 ? A0 : A1));
                const uint32_t w_base = saddr(sm + (l == 0 ? W0 : l < 4 ? W1 + (l - 1) * KGH * 8 * 128 : W4));
                const uint32_t n_out = l < 4 ? 64u : 16u;
                const uint32_t w_sbo = 128, w_lbo = (n_out / 8) * 128;
                for (int k = 0; k < kgs / 2; k++)
                    mma(tmem, sdesc(a_base + 2 * k * (16 * 128), 16 * 128, 128),
                        sdesc(w_base + 2 * k * w_lbo, w_lbo, w_sbo), idesc(n_out), k > 0);
                commit(b);
            }
            // every thread of the group waits; one that gives up stops the group
            if (group_sync_or(g, !wait(b, phase))) {
                if (gt == 0) dev_error(status, TGX_ERR_TIMEOUT, 40 + l, tile);
                ok = false;
                break;
            }
            phase ^= 1u;
            fence_after();
            if (l < 4) {
                // the 64 accumulator columns in one TMEM round trip
                {
                    float v[64];
#pragma unroll
                    for (int q = 0; q < 4; q++) ld16(lanes + q * 16, v + 16 * q);
                    ld_wait();
#pragma unroll
                    for (int j = 0; j < 64; j++) v[j] = fmaxf(v[j], 0.0f);
#pragma unroll
                    for (int q = 0; q < 8; q++) put8(ga + A1, q, (int)gt, v + 8 * q);
                }
                fence_async_smem();
            } else {
                float v[16];
                ld16(lanes, v);
                ld_wait();
                if (row < n) {
                    y[(uint64_t)row * NO + 0] = v[0];
                    y[(uint64_t)row * NO + 1] = v[1];
                    y[(uint64_t)row * NO + 2] = v[2];
                }
            }
            fence_before();
            group_sync(g);
        }
    }
    if (!ok) wait(b, phase);   // let MMAs still in flight land (bounded) before the columns are freed
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(*tmem_slot), "r"(TMEM_COLS) : "memory");
}

// ---------------------------------------------------------------------------
// Training on tcgen05: forward, backward and weight gradients in one kernel
// ---------------------------------------------------------------------------
//
// One CTA of 128 * CS threads per SM works through tiles of 128 samples;
// thread t owns sample t mod 128 (row t mod 128 of the forward and backward
// GEMMs, TMEM lane t mod 128) and the 64 / CS accumulator columns of its
// part t / 128: the CS warps of a TMEM lane quarter split each epilogue and
// the feature encoding, so more warps hide each other's latency.  All
// operands stay in shared memory in the core-matrix layout the forward uses
// ([column group][row group][8 rows x 16 B]).  The backward reads the
// forward's weight tiles, and the weight gradients read the activation and
// delta tiles, through MN-major descriptors (the transpose bits of the
// instruction descriptor), so nothing is copied or transposed:
//   forward   z_{l+1} = W_l h_l (M = 128 samples), ReLU into BF16 tiles h1..h4
//   output    dy = d(relative L2)/dy, a 128 x 16 tile (3 real columns)
//   backward  d_l = (d_{l+1} W_l) * relu'(z_l), ping-ponging two tiles
//   gradients dW_l^T += h_l^T d_{l+1}: M = 128 layer inputs, N = outputs,
//             K = the tile's samples, accumulated in TMEM over all of the
//             CTA's tiles.  Layers with fewer than 128 inputs read the next
//             tile's rows as the rest of M; those accumulator rows are never
//             read out.
// At the end each CTA writes its summed gradient into its own slice of a
// partial buffer (and its share of the loss after the n_ctas slices), and
// k_mlp_reduce adds the slices in a fixed order, so a training step is
// deterministic.

namespace tt {

using tc::KG0;
using tc::KGH;
constexpr int CS = 2;                                 // threads per sample (column parts)
constexpr int CW = 64 / CS;                           // accumulator columns per thread
constexpr int THREADS = 128 * CS;
static_assert(CW % 16 == 0 && CW <= 32, "column parts");
constexpr int W0 = 0;                                 // [28 kg][8 ng][128 B]
constexpr int W1 = W0 + KG0 * 8 * 128;                // [8 kg][8 ng][128 B] x 3 (W1, W2, W3)
constexpr int W4 = W1 + 3 * KGH * 8 * 128;            // [8 kg][2 ng][128 B] (16 rows, 3 real)
constexpr int X0 = W4 + KGH * 2 * 128;                // features: [28 kg][16 mg][128 B]
constexpr int H = X0 + KG0 * 16 * 128;                // h1..h4: [8 kg][16 mg][128 B] each
constexpr int TILE64 = KGH * 16 * 128;
constexpr int DA = H + 4 * TILE64;                    // delta tiles (dy uses the first 2 kg of DB)
constexpr int DB = DA + TILE64;
constexpr int BAR = DB + TILE64;                      // mbarrier, TMEM address
constexpr int SMEM = BAR + 64;
// gradient reads of M = 128 rows run 16 column groups past a tile's base
static_assert(X0 + 32 * 16 * 128 <= SMEM && H + 3 * TILE64 + 16 * 16 * 128 <= SMEM, "gradient operand over-read");
// TMEM columns
constexpr uint32_t ACC = 0;        // layer accumulator (64 columns)
constexpr uint32_t G0A = 64;       // dW0^T inputs 0..127
constexpr uint32_t G0B = 128;      // dW0^T inputs 128..255 (216 real)
constexpr uint32_t G1 = 192, G2 = 256, G3 = 320;   // dW1^T .. dW3^T (64 real rows)
constexpr uint32_t G4 = 384;       // dW4^T (64 real rows, 16 columns, 3 real)
constexpr uint32_t TMEM_COLS = 512;

__host__ __device__ constexpr uint32_t idesc_t(uint32_t n, bool ta, bool tb)
{
    return tc::idesc(n) | (ta ? 1u << 15 : 0u) | (tb ? 1u << 16 : 0u);
}

}  // namespace tt

// One network's training batch in a launch that may carry two networks
// (the cache's two networks train side by side): CTAs first_cta ..
// first_cta + n_ctas - 1 of the grid work on it.
struct TrainJob
{
    const __nv_bfloat16* wimg;
    const float* x;
    const float* target;
    float* partial;              // n_ctas gradient slices, then n_ctas losses
    uint32_t n, first_cta, n_ctas;
};
struct TrainJobs
{
    TrainJob j[2];
};

__global__ void __launch_bounds__(tt::THREADS, 1) k_mlp_train_tc(TrainJobs jobs, tgx_dev_status* __restrict__ status)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    using namespace tc;
    const bool second = blockIdx.x >= jobs.j[1].first_cta;   // field by field: no local copy of the table
    const __nv_bfloat16* wimg = second ? jobs.j[1].wimg : jobs.j[0].wimg;
    const float* x = second ? jobs.j[1].x : jobs.j[0].x;
    const float* target = second ? jobs.j[1].target : jobs.j[0].target;
    float* partial = second ? jobs.j[1].partial : jobs.j[0].partial;
    const uint32_t n = second ? jobs.j[1].n : jobs.j[0].n;
    const uint32_t cta = blockIdx.x - (second ? jobs.j[1].first_cta : jobs.j[0].first_cta);
    const uint32_t n_ctas = second ? jobs.j[1].n_ctas : jobs.j[0].n_ctas;
    const uint32_t t = threadIdx.x, warp = t >> 5;
    const uint32_t r = t & 127u;                 // the thread's sample row of a tile and TMEM lane
    const uint32_t part = t >> 7;                // its accumulator columns [part * CW, part * CW + CW)
    constexpr int CW = tt::CW;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + tt::BAR);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + tt::BAR + 16);
    float* warp_loss = reinterpret_cast<float*>(sm + tt::BAR + 32);   // the 4 sample warps' loss sums
    pdl_wait();      // the weight image and the batch come from earlier kernels of the stream
    pdl_trigger();
    stage_weights(sm + tt::W0, wimg + B_W0, S0, NH, NH, KG0);
    stage_weights(sm + tt::W1 + 0 * KGH * 8 * 128, wimg + B_W1, SH, NH, NH, KGH);
    stage_weights(sm + tt::W1 + 1 * KGH * 8 * 128, wimg + B_W2, SH, NH, NH, KGH);
    stage_weights(sm + tt::W1 + 2 * KGH * 8 * 128, wimg + B_W3, SH, NH, NH, KGH);
    stage_weights(sm + tt::W4, wimg + B_W4, SH, 8, 16, KGH);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(saddr(tmem_slot)), "r"(tt::TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lanes = tmem + (((warp & 3u) * 32u) << 16);   // this warp's 32 lanes
    const uint32_t cols = part * (uint32_t)CW;                    // its first accumulator column
    const uint32_t b = saddr(bar);
    const uint32_t x0 = saddr(sm + tt::X0), hb = saddr(sm + tt::H), da = saddr(sm + tt::DA), db = saddr(sm + tt::DB);
    const uint32_t w0 = saddr(sm + tt::W0), w1 = saddr(sm + tt::W1), w4 = saddr(sm + tt::W4);
    uint32_t phase = 0;
    bool ok = true;
    const float inv = 1.0f / (3.0f * (float)n);
    float lsum = 0.0f;
    const uint32_t tiles = (n + 127) / 128;
    uint32_t acc_g = 0;   // gradient accumulators hold a previous tile's sums
    // all threads wait for the MMAs of one commit; any thread that gives up stops the CTA
    auto sync_mma = [&](int where, uint32_t tile) -> bool {
        const bool late = !wait(b, phase);
        if (__syncthreads_or(late)) {
            if (t == 0) dev_error(status, TGX_ERR_TIMEOUT, where, tile);
            return false;   // phase stays on the commit still in flight
        }
        phase ^= 1u;
        fence_after();
        return true;
    };
    auto publish = [&]() {   // this thread's shared-memory writes, visible to the tensor core
        fence_async_smem();
        fence_before();
        __syncthreads();
    };
    for (uint32_t tile = cta; tile < tiles && ok; tile += n_ctas) {
        const uint32_t row = tile * 128 + r;
        const bool valid = row < n;
        for (int i = (int)part; i < NI; i += tt::CS)
            encode_input(sm + tt::X0, i, (int)r, valid ? x[(uint64_t)row * NI + i] : 0.0f);
        if (part == tt::CS - 1) {
            const float z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            put8(sm + tt::X0, KG0 - 1, (int)r, z);   // features 216..223
        }
        // ---- forward ----
        uint32_t mask[4];   // relu'(z) of the thread's columns per hidden layer
        float y[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int l = 0; l < 5 && ok; l++) {
            publish();
            if (t == 0) {
                fence_after();
                if (l == 0) {
                    for (int k = 0; k < KG0 / 2; k++)
                        mma(tmem + tt::ACC, sdesc(x0 + 2 * k * 2048, 2048, 128), sdesc(w0 + 2 * k * 1024, 1024, 128),
                            idesc(64), k > 0);
                } else if (l < 4) {
                    const uint32_t a = hb + (l - 1) * tt::TILE64, w = w1 + (l - 1) * KGH * 8 * 128;
                    for (int k = 0; k < KGH / 2; k++)
                        mma(tmem + tt::ACC, sdesc(a + 2 * k * 2048, 2048, 128), sdesc(w + 2 * k * 1024, 1024, 128),
                            idesc(64), k > 0);
                } else {
                    const uint32_t a = hb + 3 * tt::TILE64;
                    for (int k = 0; k < KGH / 2; k++)
                        mma(tmem + tt::ACC, sdesc(a + 2 * k * 2048, 2048, 128), sdesc(w4 + 2 * k * 256, 256, 128),
                            idesc(16), k > 0);
                }
                commit(b);
            }
            if (!(ok = sync_mma(50 + l, tile))) break;
            if (l < 4) {
                // the thread's accumulator columns in one TMEM round trip
                unsigned char* h = sm + tt::H + l * tt::TILE64;
                float v[CW];
#pragma unroll
                for (int q = 0; q < CW / 16; q++) ld16(lanes + tt::ACC + cols + q * 16, v + 16 * q);
                ld_wait();
                mask[l] = 0u;
#pragma unroll
                for (int j = 0; j < CW; j++) {
                    v[j] = fmaxf(v[j], 0.0f);
                    if (v[j] > 0.0f) mask[l] |= 1u << j;
                }
#pragma unroll
                for (int q = 0; q < CW / 8; q++) put8(h, (int)(cols / 8) + q, (int)r, v + 8 * q);
            } else if (part == 0) {
                float v[16];
                ld16(lanes + tt::ACC, v);
                ld_wait();
                y[0] = v[0]; y[1] = v[1]; y[2] = v[2];
            }
        }
        if (!ok) break;
        // ---- output delta (relative L2), into DB ----
        if (part == 0) {
            float d[16];
#pragma unroll
            for (int j = 0; j < 16; j++) d[j] = 0.0f;
            if (valid) {
#pragma unroll
                for (int c = 0; c < NO; c++) {
                    const float tv = target[(uint64_t)row * NO + c];
                    const float den = y[c] * y[c] + 0.01f;
                    const float res = y[c] - tv;
                    lsum += res * res / den;
                    d[c] = 2.0f * res / den * inv;
                }
            }
            put8(sm + tt::DB, 0, (int)r, d);
            put8(sm + tt::DB, 1, (int)r, d + 8);
        }
        // ---- backward: stage s propagates through W_{4-s} and accumulates its gradient ----
#pragma unroll
        for (int s = 0; s < 5 && ok; s++) {
            publish();
            const uint32_t din = (s & 1) ? da : db;        // delta at the output of the layer
            if (t == 0) {
                fence_after();
                const int l = 4 - s;                       // weight layer
                if (s < 4) {
                    // next delta (pre-mask) = din * W_l: B = W_l read MN-major (N = inputs, K = outputs)
                    if (l == 4) {
                        mma(tmem + tt::ACC, sdesc(din, 2048, 128), sdesc(w4, 128, 256), tt::idesc_t(64, false, true), 0u);
                    } else {
                        const uint32_t w = w1 + (l - 1) * KGH * 8 * 128;
                        for (int k = 0; k < KGH / 2; k++)
                            mma(tmem + tt::ACC, sdesc(din + 2 * k * 2048, 2048, 128), sdesc(w + 2 * k * 128, 128, 1024),
                                tt::idesc_t(64, false, true), k > 0);
                    }
                }
                // dW_l^T += input_l^T din: A = the layer's input tile, B = din, both MN-major, K = samples
                const uint32_t nout = l == 4 ? 16u : 64u;
                const uint32_t gcol = l == 4 ? tt::G4 : l == 3 ? tt::G3 : l == 2 ? tt::G2 : l == 1 ? tt::G1 : tt::G0A;
                const uint32_t ain = l == 0 ? x0 : hb + (l - 1) * tt::TILE64;
                const int parts = l == 0 ? 2 : 1;
                for (int part = 0; part < parts; part++)
                    for (int k = 0; k < 8; k++)
                        mma(tmem + gcol + part * 64u, sdesc(ain + part * 16 * 2048 + 2 * k * 128, 128, 2048),
                            sdesc(din + 2 * k * 128, 128, 2048), tt::idesc_t(nout, true, true), (acc_g | k) ? 1u : 0u);
                commit(b);
            }
            if (!(ok = sync_mma(60 + s, tile))) break;
            if (s == 4) break;
            // mask with relu'(z) of the layer's input and store the next delta into the other tile
            const int ml = 3 - s;                           // h_{ml+1} = input of W_{4-s}
            unsigned char* dout = sm + ((s & 1) ? tt::DB : tt::DA);
            float v[CW];
#pragma unroll
            for (int q = 0; q < CW / 16; q++) ld16(lanes + tt::ACC + cols + q * 16, v + 16 * q);
            ld_wait();
#pragma unroll
            for (int j = 0; j < CW; j++) v[j] = ((mask[ml] >> j) & 1u) && valid ? v[j] : 0.0f;
#pragma unroll
            for (int q = 0; q < CW / 8; q++) put8(dout, (int)(cols / 8) + q, (int)r, v + 8 * q);
        }
        acc_g = 1u;
    }
    // ---- this CTA's gradient sums into its slice of the partial buffer ----
    fence_before();
    __syncthreads();
    fence_after();
    float* P = partial + (uint64_t)cta * N_PARAMS;
    {
#pragma unroll 1
        for (int blk = 0; blk < 5; blk++) {
            const uint32_t col = blk == 0 ? tt::G0A : blk == 1 ? tt::G0B : blk == 2 ? tt::G1 : blk == 3 ? tt::G2 : tt::G3;
            const int i = (blk == 1 ? 128 : 0) + (int)r;                  // layer input (TMEM row)
            const int ni = blk < 2 ? NE : NH;
            const int off = blk < 2 ? OFF_W0 : blk == 2 ? OFF_W1 : blk == 3 ? OFF_W2 : OFF_W3;
            // the thread's columns of the block in one TMEM round trip
            float v[CW];
#pragma unroll
            for (int q = 0; q < CW / 16; q++) ld16(lanes + col + cols + q * 16, v + 16 * q);
            ld_wait();
            if (i < ni) {
#pragma unroll
                for (int j = 0; j < CW; j++) P[off + ((int)cols + j) * ni + i] = ok && acc_g ? v[j] : 0.0f;
            }
        }
        if (part == 0) {   // dW4^T: 3 real columns
            float v[16];
            ld16(lanes + tt::G4, v);
            ld_wait();
            const int i = (int)r;
            if (i < NH) {
#pragma unroll
                for (int j = 0; j < NO; j++) P[OFF_W4 + j * NH + i] = ok && acc_g ? v[j] : 0.0f;
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((t & 31) == 0 && part == 0) warp_loss[warp] = lsum;
    if (!ok) wait(b, phase);   // let MMAs still in flight land (bounded) before the columns are freed
    fence_before();
    __syncthreads();
    fence_after();
    if (t == 0)   // this CTA's share of the loss, after the n_ctas gradient slices
        partial[(uint64_t)n_ctas * N_PARAMS + cta] = (((warp_loss[0] + warp_loss[1]) + warp_loss[2]) + warp_loss[3]) * inv;
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(tt::TMEM_COLS) : "memory");
}

// Sum of the CTAs' gradient slices of parameter p in a fixed order: eight
// running sums over the slices c = j mod 8 of the first 8 * floor(n / 8)
// (eight loads in flight instead of one chain), added 0 + 1 + ... + 7, then
// the rest in order.  Deterministic; k_mlp_reduce and k_mlp_adam share it,
// so both see the same gradient bits.
__device__ __forceinline__ float sum_slices(const float* __restrict__ partial, uint32_t n_parts, int p)
{
    float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t c = 0;
    // 32 loads in flight, then the same additions in the same order as the 8-wide loop below
    for (; c + 32 <= n_parts; c += 32) {
        float x[32];
#pragma unroll
        for (int j = 0; j < 32; j++) x[j] = partial[(uint64_t)(c + j) * N_PARAMS + p];
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int j = 0; j < 8; j++) acc[j] += x[8 * q + j];
    }
    for (; c + 8 <= n_parts; c += 8) {
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = partial[(uint64_t)(c + j) * N_PARAMS + p];
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] += x[j];
    }
    float tail = 0.0f;   // the last n_parts mod 8 slices
    for (; c < n_parts; c++) tail += partial[(uint64_t)c * N_PARAMS + p];
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j++) s += acc[j];
    return s + tail;
}

// The CTAs' losses (after the n_parts gradient slices), added in CTA order.
__device__ __forceinline__ float sum_losses(const float* __restrict__ partial, uint32_t n_parts)
{
    float l = 0.0f;
    for (uint32_t c = 0; c < n_parts; c++) l += partial[(uint64_t)n_parts * N_PARAMS + c];
    return l;
}

// The slices' sum added to the gradient; the loss.
__global__ void __launch_bounds__(256) k_mlp_reduce(const float* __restrict__ partial, uint32_t n_parts,
                                                   float* __restrict__ g, float* __restrict__ loss)
{
    pdl_wait();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) *loss = sum_losses(partial, n_parts);
    if (p >= N_PARAMS) return;
    g[p] += sum_slices(partial, n_parts, p);
}

// bf16 image position of master parameter p
__device__ __forceinline__ int image_pos(int p)
{
    if (p < OFF_W1) return B_W0 + (p / NE) * S0 + p % NE;
    if (p < OFF_W4) {
        const int l = (p - OFF_W1) / (NH * NH), r = (p - OFF_W1) % (NH * NH);
        return B_W1 + l * NH * SH + (r / NH) * SH + r % NH;
    }
    const int r = p - OFF_W4;
    return B_W4 + (r / NH) * SH + r % NH;
}

// Adam for up to two networks (blockIdx.y).  The gradient is g plus the
// n_parts slices of `partial` (the training kernel's per-CTA sums) added as
// k_mlp_reduce adds them (sum_slices).
struct AdamJob
{
    float* w;
    float* m;
    float* v;
    float* g;
    const float* partial;
    __nv_bfloat16* img;
    float* loss;
    uint32_t n_parts;
    float c1, c2;
};
struct AdamJobs
{
    AdamJob j[2];
};

__global__ void __launch_bounds__(256) k_mlp_adam(AdamJobs jobs, float lr, float b1, float b2, float eps)
{
    pdl_wait();      // the training kernel's slices
    pdl_trigger();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const AdamJob& J = jobs.j[0];
    const AdamJob& K = jobs.j[1];
    const bool second = blockIdx.y != 0;
    float* w = second ? K.w : J.w;
    float* m = second ? K.m : J.m;
    float* v = second ? K.v : J.v;
    float* g = second ? K.g : J.g;
    const float* partial = second ? K.partial : J.partial;
    const uint32_t n_parts = second ? K.n_parts : J.n_parts;
    const float c1 = second ? K.c1 : J.c1, c2 = second ? K.c2 : J.c2;
    __nv_bfloat16* img = second ? K.img : J.img;
    if (p == 0) *(second ? K.loss : J.loss) = sum_losses(partial, n_parts);
    if (p >= N_PARAMS) return;
    const float gp = g[p] + sum_slices(partial, n_parts, p);
    g[p] = 0.0f;
    const float mp = b1 * m[p] + (1.0f - b1) * gp;
    const float vp = b2 * v[p] + (1.0f - b2) * gp * gp;
    m[p] = mp;
    v[p] = vp;
    const float wp = w[p] - lr * (mp / c1) / (sqrtf(vp / c2) + eps);
    w[p] = wp;
    img[image_pos(p)] = __float2bfloat16_rn(wp);
}

__global__ void k_mlp_image(const float* __restrict__ w, __nv_bfloat16* __restrict__ img)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N_PARAMS) return;
    img[image_pos(p)] = __float2bfloat16_rn(w[p]);
}

}  // namespace

struct tgx_cache
{
    float* w = nullptr;        // FP32 master weights [N_PARAMS]
    float* m = nullptr;
    float* v = nullptr;
    float* g = nullptr;        // gradient accumulator
    __nv_bfloat16* img = nullptr;
    float* loss = nullptr;
    uint32_t step = 0;
    uint64_t seed = 0;
    DevBuf scratch;            // training activations/deltas
    tgx_cache* primary = nullptr;  // second network: mean incoming light at pixel surface points (cached GI)
};

static uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

extern "C" uint32_t tgx_cache_n_params(void) { return N_PARAMS; }

static tgx_status cache_refresh_image(tgx_ctx* c, tgx_cache* k)
{
    TGX_LAUNCH(c, TR_MLP_ADAM, (N_PARAMS + 255) / 256, 256, 0, k_mlp_image, k->w, k->img);
    return TGX_OK;
}

extern "C" tgx_status tgx_cache_create(tgx_ctx* c, uint64_t seed, tgx_cache** out)
{
    if (!c || !out) return TGX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    TGX_CUDA(cudaSetDevice(c->device));
    tgx_cache* k = new (std::nothrow) tgx_cache();
    if (!k) return TGX_ERR_OUT_OF_MEMORY;
    k->seed = seed;
    bool ok = cudaMalloc(&k->w, N_PARAMS * 4) == cudaSuccess && cudaMalloc(&k->m, N_PARAMS * 4) == cudaSuccess &&
              cudaMalloc(&k->v, N_PARAMS * 4) == cudaSuccess && cudaMalloc(&k->g, N_PARAMS * 4) == cudaSuccess &&
              cudaMalloc(&k->img, B_TOTAL * 2) == cudaSuccess && cudaMalloc(&k->loss, 16) == cudaSuccess;
    if (!ok) {
        tgx_cache_destroy(c, k);
        tgx_set_error("tgx_cache_create: out of device memory");
        return TGX_ERR_OUT_OF_MEMORY;
    }
    // He-uniform initialisation from the seed (host side, deterministic)
    std::vector<float> w(N_PARAMS);
    for (int p = 0; p < N_PARAMS; p++) {
        const int fan = p < OFF_W1 ? NE : NH;
        const float u = (float)(mix64(seed * 0x9E3779B97F4A7C15ull + p) >> 40) * (1.0f / 16777216.0f);
        w[p] = (2.0f * u - 1.0f) * sqrtf(6.0f / (float)fan);
    }
    cudaMemsetAsync(k->m, 0, N_PARAMS * 4, c->stream);
    cudaMemsetAsync(k->v, 0, N_PARAMS * 4, c->stream);
    cudaMemsetAsync(k->g, 0, N_PARAMS * 4, c->stream);
    cudaMemsetAsync(k->img, 0, B_TOTAL * 2, c->stream);
    TGX_CUDA(cudaMemcpyAsync(k->w, w.data(), N_PARAMS * 4, cudaMemcpyHostToDevice, c->stream));
    tgx_status st = cache_refresh_image(c, k);
    if (st == TGX_OK) st = cudaStreamSynchronize(c->stream) == cudaSuccess ? TGX_OK : TGX_ERR_CUDA;
    if (st != TGX_OK) { tgx_cache_destroy(c, k); return st; }
    *out = k;
    return TGX_OK;
}

extern "C" void tgx_cache_destroy(tgx_ctx* c, tgx_cache* k)
{
    if (!k) return;
    if (c) cudaStreamSynchronize(c->stream);
    tgx_cache_destroy(c, k->primary);
    cudaFree(k->w); cudaFree(k->m); cudaFree(k->v); cudaFree(k->g); cudaFree(k->img); cudaFree(k->loss);
    devbuf_free(k->scratch);
    delete k;
}

// The cache's second network, created on first use from a seed derived from the cache's.
tgx_status cache_primary(tgx_ctx* c, tgx_cache* k, tgx_cache** out)
{
    if (!k->primary) TGX_TRY(tgx_cache_create(c, mix64(k->seed ^ 0x7072696d617279ull), &k->primary));
    *out = k->primary;
    return TGX_OK;
}

extern "C" tgx_status tgx_cache_get_weights(tgx_ctx* c, const tgx_cache* k, float* out_w)
{
    if (!c || !k || !out_w) return TGX_ERR_INVALID_ARGUMENT;
    TGX_CUDA(cudaMemcpyAsync(out_w, k->w, N_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

extern "C" tgx_status tgx_cache_set_weights(tgx_ctx* c, tgx_cache* k, const float* w)
{
    if (!c || !k || !w) return TGX_ERR_INVALID_ARGUMENT;
    TGX_CUDA(cudaMemcpyAsync(k->w, w, N_PARAMS * 4, cudaMemcpyHostToDevice, c->stream));
    TGX_TRY(cache_refresh_image(c, k));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

// inference of n queries (min(n, *d_n) when d_n is given) on the tcgen05 kernel
static tgx_status cache_forward(tgx_ctx* c, tgx_cache* k, const uint32_t* d_n, uint32_t n, const float* d_x,
                                float* d_rgb)
{
    static bool attr = false;
    if (!attr) {
        TGX_CUDA(cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM));
        attr = true;
    }
    const uint32_t tiles = (n + tc::M - 1) / tc::M;
    const uint32_t grid = std::max(1u, std::min<uint32_t>((tiles + tc::NG - 1) / tc::NG, (uint32_t)c->num_sms));
    TGX_LAUNCH(c, TR_MLP, grid, tc::THREADS, tc::SMEM, k_mlp_forward_tc, k->img, n, d_n, d_x, d_rgb, c->d_status);
    return TGX_OK;
}

extern "C" tgx_status tgx_cache_infer(tgx_ctx* c, tgx_cache* k, uint32_t n, const float* d_x, float* d_rgb)
{
    if (!c || !k || (n && (!d_x || !d_rgb))) return TGX_ERR_INVALID_ARGUMENT;
    if (!n) return TGX_OK;
    return cache_forward(c, k, nullptr, n, d_x, d_rgb);
}

tgx_status cache_infer_counted(tgx_ctx* c, tgx_cache* k, const uint32_t* d_n, uint32_t max_n, const float* d_x,
                               float* d_rgb)
{
    if (!max_n) return TGX_OK;
    return cache_forward(c, k, d_n, max_n, d_x, d_rgb);
}

// Computes the batch gradient into the accumulator (no update); returns the loss if out_loss.
// The fused training kernel over one network's n samples, or over two
// networks' batches side by side in one launch; leaves each network's per-CTA
// gradient slices in its scratch (parts[i] of them).
static tgx_status cache_grad_parts(tgx_ctx* c, tgx_cache* const* k, const uint32_t* n, const float* const* d_x,
                                   const float* const* d_t, uint32_t n_nets, uint32_t* parts)
{
    static bool attr = false;
    if (!attr) {
        TGX_CUDA(cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tt::SMEM));
        attr = true;
    }
    TrainJobs jobs;
    uint32_t grid = 0;
    // One wave of CTAs (one per SM: the kernel holds most of an SM's shared
    // memory) shared between the jobs in proportion to their 128-sample tiles,
    // so that every CTA loops over about as many tiles.
    const uint32_t sms = (uint32_t)c->num_sms;
    uint32_t total = 0;
    for (uint32_t i = 0; i < n_nets; i++) total += (n[i] + 127) / 128;
    for (uint32_t i = 0; i < 2; i++) {
        TrainJob& J = jobs.j[i];
        if (i >= n_nets) {   // an empty second job past the end of the grid
            J = jobs.j[0];
            J.first_cta = 0xffffffffu;
            continue;
        }
        const uint32_t tiles = (n[i] + 127) / 128;
        const uint32_t share = total <= sms ? tiles : (uint32_t)((uint64_t)tiles * sms / total);
        const uint32_t ctas = std::max(1u, std::min(tiles, share));
        TGX_TRY(devbuf_reserve(k[i]->scratch, (size_t)ctas * (N_PARAMS + 1) * 4));
        J.wimg = k[i]->img;
        J.x = d_x[i];
        J.target = d_t[i];
        J.partial = (float*)k[i]->scratch.ptr;
        J.n = n[i];
        J.first_cta = grid;
        J.n_ctas = ctas;
        parts[i] = ctas;
        grid += ctas;
    }
    TGX_LAUNCH_PDL(c, TR_MLP_FWD_BWD, grid, tt::THREADS, tt::SMEM, k_mlp_train_tc, jobs, c->d_status);
    return TGX_OK;
}

// ... and their sum added to the gradient
static tgx_status cache_grad(tgx_ctx* c, tgx_cache* k, uint32_t n, const float* d_x, const float* d_t)
{
    uint32_t parts = 0;
    TGX_TRY(cache_grad_parts(c, &k, &n, &d_x, &d_t, 1, &parts));
    TGX_LAUNCH(c, TR_MLP_WGRAD, (N_PARAMS + 255) / 256, 256, 0, k_mlp_reduce, (const float*)k->scratch.ptr, parts, k->g,
               k->loss);
    return TGX_OK;
}

extern "C" tgx_status tgx_cache_gradient(tgx_ctx* c, tgx_cache* k, uint32_t n, const float* d_x, const float* d_t,
                                         float* out_grad, float* out_loss)
{
    if (!c || !k || !n || !d_x || !d_t) return TGX_ERR_INVALID_ARGUMENT;
    TGX_CUDA(cudaMemsetAsync(k->g, 0, N_PARAMS * 4, c->stream));
    TGX_TRY(cache_grad(c, k, n, d_x, d_t));
    if (out_grad) TGX_CUDA(cudaMemcpyAsync(out_grad, k->g, N_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream));
    if (out_loss) TGX_CUDA(cudaMemcpyAsync(out_loss, k->loss, 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaMemsetAsync(k->g, 0, N_PARAMS * 4, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

// One Adam step of one network, or of two networks side by side (shared
// training and Adam launches); n[i] samples each.
tgx_status cache_train_pair(tgx_ctx* c, tgx_cache* const* k, const uint32_t* n, const float* const* d_x,
                            const float* const* d_t, uint32_t n_nets, float lr)
{
    uint32_t parts[2] = {0, 0};
    TGX_TRY(cache_grad_parts(c, k, n, d_x, d_t, n_nets, parts));
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-15f;
    AdamJobs jobs;
    for (uint32_t i = 0; i < n_nets; i++) {
        k[i]->step++;
        AdamJob& J = jobs.j[i];
        J.w = k[i]->w; J.m = k[i]->m; J.v = k[i]->v; J.g = k[i]->g;
        J.partial = (const float*)k[i]->scratch.ptr;
        J.img = k[i]->img;
        J.loss = k[i]->loss;
        J.n_parts = parts[i];
        J.c1 = (float)(1.0 - pow((double)b1, (double)k[i]->step));
        J.c2 = (float)(1.0 - pow((double)b2, (double)k[i]->step));
    }
    if (n_nets < 2) jobs.j[1] = jobs.j[0];
    TGX_LAUNCH_PDL(c, TR_MLP_ADAM, dim3((N_PARAMS + 255) / 256, n_nets), 256, 0, k_mlp_adam, jobs, lr, b1, b2, eps);
    return TGX_OK;
}

extern "C" tgx_status tgx_cache_train_step(tgx_ctx* c, tgx_cache* k, uint32_t n, const float* d_x, const float* d_t,
                                           float lr)
{
    if (!c || !k || !n || !d_x || !d_t) return TGX_ERR_INVALID_ARGUMENT;
    return cache_train_pair(c, &k, &n, &d_x, &d_t, 1, lr);
}

extern "C" tgx_status tgx_cache_last_loss(tgx_ctx* c, const tgx_cache* k, float* out_loss)
{
    if (!c || !k || !out_loss) return TGX_ERR_INVALID_ARGUMENT;
    TGX_CUDA(cudaMemcpyAsync(out_loss, k->loss, 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

// checkpoint: magic, step, weights, m, v
extern "C" tgx_status tgx_cache_save(tgx_ctx* c, const tgx_cache* k, const char* path)
{
    if (!c || !k || !path) return TGX_ERR_INVALID_ARGUMENT;
    std::vector<float> buf(3 * (size_t)N_PARAMS);
    TGX_CUDA(cudaMemcpyAsync(buf.data(), k->w, N_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaMemcpyAsync(buf.data() + N_PARAMS, k->m, N_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaMemcpyAsync(buf.data() + 2 * N_PARAMS, k->v, N_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    FILE* f = fopen(path, "wb");
    if (!f) { tgx_set_error("tgx_cache_save: cannot open %s", path); return TGX_ERR_INVALID_ARGUMENT; }
    const uint32_t hdr[4] = {0x43584754u /* "TGXC" */, 1u, (uint32_t)N_PARAMS, k->step};
    const bool ok = fwrite(hdr, sizeof(hdr), 1, f) == 1 && fwrite(buf.data(), 4, buf.size(), f) == buf.size();
    fclose(f);
    if (!ok) { tgx_set_error("tgx_cache_save: write failed"); return TGX_ERR_INVALID_ARGUMENT; }
    return TGX_OK;
}

extern "C" tgx_status tgx_cache_load(tgx_ctx* c, tgx_cache* k, const char* path)
{
    if (!c || !k || !path) return TGX_ERR_INVALID_ARGUMENT;
    FILE* f = fopen(path, "rb");
    if (!f) { tgx_set_error("tgx_cache_load: cannot open %s", path); return TGX_ERR_INVALID_ARGUMENT; }
    uint32_t hdr[4];
    std::vector<float> buf(3 * (size_t)N_PARAMS);
    const bool ok = fread(hdr, sizeof(hdr), 1, f) == 1 && hdr[0] == 0x43584754u && hdr[1] == 1u &&
                    hdr[2] == (uint32_t)N_PARAMS && fread(buf.data(), 4, buf.size(), f) == buf.size();
    fclose(f);
    if (!ok) { tgx_set_error("tgx_cache_load: %s is not a tgx cache checkpoint", path); return TGX_ERR_INVALID_ARGUMENT; }
    TGX_CUDA(cudaMemcpyAsync(k->w, buf.data(), N_PARAMS * 4, cudaMemcpyHostToDevice, c->stream));
    TGX_CUDA(cudaMemcpyAsync(k->m, buf.data() + N_PARAMS, N_PARAMS * 4, cudaMemcpyHostToDevice, c->stream));
    TGX_CUDA(cudaMemcpyAsync(k->v, buf.data() + 2 * N_PARAMS, N_PARAMS * 4, cudaMemcpyHostToDevice, c->stream));
    k->step = hdr[3];
    TGX_TRY(cache_refresh_image(c, k));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}
