// mlp.cu -- the learned radiance cache: a small MLP on the tensor cores.
//
// New functionality (the reference has no learned component).  The network
// and its loss are defined by the FP64 oracle (oracle/oracle_mlp.c):
//   9 inputs (position normalised to [0,1]^3, normal, direction) ->
//   216 sin/cos features (12 octaves of pi) -> 4 ReLU layers of 64 -> RGB,
//   no biases, relative L2 loss, Adam.
// Weights and activations are BF16, accumulation is FP32, master weights and
// Adam moments are FP32.  Inference runs on tcgen05 (TMEM accumulators);
// training on mma.sync m16n8k16.
//
// Kernels:
//   k_mlp_forward_tc inference on tcgen05: 128 queries per tile, operands in
//                   shared memory, FP32 accumulators in TMEM, one elected
//                   thread issues the MMAs of a layer (below).
//   k_mlp_fwd_bwd   one warp per 16 samples: the forward with the accumulators
//                   of one layer re-packed as the A fragments of the next, the
//                   relative-L2 gradient, and the
//                   backward pass through W4..W1 (deltas masked by ReLU');
//                   writes each layer's input activations and output deltas
//                   (BF16) for the weight gradients.
//   k_mlp_wgrad     dW_l = sum_s delta_l[s] (x) act_l[s] for all layers in one
//                   launch, on the tensor cores (ldmatrix.trans tiles of 16
//                   samples), split over samples, per-CTA sums in shared
//                   memory, FP32 atomics into the gradient.
//   k_mlp_adam      Adam on the FP32 master weights; refreshes the BF16
//                   copies in the layouts the kernels read (row-major for the
//                   forward, transposed for the backward).

#include "tgx_internal.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <cstdio>
#include <vector>

namespace {

constexpr int NI = 9, NF = 12, NE = 216, NEP = 224, NH = 64, NO = 3;
constexpr int OFF_W0 = 0, OFF_W1 = OFF_W0 + NH * NE, OFF_W2 = OFF_W1 + NH * NH, OFF_W3 = OFF_W2 + NH * NH,
              OFF_W4 = OFF_W3 + NH * NH, N_PARAMS = OFF_W4 + NO * NH;

// BF16 weight images (element strides padded against shared-memory bank conflicts)
constexpr int S0 = 232;   // W0  [64][S0]   k < 216 real
constexpr int SH = 72;    // W1..W3 [64][SH] and their transposes
constexpr int S4T = 24;   // W4t [64][S4T]  k < 3 real
// offsets in bf16 elements inside the packed image
constexpr int B_W0 = 0;
constexpr int B_W1 = B_W0 + NH * S0;
constexpr int B_W2 = B_W1 + NH * SH;
constexpr int B_W3 = B_W2 + NH * SH;
constexpr int B_W4 = B_W3 + NH * SH;         // [8][SH], rows >= 3 zero
constexpr int B_W1T = B_W4 + 8 * SH;
constexpr int B_W2T = B_W1T + NH * SH;
constexpr int B_W3T = B_W2T + NH * SH;
constexpr int B_W4T = B_W3T + NH * SH;       // [64][S4T], cols >= 3 zero
constexpr int B_TOTAL = B_W4T + NH * S4T;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// feature pair (sin, cos) of column c (even) for input row x
__device__ __forceinline__ uint32_t feature_pair(const float* x, int c)
{
    if (c >= NE) return 0u;
    const int i = c / (2 * NF), k = (c / 2) % NF;
    float s, co;
    sincospif(ldexpf(x[i], k), &s, &co);
    return pack_bf16(s, co);
}

// One hidden layer: acc[8][4] = A(16 x K) * W^T, W is [64][stride] bf16 in shared memory
template <int KSTEPS>
__device__ __forceinline__ void layer(const uint32_t (*A)[4], const __nv_bfloat16* W, int stride, float acc[8][4],
                                      int g, int t)
{
#pragma unroll
    for (int n = 0; n < 8; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < KSTEPS; kt++)
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const __nv_bfloat16* row = W + (n * 8 + g) * stride + kt * 16 + 2 * t;
            mma16816(acc[n], A[kt], lds32(row), lds32(row + 8));
        }
}

// accumulators -> ReLU -> BF16 A fragments of the next layer (the C layout of
// n-tiles 2k, 2k+1 is the A layout of k-step k)
__device__ __forceinline__ void relu_pack(const float acc[8][4], uint32_t A[4][4])
{
#pragma unroll
    for (int k = 0; k < 4; k++) {
        A[k][0] = pack_bf16(fmaxf(acc[2 * k][0], 0.0f), fmaxf(acc[2 * k][1], 0.0f));
        A[k][1] = pack_bf16(fmaxf(acc[2 * k][2], 0.0f), fmaxf(acc[2 * k][3], 0.0f));
        A[k][2] = pack_bf16(fmaxf(acc[2 * k + 1][0], 0.0f), fmaxf(acc[2 * k + 1][1], 0.0f));
        A[k][3] = pack_bf16(fmaxf(acc[2 * k + 1][2], 0.0f), fmaxf(acc[2 * k + 1][3], 0.0f));
    }
}

__device__ __forceinline__ void load_weights(__nv_bfloat16* dst, const __nv_bfloat16* src, int n)
{
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int i = threadIdx.x; i < n / 8; i += blockDim.x) d[i] = s[i];
}

// The forward of one 16-sample tile; x0/x1 are this lane's two sample rows.
// Leaves the hidden activations h1..h4 as A fragments and y in acc4.
__device__ __forceinline__ void forward_tile(const __nv_bfloat16* sw, const float* x0, const float* x1, int g, int t,
                                             uint32_t H[4][4][4], float acc4[4], __nv_bfloat16* enc_out,
                                             uint64_t row0, uint64_t row1)
{
    float acc[8][4];
#pragma unroll
    for (int n = 0; n < 8; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
    for (int kt = 0; kt < NEP / 16; kt++) {
        const int c0 = kt * 16 + 2 * t, c1 = c0 + 8;
        uint32_t a[4];
        a[0] = feature_pair(x0, c0);
        a[1] = feature_pair(x1, c0);
        a[2] = feature_pair(x0, c1);
        a[3] = feature_pair(x1, c1);
        if (enc_out) {
            *reinterpret_cast<uint32_t*>(enc_out + row0 * NEP + c0) = a[0];
            *reinterpret_cast<uint32_t*>(enc_out + row1 * NEP + c0) = a[1];
            *reinterpret_cast<uint32_t*>(enc_out + row0 * NEP + c1) = a[2];
            *reinterpret_cast<uint32_t*>(enc_out + row1 * NEP + c1) = a[3];
        }
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const __nv_bfloat16* row = sw + B_W0 + (n * 8 + g) * S0 + kt * 16 + 2 * t;
            mma16816(acc[n], a, lds32(row), lds32(row + 8));
        }
    }
    relu_pack(acc, H[0]);
    layer<4>(H[0], sw + B_W1, SH, acc, g, t);
    relu_pack(acc, H[1]);
    layer<4>(H[1], sw + B_W2, SH, acc, g, t);
    relu_pack(acc, H[2]);
    layer<4>(H[2], sw + B_W3, SH, acc, g, t);
    relu_pack(acc, H[3]);
    acc4[0] = acc4[1] = acc4[2] = acc4[3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        const __nv_bfloat16* row = sw + B_W4 + g * SH + kt * 16 + 2 * t;
        mma16816(acc4, H[3][kt], lds32(row), lds32(row + 8));
    }
}

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05, accumulators in TMEM)
// ---------------------------------------------------------------------------
//
// A CTA of 256 threads holds two independent groups of 4 warps that share the
// weights in shared memory.  Each group works through tiles of 128 queries:
// thread t of the group owns query t of its tile, which is row t of every
// GEMM and TMEM lane t.  While one group waits for its MMAs the other encodes
// or drains its accumulators, so the tensor core and the CUDA cores overlap.
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
constexpr int THREADS = 256;                // two groups of 128
// byte offsets in dynamic shared memory (all 1024-aligned)
constexpr int W0 = 0;                                   // [28 kg][8 ng][128 B]
constexpr int W1 = W0 + KG0 * 8 * 128;                  // [8 kg][8 ng][128 B] x 3
constexpr int W4 = W1 + 3 * KGH * 8 * 128;              // [8 kg][2 ng][128 B] (16 rows, 3 real)
constexpr int GROUP = W4 + KGH * 2 * 128;               // per group:
constexpr int A0 = 0;                                   //   [28 kg][16 mg][128 B]
constexpr int A1 = A0 + KG0 * 16 * 128;                 //   [8 kg][16 mg][128 B]
constexpr int GROUP_BYTES = A1 + KGH * 16 * 128;
constexpr int BAR = GROUP + 2 * GROUP_BYTES;            // 2 mbarriers, TMEM address
constexpr int SMEM = BAR + 64;
constexpr uint32_t TMEM_COLS = 128;                     // 64 per group
constexpr uint32_t kWaitLimit = 1u << 22;

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

// bounded wait for mbarrier phase `parity`; false when the limit ran out
__device__ __forceinline__ bool wait(uint32_t bar, uint32_t parity)
{
    for (uint32_t i = 0; i < kWaitLimit; i++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

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
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&bars[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&bars[1])));
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
    for (uint32_t tile = blockIdx.x * 2 + g; tile < tiles && ok; tile += gridDim.x * 2) {
        const uint32_t row = tile * M + gt;
#pragma unroll
        for (int i = 0; i < NI; i++) encode_input(ga + A0, i, (int)gt, row < n ? x[(uint64_t)row * NI + i] : 0.0f);
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
                float v[16];
#pragma unroll 1
                for (int q = 0; q < 4; q++) {
                    ld16(lanes + q * 16, v);
                    ld_wait();
#pragma unroll
                    for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j], 0.0f);
                    put8(ga + A1, 2 * q, (int)gt, v);
                    put8(ga + A1, 2 * q + 1, (int)gt, v + 8);
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

// Training forward + backward.  Writes, per sample s:
//   enc[s][224]          layer-0 input (features)
//   act[l][s][64]        input of layer l+1 (h1..h4), BF16
//   dlt[l][s][64]        delta at the output of layer l (pre-activation of h_{l+1}), l = 0..3
//   dy[s][16]            delta at the network output (3 real columns), BF16
// and adds the batch loss (times 1/(3n)) to *loss.
__global__ void __launch_bounds__(128) k_mlp_fwd_bwd(const __nv_bfloat16* __restrict__ wimg, uint32_t n,
                                                    const float* __restrict__ x, const float* __restrict__ target,
                                                    __nv_bfloat16* __restrict__ enc, __nv_bfloat16* __restrict__ act,
                                                    __nv_bfloat16* __restrict__ dlt, __nv_bfloat16* __restrict__ dy,
                                                    float* __restrict__ loss)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    load_weights(sw, wimg, B_TOTAL);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const uint32_t tiles = (n + 15) / 16;
    const uint64_t np = (uint64_t)tiles * 16;   // per-layer stride of act and dlt
    const float inv = 1.0f / (3.0f * (float)n);
    float lsum = 0.0f;
    for (uint32_t tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
        const uint32_t r0 = tile * 16 + g, r1 = r0 + 8;
        const bool v0 = r0 < n, v1 = r1 < n;
        float x0[NI], x1[NI];
#pragma unroll
        for (int i = 0; i < NI; i++) {
            x0[i] = v0 ? x[(uint64_t)r0 * NI + i] : 0.0f;
            x1[i] = v1 ? x[(uint64_t)r1 * NI + i] : 0.0f;
        }
        uint32_t H[4][4][4];
        float y[4];
        forward_tile(sw, x0, x1, g, t, H, y, enc, r0, r1);
        // output delta: columns 2t, 2t+1 of rows r0 (y0,y1) and r1 (y2,y3)
        float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int col = 2 * t + (q & 1);
            const bool row_ok = (q < 2) ? v0 : v1;
            const uint32_t r = (q < 2) ? r0 : r1;
            if (col < NO && row_ok) {
                const float tv = target[(uint64_t)r * NO + col];
                const float den = y[q] * y[q] + 0.01f;
                const float res = y[q] - tv;
                lsum += res * res / den;
                d[q] = 2.0f * res / den * inv;
            }
        }
        // dy as an A fragment (16 x 16, columns 8..15 zero)
        uint32_t A[4][4];
        uint32_t ady[4] = {pack_bf16(d[0], d[1]), pack_bf16(d[2], d[3]), 0u, 0u};
        {
            __nv_bfloat16* p0 = dy + (uint64_t)r0 * 16 + 2 * t;
            __nv_bfloat16* p1 = dy + (uint64_t)r1 * 16 + 2 * t;
            *reinterpret_cast<uint32_t*>(p0) = ady[0];
            *reinterpret_cast<uint32_t*>(p1) = ady[1];
            *reinterpret_cast<uint32_t*>(p0 + 8) = 0u;
            *reinterpret_cast<uint32_t*>(p1 + 8) = 0u;
        }
        // delta into h4: dy * W4 (B = W4^T slice [in][k]), masked by h4 > 0
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
            const __nv_bfloat16* row = sw + B_W4T + (nt * 8 + g) * S4T + 2 * t;
            mma16816(acc[nt], ady, lds32(row), lds32(row + 8));
        }
        const int WT[3] = {B_W3T, B_W2T, B_W1T};
        for (int l = 3; l >= 0; l--) {
            // mask with relu'(h_{l+1}) where h_{l+1} = H[l]; pack as A; store the delta
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint32_t m0 = H[l][k][0], m1 = H[l][k][1], m2 = H[l][k][2], m3 = H[l][k][3];
                A[k][0] = pack_bf16(bf_lo(m0) > 0.0f ? acc[2 * k][0] : 0.0f, bf_hi(m0) > 0.0f ? acc[2 * k][1] : 0.0f);
                A[k][1] = pack_bf16(bf_lo(m1) > 0.0f ? acc[2 * k][2] : 0.0f, bf_hi(m1) > 0.0f ? acc[2 * k][3] : 0.0f);
                A[k][2] = pack_bf16(bf_lo(m2) > 0.0f ? acc[2 * k + 1][0] : 0.0f, bf_hi(m2) > 0.0f ? acc[2 * k + 1][1] : 0.0f);
                A[k][3] = pack_bf16(bf_lo(m3) > 0.0f ? acc[2 * k + 1][2] : 0.0f, bf_hi(m3) > 0.0f ? acc[2 * k + 1][3] : 0.0f);
                __nv_bfloat16* q0 = dlt + ((uint64_t)l * np + r0) * NH + k * 16 + 2 * t;
                __nv_bfloat16* q1 = dlt + ((uint64_t)l * np + r1) * NH + k * 16 + 2 * t;
                __nv_bfloat16* h0 = act + ((uint64_t)l * np + r0) * NH + k * 16 + 2 * t;
                __nv_bfloat16* h1 = act + ((uint64_t)l * np + r1) * NH + k * 16 + 2 * t;
                if (v0) {
                    *reinterpret_cast<uint32_t*>(q0) = A[k][0];
                    *reinterpret_cast<uint32_t*>(q0 + 8) = A[k][2];
                    *reinterpret_cast<uint32_t*>(h0) = m0;
                    *reinterpret_cast<uint32_t*>(h0 + 8) = m2;
                }
                if (v1) {
                    *reinterpret_cast<uint32_t*>(q1) = A[k][1];
                    *reinterpret_cast<uint32_t*>(q1 + 8) = A[k][3];
                    *reinterpret_cast<uint32_t*>(h1) = m1;
                    *reinterpret_cast<uint32_t*>(h1 + 8) = m3;
                }
            }
            if (l == 0) break;
            // delta into h_l: delta_{l} * W_l, B = W_l^T [in][out]
            layer<4>(A, sw + WT[3 - l], SH, acc, g, t);
        }
    }
    // warp-reduce the loss
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0) atomicAdd(loss, lsum * inv);
}

__device__ __forceinline__ void ldsm_x4_trans(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p)
{
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(a));
}

// Weight gradients of all five layers in one launch: grad_l[o][i] +=
// sum_s D_l[s][o] * X_l[s][i].  A CTA owns one 16 (o) x 64 (i) tile of one
// layer and a range of 4 * chunk samples; each of its warps reduces `chunk`
// samples on the tensor cores (ldmatrix.trans tiles of 16 samples), the four
// partial tiles are summed in shared memory and added to the gradient with
// FP32 atomics.
struct WgradLayer
{
    const __nv_bfloat16* D;   // [s][ds], o < no real
    const __nv_bfloat16* X;   // [s][xs], i < ni real
    float* grad;              // [no][ni]
    int ds, no, xs, ni;
    int o_tiles, i_groups;
    uint32_t first_cta;
};
struct WgradArgs
{
    WgradLayer l[5];
    uint32_t n, chunk, ctas_per_tile;
};

__global__ void __launch_bounds__(128) k_mlp_wgrad(WgradArgs args)
{
    __shared__ __align__(16) __nv_bfloat16 sD[4][16][24];
    __shared__ __align__(16) __nv_bfloat16 sX[4][16][72];
    __shared__ float red[3][32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    int li = 0;
#pragma unroll
    for (int k = 1; k < 5; k++)
        if (blockIdx.x >= args.l[k].first_cta) li = k;
    const WgradLayer& L = args.l[li];
    const uint32_t local = blockIdx.x - L.first_cta;
    const uint32_t tile = local / args.ctas_per_tile, part = local % args.ctas_per_tile;
    const int ot = (int)(tile % L.o_tiles), ig = (int)(tile / L.o_tiles);
    const uint32_t s_begin = (part * 4 + warp) * args.chunk;
    const uint32_t s_end = min(args.n, s_begin + args.chunk);
    float acc[8][4];
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.0f;
    for (uint32_t s0 = s_begin; s0 < s_end; s0 += 16) {
        // stage 16 samples x 16 o of D and 16 samples x 64 i of X
        __syncwarp();
        for (int e = lane; e < 16 * 2; e += 32) {
            const int r = e >> 1, h = e & 1;
            const uint32_t s = s0 + r;
            uint4 v = make_uint4(0, 0, 0, 0);
            const int oc = ot * 16 + h * 8;
            if (s < s_end && oc < L.ds) v = *reinterpret_cast<const uint4*>(L.D + (uint64_t)s * L.ds + oc);
            *reinterpret_cast<uint4*>(&sD[warp][r][h * 8]) = v;
        }
        for (int e = lane; e < 16 * 8; e += 32) {
            const int r = e >> 3, h = e & 7;
            const uint32_t s = s0 + r;
            const int ic = ig * 64 + h * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (s < s_end && ic < L.xs) v = *reinterpret_cast<const uint4*>(L.X + (uint64_t)s * L.xs + ic);
            *reinterpret_cast<uint4*>(&sX[warp][r][h * 8]) = v;
        }
        __syncwarp();
        // A = D^T (16 o x 16 s): matrices (s0-7,o0-7), (s0-7,o8-15), (s8-15,o0-7), (s8-15,o8-15)
        uint32_t a[4];
        {
            const int mtx = lane >> 3, r = lane & 7;
            const int srow = (mtx & 2) ? 8 + r : r;
            const int ocol = (mtx & 1) ? 8 : 0;
            ldsm_x4_trans(a[0], a[1], a[2], a[3], &sD[warp][srow][ocol]);
        }
        // B = X (16 s x 8 i) per n-tile: matrices (s0-7, i), (s8-15, i) for two n-tiles per ldmatrix
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int mtx = lane >> 3, r = lane & 7;
            const int srow = (mtx & 1) ? 8 + r : r;
            const int icol = q * 16 + ((mtx & 2) ? 8 : 0);
            uint32_t b0, b1, b2, b3;
            ldsm_x4_trans(b0, b1, b2, b3, &sX[warp][srow][icol]);
            mma16816(acc[2 * q], a, b0, b1);
            mma16816(acc[2 * q + 1], a, b2, b3);
        }
    }
    // sum the four warps' tiles in shared memory, then one atomic per element
    if (warp > 0) {
#pragma unroll
        for (int q = 0; q < 8; q++)
#pragma unroll
            for (int e = 0; e < 4; e++) red[warp - 1][lane][q * 4 + e] = acc[q][e];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < 8; q++)
#pragma unroll
            for (int e = 0; e < 4; e++) acc[q][e] += red[0][lane][q * 4 + e] + red[1][lane][q * 4 + e] + red[2][lane][q * 4 + e];
        // C rows o = ot*16 + g (+8), cols i = ig*64 + q*8 + 2t (+1)
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int i = ig * 64 + q * 8 + 2 * t;
            const int o0 = ot * 16 + g, o1 = o0 + 8;
            if (o0 < L.no && i < L.ni) atomicAdd(&L.grad[o0 * L.ni + i], acc[q][0]);
            if (o0 < L.no && i + 1 < L.ni) atomicAdd(&L.grad[o0 * L.ni + i + 1], acc[q][1]);
            if (o1 < L.no && i < L.ni) atomicAdd(&L.grad[o1 * L.ni + i], acc[q][2]);
            if (o1 < L.no && i + 1 < L.ni) atomicAdd(&L.grad[o1 * L.ni + i + 1], acc[q][3]);
        }
    }
}

// bf16 image position of master parameter p (forward layout), and of its transpose (or -1)
__device__ __forceinline__ void image_pos(int p, int& fwd, int& bwd)
{
    bwd = -1;
    if (p < OFF_W1) { const int o = p / NE, i = p % NE; fwd = B_W0 + o * S0 + i; return; }
    if (p < OFF_W4) {
        const int l = (p - OFF_W1) / (NH * NH), r = (p - OFF_W1) % (NH * NH), o = r / NH, i = r % NH;
        fwd = B_W1 + l * NH * SH + o * SH + i;
        bwd = B_W1T + l * NH * SH + i * SH + o;
        return;
    }
    const int r = p - OFF_W4, o = r / NH, i = r % NH;
    fwd = B_W4 + o * SH + i;
    bwd = B_W4T + i * S4T + o;
}

__global__ void __launch_bounds__(256) k_mlp_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                                                 float* __restrict__ g, float lr, float b1, float b2, float eps,
                                                 float c1, float c2, __nv_bfloat16* __restrict__ img)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N_PARAMS) return;
    const float gp = g[p];
    g[p] = 0.0f;
    const float mp = b1 * m[p] + (1.0f - b1) * gp;
    const float vp = b2 * v[p] + (1.0f - b2) * gp * gp;
    m[p] = mp;
    v[p] = vp;
    const float wp = w[p] - lr * (mp / c1) / (sqrtf(vp / c2) + eps);
    w[p] = wp;
    int f, b;
    image_pos(p, f, b);
    img[f] = __float2bfloat16_rn(wp);
    if (b >= 0) img[b] = __float2bfloat16_rn(wp);
}

__global__ void k_mlp_image(const float* __restrict__ w, __nv_bfloat16* __restrict__ img)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N_PARAMS) return;
    int f, b;
    image_pos(p, f, b);
    img[f] = __float2bfloat16_rn(w[p]);
    if (b >= 0) img[b] = __float2bfloat16_rn(w[p]);
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

static int all_smem() { return B_TOTAL * 2; }

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
    const uint32_t grid = std::max(1u, std::min<uint32_t>((tiles + 1) / 2, (uint32_t)c->num_sms));
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
static tgx_status cache_grad(tgx_ctx* c, tgx_cache* k, uint32_t n, const float* d_x, const float* d_t)
{
    static bool attr = false;
    if (!attr) {
        TGX_CUDA(cudaFuncSetAttribute(k_mlp_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, all_smem()));
        attr = true;
    }
    const uint64_t np = ((uint64_t)n + 15) / 16 * 16;
    const size_t bytes = np * NEP * 2 + 4 * np * NH * 2 * 2 + np * 16 * 2;
    TGX_TRY(devbuf_reserve(k->scratch, bytes));
    __nv_bfloat16* enc = (__nv_bfloat16*)k->scratch.ptr;
    __nv_bfloat16* act = enc + np * NEP;
    __nv_bfloat16* dlt = act + 4 * np * NH;
    __nv_bfloat16* dy = dlt + 4 * np * NH;
    TGX_CUDA(cudaMemsetAsync(k->loss, 0, 4, c->stream));
    const uint32_t tiles = (uint32_t)(np / 16);
    const uint32_t grid = std::min<uint32_t>((tiles + 3) / 4, (uint32_t)c->num_sms * 4);
    TGX_LAUNCH(c, TR_MLP_FWD_BWD, grid, 128, all_smem(), k_mlp_fwd_bwd, k->img, n, d_x, d_t, enc, act, dlt, dy, k->loss);
    // weight gradients of all layers: D [s][o] against the layer input X [s][i]
    WgradArgs a;
    a.n = n;
    a.chunk = 256;
    a.ctas_per_tile = (n + 4 * a.chunk - 1) / (4 * a.chunk);
    const WgradLayer ls[5] = {
        {dlt + 0 * np * NH, enc, k->g + OFF_W0, NH, NH, NEP, NE, 0, 0, 0},
        {dlt + 1 * np * NH, act + 0 * np * NH, k->g + OFF_W1, NH, NH, NH, NH, 0, 0, 0},
        {dlt + 2 * np * NH, act + 1 * np * NH, k->g + OFF_W2, NH, NH, NH, NH, 0, 0, 0},
        {dlt + 3 * np * NH, act + 2 * np * NH, k->g + OFF_W3, NH, NH, NH, NH, 0, 0, 0},
        {dy, act + 3 * np * NH, k->g + OFF_W4, 16, NO, NH, NH, 0, 0, 0},
    };
    uint32_t ctas = 0;
    for (int l = 0; l < 5; l++) {
        a.l[l] = ls[l];
        a.l[l].o_tiles = (ls[l].no + 15) / 16;
        a.l[l].i_groups = (ls[l].ni + 63) / 64;
        a.l[l].first_cta = ctas;
        ctas += (uint32_t)(a.l[l].o_tiles * a.l[l].i_groups) * a.ctas_per_tile;
    }
    TGX_LAUNCH(c, TR_MLP_WGRAD, ctas, 128, 0, k_mlp_wgrad, a);
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

extern "C" tgx_status tgx_cache_train_step(tgx_ctx* c, tgx_cache* k, uint32_t n, const float* d_x, const float* d_t,
                                           float lr)
{
    if (!c || !k || !n || !d_x || !d_t) return TGX_ERR_INVALID_ARGUMENT;
    TGX_TRY(cache_grad(c, k, n, d_x, d_t));
    k->step++;
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-15f;
    const float c1 = (float)(1.0 - pow((double)b1, (double)k->step)), c2 = (float)(1.0 - pow((double)b2, (double)k->step));
    TGX_LAUNCH(c, TR_MLP_ADAM, (N_PARAMS + 255) / 256, 256, 0, k_mlp_adam, k->w, k->m, k->v, k->g, lr, b1, b2, eps, c1, c2,
               k->img);
    return TGX_OK;
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
