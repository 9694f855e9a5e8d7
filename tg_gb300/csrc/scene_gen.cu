// scene_gen.cu -- the synthetic scene generator on the device, and scene download.
//
// tg fills its cluster store on the CPU, one noise loop per object, and
// uploads it cluster by cluster (tgvk_raytracer.c:870-978, "TODO: gen on GPU"
// at :868).  tgx_generate_scene_device builds the whole store in HBM instead:
// the object records come from the host generator's per-object code, then one
// thread per voxel evaluates the same counter-based hashes and (for value
// noise) the same exactly rounded float steps as host_scene.c, so the device
// scene equals tgx_generate_scene's byte for byte.  A warp ballot packs 32
// consecutive voxels into one bit word.

#include "tgx_internal.cuh"

#include <vector>

extern "C" uint64_t tgx__gen_objects(const tgx_gen_params* p, tgx_object* objects);
extern "C" void tgx__gen_luts(const tgx_gen_params* p, tgx_material* luts);
tgx_status scene_finish(tgx_ctx* c, tgx_scene* s);
void scene_release(tgx_scene* s);

namespace {

enum { ST_DIMS = 1, ST_TRANS, ST_QUAT, ST_BITS, ST_NOISE, ST_MAT, ST_LUT, ST_OBJLUT, ST_NOISEOFF };

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ uint64_t hash3(uint64_t seed, uint64_t stream, uint64_t i)
{
    return mix64(mix64(seed * 0x2545F4914F6CDD1Dull ^ mix64(stream)) ^ i);
}

__device__ __forceinline__ float unit_f32(uint64_t h) { return xmul((float)(h >> 40), 1.0f / 16777216.0f); }

__device__ __forceinline__ float smooth(float f) { return xmul(xmul(f, f), xsub(3.0f, xmul(2.0f, f))); }

__device__ __forceinline__ float lattice(uint64_t seed, int64_t i, int64_t j, int64_t k)
{
    const uint64_t key = ((uint64_t)(i & 0x1FFFFF) << 42) | ((uint64_t)(j & 0x1FFFFF) << 21) | (uint64_t)(k & 0x1FFFFF);
    return unit_f32(hash3(seed, ST_NOISE, key));
}

__device__ __forceinline__ float lerp_(float a, float b, float t) { return xadd(a, xmul(t, xsub(b, a))); }

__device__ float value_noise(uint64_t seed, float px, float py, float pz)
{
    const float fx0 = floorf(px), fy0 = floorf(py), fz0 = floorf(pz);
    const int64_t ix = (int64_t)fx0, iy = (int64_t)fy0, iz = (int64_t)fz0;
    const float sx = smooth(xsub(px, fx0)), sy = smooth(xsub(py, fy0)), sz = smooth(xsub(pz, fz0));
    const float x00 = lerp_(lattice(seed, ix, iy, iz), lattice(seed, ix + 1, iy, iz), sx);
    const float x10 = lerp_(lattice(seed, ix, iy + 1, iz), lattice(seed, ix + 1, iy + 1, iz), sx);
    const float x01 = lerp_(lattice(seed, ix, iy, iz + 1), lattice(seed, ix + 1, iy, iz + 1), sx);
    const float x11 = lerp_(lattice(seed, ix, iy + 1, iz + 1), lattice(seed, ix + 1, iy + 1, iz + 1), sx);
    return lerp_(lerp_(x00, x10, sy), lerp_(x01, x11, sy), sz);
}

struct GenConst
{
    unsigned long long seed;
    uint32_t kind, bern;
    float period, threshold;
};

// one thread per voxel of the store; objects are sorted by first cluster pointer
__global__ void __launch_bounds__(256) k_gen_clusters(const tgx_object* __restrict__ objects, uint32_t n_objects,
                                                     uint64_t n_voxels, GenConst g, uint32_t* __restrict__ ptrs,
                                                     uint32_t* __restrict__ c2o, uint32_t* __restrict__ bits,
                                                     uint8_t* __restrict__ mat)
{
    const uint64_t gvi = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;   // n_voxels is a multiple of 512
    if (gvi >= n_voxels) return;
    const uint32_t c = (uint32_t)(gvi >> 9), v = (uint32_t)(gvi & 511u);
    uint32_t lo = 0, hi = n_objects - 1;   // last object whose first pointer <= c
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (objects[mid].first_cluster_pointer <= c) lo = mid;
        else hi = mid - 1;
    }
    const uint32_t oi = lo;
    const tgx_object& o = objects[oi];
    bool solid;
    if (g.kind == 0) {
        solid = (uint32_t)(hash3(g.seed, ST_BITS, gvi) >> 40) < g.bern;
    } else {
        const uint32_t rel = c - o.first_cluster_pointer;
        const uint32_t nx = o.n_cluster_pointers_per_dim[0], ny = o.n_cluster_pointers_per_dim[1];
        const uint32_t cx = rel % nx, cy = (rel / nx) % ny, cz = rel / (nx * ny);
        const float ox = (float)(hash3(g.seed, ST_NOISEOFF, 3ull * oi + 0) % 4096u);
        const float oy = (float)(hash3(g.seed, ST_NOISEOFF, 3ull * oi + 1) % 4096u);
        const float oz = (float)(hash3(g.seed, ST_NOISEOFF, 3ull * oi + 2) % 4096u);
        const float X = xadd(xadd((float)(8u * cx + (v & 7u)), 0.5f), ox);
        const float Y = xadd(xadd((float)(8u * cy + ((v >> 3) & 7u)), 0.5f), oy);
        const float Z = xadd(xadd((float)(8u * cz + (v >> 6)), 0.5f), oz);
        solid = value_noise(g.seed, xdiv(X, g.period), xdiv(Y, g.period), xdiv(Z, g.period)) > g.threshold;
    }
    // 32 consecutive voxels of the warp = one bit word
    const uint32_t word = __ballot_sync(__activemask(), solid);
    if ((threadIdx.x & 31u) == 0) bits[gvi >> 5] = word;
    mat[gvi] = (uint8_t)(hash3(g.seed, ST_MAT, gvi) & 255u);
    if (v == 0) {
        ptrs[c] = c;
        c2o[c] = oi;
    }
}

}  // namespace

extern "C" tgx_status tgx_generate_scene_device(tgx_ctx* c, const tgx_gen_params* p, tgx_scene** out)
{
    if (!c || !p || !out || p->n_objects == 0 || p->min_clusters_per_axis == 0 ||
        p->max_clusters_per_axis < p->min_clusters_per_axis || p->kind > 1) {
        tgx_set_error("tgx_generate_scene_device: bad parameters");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    TGX_CUDA(cudaSetDevice(c->device));
    std::vector<tgx_object> objects(p->n_objects);
    const uint64_t total = tgx__gen_objects(p, objects.data());
    if (total == 0) { tgx_set_error("tgx_generate_scene_device: 2^31 clusters or more"); return TGX_ERR_CAPACITY; }
    const uint32_t n_luts = p->n_luts ? p->n_luts : 1;
    std::vector<tgx_material> luts((size_t)n_luts * 256);
    tgx__gen_luts(p, luts.data());
    tgx_scene* s = new (std::nothrow) tgx_scene();
    if (!s) return TGX_ERR_OUT_OF_MEMORY;
    s->n_objects = p->n_objects;
    s->n_cluster_pointers = s->n_clusters = (uint32_t)total;
    s->n_luts = n_luts;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_objects, objects.size() * sizeof(tgx_object));
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_cluster_pointers, total * 4);
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_c2o, total * 4);
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_bits, total * 64);
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_material, total * 512);
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_luts, luts.size() * sizeof(tgx_material));
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_inv_rot, (size_t)p->n_objects * 9 * sizeof(float));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_objects, objects.data(), objects.size() * sizeof(tgx_object), cudaMemcpyHostToDevice,
                            c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_luts, luts.data(), luts.size() * sizeof(tgx_material), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        tgx_set_error("tgx_generate_scene_device: %s", cudaGetErrorString(e));
        cudaStreamSynchronize(c->stream);
        c->mem_scenes -= s->bytes;
        scene_release(s);
        return e == cudaErrorMemoryAllocation ? TGX_ERR_OUT_OF_MEMORY : TGX_ERR_CUDA;
    }
    GenConst g;
    g.seed = p->seed;
    g.kind = p->kind;
    g.bern = (uint32_t)((double)p->bernoulli_p * 16777216.0);
    g.period = p->noise_period > 0.0f ? p->noise_period : 64.0f;
    g.threshold = p->noise_threshold;
    const uint64_t n_voxels = total * 512;
    auto launch = [&]() -> tgx_status {
        TGX_LAUNCH(c, TR_OBJECT_SETUP, (uint32_t)((n_voxels + 255) / 256), 256, 0, k_gen_clusters, s->d_objects,
                   p->n_objects, n_voxels, g, s->d_cluster_pointers, s->d_c2o, s->d_bits, s->d_material);
        return TGX_OK;
    };
    tgx_status st = launch();
    if (st == TGX_OK) st = scene_finish(c, s);
    if (st != TGX_OK) {
        cudaStreamSynchronize(c->stream);
        c->mem_scenes -= s->bytes;
        scene_release(s);
        return st;
    }
    *out = s;
    return TGX_OK;
}

extern "C" tgx_status tgx_scene_counts(const tgx_scene* s, uint32_t* n_objects, uint32_t* n_cluster_pointers,
                                       uint32_t* n_clusters, uint32_t* n_luts)
{
    if (!s) return TGX_ERR_INVALID_ARGUMENT;
    if (n_objects) *n_objects = s->n_objects;
    if (n_cluster_pointers) *n_cluster_pointers = s->n_cluster_pointers;
    if (n_clusters) *n_clusters = s->n_clusters;
    if (n_luts) *n_luts = s->n_luts;
    return TGX_OK;
}

extern "C" tgx_status tgx_scene_download(tgx_ctx* c, const tgx_scene* s, tgx_object* objects,
                                         uint32_t* cluster_pointers, uint32_t* cluster_idx_to_object_idx,
                                         uint32_t* voxel_bits, uint8_t* material_idx, tgx_material* luts)
{
    if (!c || !s) return TGX_ERR_INVALID_ARGUMENT;
    if (objects) TGX_CUDA(cudaMemcpyAsync(objects, s->d_objects, (size_t)s->n_objects * sizeof(tgx_object), cudaMemcpyDeviceToHost, c->stream));
    if (cluster_pointers) TGX_CUDA(cudaMemcpyAsync(cluster_pointers, s->d_cluster_pointers, (size_t)s->n_cluster_pointers * 4, cudaMemcpyDeviceToHost, c->stream));
    if (cluster_idx_to_object_idx) TGX_CUDA(cudaMemcpyAsync(cluster_idx_to_object_idx, s->d_c2o, (size_t)s->n_clusters * 4, cudaMemcpyDeviceToHost, c->stream));
    if (voxel_bits) TGX_CUDA(cudaMemcpyAsync(voxel_bits, s->d_bits, (size_t)s->n_clusters * 64, cudaMemcpyDeviceToHost, c->stream));
    if (material_idx && s->d_material) TGX_CUDA(cudaMemcpyAsync(material_idx, s->d_material, (size_t)s->n_clusters * 512, cudaMemcpyDeviceToHost, c->stream));
    if (luts && s->d_luts) TGX_CUDA(cudaMemcpyAsync(luts, s->d_luts, (size_t)s->n_luts * 256 * sizeof(tgx_material), cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

extern "C" tgx_status tgx_scene_set_objects(tgx_ctx* c, tgx_scene* s, uint32_t first, uint32_t n, const tgx_object* objects)
{
    if (!c || !s || (n && !objects)) { tgx_set_error("tgx_scene_set_objects: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    if ((uint64_t)first + n > s->n_objects) {
        tgx_set_error("tgx_scene_set_objects: objects %u..%u outside the scene's %u", first, first + n, s->n_objects);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return TGX_OK;
    TGX_CUDA(cudaSetDevice(c->device));
    std::vector<tgx_object> cur(n);
    TGX_CUDA(cudaMemcpyAsync(cur.data(), s->d_objects + first, (size_t)n * sizeof(tgx_object), cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    for (uint32_t i = 0; i < n; i++) {
        const tgx_object &o = objects[i], &w = cur[i];
        if (o.first_cluster_pointer != w.first_cluster_pointer || o.n_cluster_pointers_per_dim[0] != w.n_cluster_pointers_per_dim[0] ||
            o.n_cluster_pointers_per_dim[1] != w.n_cluster_pointers_per_dim[1] ||
            o.n_cluster_pointers_per_dim[2] != w.n_cluster_pointers_per_dim[2]) {
            tgx_set_error("tgx_scene_set_objects: object %u changes its cluster layout", first + i);
            return TGX_ERR_INVALID_ARGUMENT;
        }
        if (s->d_luts && o.lut_idx >= s->n_luts) {
            tgx_set_error("tgx_scene_set_objects: object %u lut_idx out of range", first + i);
            return TGX_ERR_INVALID_ARGUMENT;
        }
    }
    TGX_CUDA(cudaMemcpyAsync(s->d_objects + first, objects, (size_t)n * sizeof(tgx_object), cudaMemcpyHostToDevice, c->stream));
    return scene_finish(c, s);
}
