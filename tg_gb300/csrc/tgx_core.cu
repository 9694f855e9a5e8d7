// tgx_core.cu -- context, errors, scene upload and picking of the C ABI.
//
// Replaces the buffer set-up and staging uploads of tg's Vulkan raytracer
// (tg__init_buffers tgvk_raytracer.c:156-274, tg_raytracer_create_object
// :805-992, tg_raytracer_get_hovered_voxel :1605-1655) with plain device
// allocations on one stream.

#include "tgx_internal.cuh"

#include <algorithm>

#include <cstdarg>
#include <cstdlib>
#include <new>

static thread_local char g_error[1024];

void tgx_set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

extern "C" const char* tgx_last_error_string(void) { return g_error; }

extern "C" uint32_t tgx_abi_version(void) { return TGX_ABI_VERSION; }

extern "C" const char* tgx_status_string(tgx_status s)
{
    switch (s) {
        case TGX_OK: return "ok";
        case TGX_ERR_INVALID_ARGUMENT: return "invalid argument";
        case TGX_ERR_OUT_OF_MEMORY: return "out of memory";
        case TGX_ERR_CUDA: return "CUDA error";
        case TGX_ERR_CAPACITY: return "capacity exceeded";
        case TGX_ERR_TIMEOUT: return "step budget exhausted";
        case TGX_ERR_NOT_SUPPORTED: return "not supported";
        case TGX_ERR_NO_DEVICE: return "no CUDA device";
        case TGX_ERR_DEVICE_FAULT: return "device-side error recorded";
    }
    return "unknown status";
}

tgx_status devbuf_reserve(DevBuf& b, size_t bytes)
{
    if (bytes <= b.bytes && b.ptr) return TGX_OK;
    if (b.ptr) { cudaFree(b.ptr); b.ptr = nullptr; b.bytes = 0; }
    size_t want = bytes < 256 ? 256 : bytes;
    want = want + want / 4;   // headroom so slowly growing scenes do not reallocate every frame
    TGX_CUDA(cudaMalloc(&b.ptr, want));
    b.bytes = want;
    return TGX_OK;
}

void devbuf_free(DevBuf& b)
{
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

extern "C" tgx_status tgx_create(const tgx_config* cfg, tgx_ctx** out)
{
    if (!out) { tgx_set_error("tgx_create: out_ctx is NULL"); return TGX_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        tgx_set_error("tgx_create: no CUDA device");
        return TGX_ERR_NO_DEVICE;
    }
    tgx_config def = {};
    if (!cfg) cfg = &def;
    if (cfg->device < 0 || cfg->device >= n || (cfg->flags & ~(TGX_FLAG_MIN_BIN_CAPACITY | TGX_FLAG_TEST_LOST_COPY)) != 0) {
        tgx_set_error("tgx_create: bad device %d or flags %u", cfg->device, cfg->flags);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    const uint32_t tw = cfg->tile_w ? cfg->tile_w : 16, th = cfg->tile_h ? cfg->tile_h : 16;
    if (tw * th > 512 || tw * th < 32 || (tw * th) % 32 != 0) {
        tgx_set_error("tgx_create: tile %ux%u must hold 32..512 pixels in whole warps", tw, th);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (cfg->trace_steps > 256) {
        tgx_set_error("tgx_create: trace_steps %u outside 1..256", cfg->trace_steps);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    TGX_CUDA(cudaSetDevice(cfg->device));
    tgx_ctx* c = new (std::nothrow) tgx_ctx();
    if (!c) return TGX_ERR_OUT_OF_MEMORY;
    c->device = cfg->device;
    c->tile_w = tw;
    c->tile_h = th;
    c->flags = cfg->flags;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, cfg->device);
    if (cfg->trace_steps) c->trace_steps_per_round = cfg->trace_steps;
    if (cfg->stream) {
        c->stream = (cudaStream_t)cfg->stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            tgx_set_error("tgx_create: cudaStreamCreate failed");
            delete c;
            return TGX_ERR_CUDA;
        }
        c->own_stream = true;
    }
    if (cudaMalloc(&c->d_status, sizeof(tgx_dev_status)) != cudaSuccess ||
        cudaMemset(c->d_status, 0, sizeof(tgx_dev_status)) != cudaSuccess ||
        cudaMallocHost(&c->h_counter, 64) != cudaSuccess || cudaMallocHost(&c->h_vis_counters, 64) != cudaSuccess) {
        tgx_set_error("tgx_create: allocation failed");
        tgx_destroy(c);
        return TGX_ERR_OUT_OF_MEMORY;
    }
    if (const tgx_status st = vis_prepare_device(c); st != TGX_OK) {
        tgx_destroy(c);
        return st;
    }
    *out = c;
    return TGX_OK;
}

extern "C" void tgx_destroy(tgx_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    trace_free(c);
    devbuf_free(c->vis_records);
    devbuf_free(c->vis_counters);
    devbuf_free(c->vis_tile_cnt);
    devbuf_free(c->vis_tile_off);
    devbuf_free(c->vis_bins);
    devbuf_free(c->vis_views);
    devbuf_free(c->svo_counters);
    devbuf_free(c->svo_pairs);
    devbuf_free(c->svo_scratch);
    devbuf_free(c->svo_sort);
    devbuf_free(c->gi_scratch);
    devbuf_free(c->host_stage);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    if (c->h_counter) cudaFreeHost(c->h_counter);
    if (c->h_vis_counters) cudaFreeHost(c->h_vis_counters);
    if (c->vis_done) cudaEventDestroy(c->vis_done);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    for (int i = 0; i < 2; i++) {
        devbuf_free(c->host_slot[i]);
        if (c->host_rendered[i]) cudaEventDestroy(c->host_rendered[i]);
        if (c->host_copied[i]) cudaEventDestroy(c->host_copied[i]);
    }
    if (c->d_status) cudaFree(c->d_status);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

// ---- tracing ----

static const char* kTraceNames[TR_COUNT] = {
    "k_object_setup", "k_vis_cluster_setup", "k_vis_count", "k_vis_prefix", "k_vis_scan", "k_vis_bin_fill", "k_vis_tiles",
    "k_svo_candidates", "k_svo_alloc", "k_svo_voxelize", "k_svo_pyramid", "k_svo_trace", "k_gi_paths", "k_trace_queue", "k_mlp_forward",
    "k_mlp_train_tc", "k_mlp_reduce", "k_mlp_adam"};

static cudaEvent_t trace_event(tgx_ctx* c)
{
    TraceState& t = c->trace;
    if (t.n_free) return t.free_events[--t.n_free];
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void trace_begin(tgx_ctx* c, int slot)
{
    TraceState& t = c->trace;
    if (!t.enabled) return;
    if (t.n_pending == t.cap_pending) {
        t.cap_pending = t.cap_pending ? 2 * t.cap_pending : 64;
        t.pending = (TraceState::Pending*)realloc(t.pending, t.cap_pending * sizeof(TraceState::Pending));
    }
    TraceState::Pending& p = t.pending[t.n_pending++];
    p.slot = slot;
    p.a = trace_event(c);
    p.b = trace_event(c);
    cudaEventRecord(p.a, c->stream);
}

void trace_end(tgx_ctx* c, int slot)
{
    TraceState& t = c->trace;
    if (!t.enabled || !t.n_pending) return;
    (void)slot;
    cudaEventRecord(t.pending[t.n_pending - 1].b, c->stream);
}

static void trace_collect(tgx_ctx* c)
{
    TraceState& t = c->trace;
    if (!t.n_pending) return;
    cudaStreamSynchronize(c->stream);
    for (size_t i = 0; i < t.n_pending; i++) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, t.pending[i].a, t.pending[i].b) == cudaSuccess) {
            t.ms[t.pending[i].slot] += ms;
            t.launches[t.pending[i].slot]++;
        }
        for (cudaEvent_t e : {t.pending[i].a, t.pending[i].b}) {
            if (t.n_free == t.cap_free) {
                t.cap_free = t.cap_free ? 2 * t.cap_free : 128;
                t.free_events = (cudaEvent_t*)realloc(t.free_events, t.cap_free * sizeof(cudaEvent_t));
            }
            t.free_events[t.n_free++] = e;
        }
    }
    t.n_pending = 0;
    cudaGetLastError();
}

void trace_free(tgx_ctx* c)
{
    TraceState& t = c->trace;
    trace_collect(c);
    for (size_t i = 0; i < t.n_free; i++) cudaEventDestroy(t.free_events[i]);
    free(t.free_events);
    free(t.pending);
    t = TraceState();
}

extern "C" uint32_t tgx_trace_slots(void) { return TR_COUNT; }

extern "C" tgx_status tgx_trace_enable(tgx_ctx* c, int enable)
{
    if (!c) return TGX_ERR_INVALID_ARGUMENT;
    if (!enable) trace_collect(c);
    c->trace.enabled = enable != 0;
    return TGX_OK;
}

extern "C" tgx_status tgx_trace_reset(tgx_ctx* c)
{
    if (!c) return TGX_ERR_INVALID_ARGUMENT;
    trace_collect(c);
    for (int i = 0; i < TR_COUNT; i++) { c->trace.ms[i] = 0.0; c->trace.launches[i] = 0; }
    return TGX_OK;
}

extern "C" tgx_status tgx_trace_get(tgx_ctx* c, uint32_t slot, const char** name, double* ms, uint64_t* launches)
{
    if (!c || slot >= TR_COUNT) return TGX_ERR_INVALID_ARGUMENT;
    trace_collect(c);
    if (name) *name = kTraceNames[slot];
    if (ms) *ms = c->trace.ms[slot];
    if (launches) *launches = c->trace.launches[slot];
    return TGX_OK;
}

extern "C" void* tgx_stream(tgx_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" uint64_t tgx_launch_count(tgx_ctx* c) { return c ? c->launches : 0; }

extern "C" tgx_status tgx_sync(tgx_ctx* c)
{
    if (!c) return TGX_ERR_INVALID_ARGUMENT;
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    return TGX_OK;
}

extern "C" tgx_status tgx_set_trace_steps(tgx_ctx* c, uint32_t steps)
{
    if (!c || steps < 1 || steps > 256) {
        tgx_set_error("tgx_set_trace_steps: steps %u outside 1..256", steps);
        return TGX_ERR_INVALID_ARGUMENT;
    }
    c->trace_steps_per_round = steps;
    return TGX_OK;
}

extern "C" tgx_status tgx_last_device_error(tgx_ctx* c, tgx_device_error* out)
{
    if (!c || !out) return TGX_ERR_INVALID_ARGUMENT;
    tgx_dev_status s;
    TGX_CUDA(cudaMemcpyAsync(&s, c->d_status, sizeof(s), cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    TGX_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(s), c->stream));
    out->code = s.code;
    out->where = s.where;
    out->detail = s.detail;
    return s.code ? (tgx_status)s.code : TGX_OK;
}

// Per-object 3x3 linear part of inverse(rotation) (visibility.frag:59, with
// tgm_m4_inverse's operation order).  For every cluster of an object the
// first three columns of ws2ms (visibility.frag:62) equal this matrix in
// value, so the ray direction can be transformed once per (pixel, object).
__global__ void k_object_setup(const tgx_object* __restrict__ objs, uint32_t n, float* __restrict__ inv_rot)
{
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

// per cluster pointer p: c2o[cluster_pointers[p]], with bit 31 set when that
// cluster has no set voxel (such a cluster never writes a visibility word)
__global__ void k_scene_cp_obj(const uint32_t* __restrict__ cluster_pointers, const uint32_t* __restrict__ c2o,
                               const uint32_t* __restrict__ bits, uint32_t n, uint32_t* __restrict__ out)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t ci = cluster_pointers[p];
    const uint4* w = reinterpret_cast<const uint4*>(bits + (uint64_t)ci * 16u);
    const uint4 a = w[0], b = w[1], c = w[2], d = w[3];
    const bool empty = !(a.x | a.y | a.z | a.w | b.x | b.y | b.z | b.w | c.x | c.y | c.z | c.w | d.x | d.y | d.z | d.w);
    out[p] = c2o[ci] | (empty ? 0x80000000u : 0u);
}

void scene_release(tgx_scene* s)
{
    if (!s) return;
    cudaFree(s->d_cp_obj);
    cudaFree(s->d_objects);
    cudaFree(s->d_inv_rot);
    cudaFree(s->d_cluster_pointers);
    cudaFree(s->d_c2o);
    cudaFree(s->d_bits);
    cudaFree(s->d_material);
    cudaFree(s->d_luts);
    delete s;
}
static void scene_free(tgx_scene* s) { scene_release(s); }

// per-object inverse rotations of a scene whose arrays are on the device; synchronous
tgx_status scene_finish(tgx_ctx* c, tgx_scene* s)
{
    if (!s->d_cp_obj) {
        // the cull's per-pointer table, once per scene (its inputs never change)
        const cudaError_t e = scene_malloc(c, s, (void**)&s->d_cp_obj, (size_t)s->n_cluster_pointers * 4);
        if (e != cudaSuccess) {
            cudaGetLastError();
            tgx_set_error("scene setup: out of device memory or past the context's budget (%u-word pointer table)",
                          s->n_cluster_pointers);
            return e == cudaErrorMemoryAllocation ? TGX_ERR_OUT_OF_MEMORY : TGX_ERR_CUDA;
        }
        k_scene_cp_obj<<<(s->n_cluster_pointers + 255) / 256, 256, 0, c->stream>>>(
            s->d_cluster_pointers, s->d_c2o, s->d_bits, s->n_cluster_pointers, s->d_cp_obj);
        if (cudaGetLastError() == cudaSuccess) c->launches++;
    }
    trace_begin(c, TR_OBJECT_SETUP);
    k_object_setup<<<(s->n_objects + 127) / 128, 128, 0, c->stream>>>(s->d_objects, s->n_objects, s->d_inv_rot);
    cudaError_t le = cudaGetLastError();
    trace_end(c, TR_OBJECT_SETUP);
    if (le == cudaSuccess) c->launches++;
    if (le == cudaSuccess) le = cudaStreamSynchronize(c->stream);
    if (le != cudaSuccess) {
        tgx_set_error("scene setup: %s", cudaGetErrorString(le));
        return TGX_ERR_CUDA;
    }
    return TGX_OK;
}

// A scene-store array: refused (as an allocation failure, nothing allocated)
// when it would take the context's live scene stores past its budget.
cudaError_t scene_malloc(tgx_ctx* c, tgx_scene* s, void** p, size_t bytes)
{
    if (c->mem_budget && c->mem_scenes + bytes > c->mem_budget) return cudaErrorMemoryAllocation;
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) {
        c->mem_scenes += bytes;
        s->bytes += bytes;
    }
    return e;
}

extern "C" tgx_status tgx_set_memory_budget(tgx_ctx* c, uint64_t bytes)
{
    if (!c) return TGX_ERR_INVALID_ARGUMENT;
    c->mem_budget = bytes;
    return TGX_OK;
}

extern "C" tgx_status tgx_get_memory(tgx_ctx* c, uint64_t* out_budget, uint64_t* out_scene_bytes)
{
    if (!c) return TGX_ERR_INVALID_ARGUMENT;
    if (out_budget) *out_budget = c->mem_budget;
    if (out_scene_bytes) *out_scene_bytes = c->mem_scenes;
    return TGX_OK;
}

extern "C" tgx_status tgx_scene_upload(tgx_ctx* c, const tgx_scene_desc* d, tgx_scene** out)
{
    if (!c || !d || !out) { tgx_set_error("tgx_scene_upload: NULL argument"); return TGX_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    if (!d->objects || !d->cluster_pointers || !d->cluster_idx_to_object_idx || !d->voxel_bits ||
        d->n_objects == 0 || d->n_cluster_pointers == 0 || d->n_clusters == 0) {
        tgx_set_error("tgx_scene_upload: empty scene or missing array");
        return TGX_ERR_INVALID_ARGUMENT;
    }
    if (d->n_clusters > (1u << TGX_CLUSTER_IDX_BITS) || d->n_cluster_pointers > (1u << TGX_CLUSTER_IDX_BITS)) {
        tgx_set_error("tgx_scene_upload: more than 2^31 clusters");
        return TGX_ERR_CAPACITY;
    }
    if (d->n_objects >= 0x80000000u) {   // the cull's pointer table keeps an object index in 31 bits
        tgx_set_error("tgx_scene_upload: 2^31 or more objects");
        return TGX_ERR_CAPACITY;
    }
    // Host-side validation of the data model (the reference only asserts).
    for (uint32_t p = 0; p < d->n_cluster_pointers; p++) {
        const uint32_t ci = d->cluster_pointers[p];
        if (ci >= d->n_clusters) { tgx_set_error("cluster pointer %u -> cluster %u out of range", p, ci); return TGX_ERR_INVALID_ARGUMENT; }
        const uint32_t oi = d->cluster_idx_to_object_idx[ci];
        if (oi >= d->n_objects) { tgx_set_error("cluster %u -> object %u out of range", ci, oi); return TGX_ERR_INVALID_ARGUMENT; }
        const tgx_object& o = d->objects[oi];
        const uint64_t cnt = (uint64_t)o.n_cluster_pointers_per_dim[0] * o.n_cluster_pointers_per_dim[1] * o.n_cluster_pointers_per_dim[2];
        if (cnt == 0 || p < o.first_cluster_pointer || (uint64_t)p >= o.first_cluster_pointer + cnt) {
            tgx_set_error("cluster pointer %u is outside the range of its object %u", p, oi);
            return TGX_ERR_INVALID_ARGUMENT;
        }
    }
    for (uint32_t i = 0; i < d->n_objects; i++) {
        const tgx_object& o = d->objects[i];
        const uint64_t cnt = (uint64_t)o.n_cluster_pointers_per_dim[0] * o.n_cluster_pointers_per_dim[1] * o.n_cluster_pointers_per_dim[2];
        if ((uint64_t)o.first_cluster_pointer + cnt > d->n_cluster_pointers) {
            tgx_set_error("object %u's cluster pointers run past the %u given", i, d->n_cluster_pointers);
            return TGX_ERR_INVALID_ARGUMENT;
        }
    }
    if (d->luts && d->n_luts == 0) { tgx_set_error("luts given with n_luts = 0"); return TGX_ERR_INVALID_ARGUMENT; }
    if (d->luts) {
        for (uint32_t i = 0; i < d->n_objects; i++)
            if (d->objects[i].lut_idx >= d->n_luts) { tgx_set_error("object %u lut_idx out of range", i); return TGX_ERR_INVALID_ARGUMENT; }
    }
    TGX_CUDA(cudaSetDevice(c->device));
    tgx_scene* s = new (std::nothrow) tgx_scene();
    if (!s) return TGX_ERR_OUT_OF_MEMORY;
    s->n_objects = d->n_objects;
    s->n_cluster_pointers = d->n_cluster_pointers;
    s->n_clusters = d->n_clusters;
    s->n_luts = d->luts ? d->n_luts : 0;
    cudaError_t e = cudaSuccess;
#define ALLOC_COPY(dst, src, bytes)                                                                 \
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&(dst), (bytes));                          \
    if (e == cudaSuccess) e = cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyHostToDevice, c->stream);
    ALLOC_COPY(s->d_objects, d->objects, (size_t)d->n_objects * sizeof(tgx_object));
    ALLOC_COPY(s->d_cluster_pointers, d->cluster_pointers, (size_t)d->n_cluster_pointers * 4);
    ALLOC_COPY(s->d_c2o, d->cluster_idx_to_object_idx, (size_t)d->n_clusters * 4);
    ALLOC_COPY(s->d_bits, d->voxel_bits, (size_t)d->n_clusters * 64);
    if (d->material_idx) { ALLOC_COPY(s->d_material, d->material_idx, (size_t)d->n_clusters * 512); }
    if (d->luts) { ALLOC_COPY(s->d_luts, d->luts, (size_t)d->n_luts * 256 * sizeof(tgx_material)); }
#undef ALLOC_COPY
    if (e == cudaSuccess) e = scene_malloc(c, s, (void**)&s->d_inv_rot, (size_t)d->n_objects * 9 * sizeof(float));
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation && c->mem_budget)
            tgx_set_error("tgx_scene_upload: out of device memory or past the context's budget of %llu bytes",
                          (unsigned long long)c->mem_budget);
        else
            tgx_set_error("tgx_scene_upload: %s", cudaGetErrorString(e));
        cudaGetLastError();
        cudaStreamSynchronize(c->stream);
        c->mem_scenes -= s->bytes;
        scene_free(s);
        return e == cudaErrorMemoryAllocation ? TGX_ERR_OUT_OF_MEMORY : TGX_ERR_CUDA;
    }
    const tgx_status st = scene_finish(c, s);
    if (st != TGX_OK) {
        c->mem_scenes -= s->bytes;
        scene_free(s);
        return st;
    }
    *out = s;
    return TGX_OK;
}

extern "C" void tgx_scene_destroy(tgx_ctx* c, tgx_scene* s)
{
    if (c) {
        cudaStreamSynchronize(c->stream);
        if (s) c->mem_scenes -= std::min(c->mem_scenes, s->bytes);
    }
    scene_free(s);
}

extern "C" tgx_status tgx_pick(tgx_ctx* c, const uint64_t* d_visbuf, uint32_t w, uint32_t h, uint32_t x, uint32_t y,
                               float* out_depth, uint32_t* out_ptr, uint32_t* out_voxel, int* out_hit)
{
    if (!c || !d_visbuf || x >= w || y >= h) { tgx_set_error("tgx_pick: bad argument"); return TGX_ERR_INVALID_ARGUMENT; }
    TGX_CUDA(cudaMemcpyAsync(c->h_counter, d_visbuf + (size_t)w * y + x, 8, cudaMemcpyDeviceToHost, c->stream));
    TGX_CUDA(cudaStreamSynchronize(c->stream));
    const int hit = tgx_vis_decode(*c->h_counter, out_depth, out_ptr, out_voxel);
    if (out_hit) *out_hit = hit;
    return TGX_OK;
}
