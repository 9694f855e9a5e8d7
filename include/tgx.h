/*
 * tgx.h -- C ABI of the GB300 voxel ray-tracing passes for tg's data model.
 *
 * Plain C99, no CUDA or C++ types in any signature.  The engine's C host code
 * calls these where tg's Vulkan raytracer sat:
 *
 *   tg_raytracer_create            (tgvk_raytracer.c:662)   -> tgx_create
 *   tg_raytracer_destroy           (tgvk_raytracer.c:791)   -> tgx_destroy
 *   tg_raytracer_create_object     (tgvk_raytracer.c:805)   -> tgx_scene_upload (whole scene store)
 *   tg_raytracer_color_lut_set     (tgvk_raytracer.c:1122)  -> tgx_scene_desc.luts
 *   tg_raytracer_clear             (tgvk_raytracer.c:1556)  -> fused into tgx_vis_render
 *   tg_raytracer_render            (tgvk_raytracer.c:1144)  -> tgx_svo_build + tgx_vis_render (+ tgx_gi_render)
 *   tg_raytracer_get_hovered_voxel (tgvk_raytracer.c:1605)  -> tgx_pick
 *   tg_svo_create                  (tg_sparse_voxel_octree.c:466) -> tgx_svo_build
 *   tg_svo_traverse                (tg_sparse_voxel_octree.c:558; GPU form svo_functions.inc:1-329) -> tgx_svo_trace
 *
 * Data model (unchanged from tg):
 *   - an object carries its clusters per axis, its first cluster pointer, a
 *     translation and a rotation (tg_object_data_ssbo, tgvk_raytracer.c:35-42);
 *   - cluster pointers map to 31-bit cluster indices (tgvk_raytracer.h:98-100);
 *   - a cluster is 8^3 one-bit voxels, 16 u32 words, bit 64z+8y+x
 *     (visibility.frag:143-148), voxel indices are 9 bits;
 *   - materials are 8-bit indices (512 B per cluster, byte v of cluster c at
 *     offset 512c+v, shading.frag:128-131) into 256-entry LUTs.
 *
 * Errors: every call returns a tgx_status and never aborts.  Device-side
 * failures (step budget exhausted, capacity exceeded, bad index) are recorded
 * in a device status word read by tgx_last_device_error after tgx_sync.
 *
 * Threading: one context per host thread; calls are ordered on the context's
 * stream and are asynchronous until tgx_sync unless stated otherwise.
 */
#ifndef TGX_H
#define TGX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TGX_ABI_VERSION                 1u

#define TGX_CLUSTER_SIDE                8u      /* TG_N_PRIMITIVES_PER_CLUSTER_CUBE_ROOT, cluster.inc:3 */
#define TGX_VOXELS_PER_CLUSTER          512u    /* TG_N_PRIMITIVES_PER_CLUSTER, cluster.inc:2 */
#define TGX_CLUSTER_WORDS               16u     /* 512 bits as u32 */
#define TGX_CLUSTER_MATERIAL_BYTES      512u    /* TG_CLUSTER_SIZE(8) */
#define TGX_CLUSTER_IDX_BITS            31u     /* TG_CLUSTERS_IDX_N_BITS, cluster.inc:4 */
#define TGX_LUT_ENTRIES                 256u
#define TGX_SVO_BLOCK_SIDE              32u     /* TG_SVO_BLOCK_SIDE_LENGTH, svo.inc:2 */
#define TGX_SVO_BLOCK_WORDS             1024u   /* 32^3 bits as u32, bit 1024z+32y+x */

/* Empty visibility-buffer word: depth field 2^24-1 means "no hit"
 * (shading.frag:118-122; clear.comp:19 intends all ones). */
#define TGX_VIS_EMPTY                   UINT64_MAX

typedef enum tgx_status
{
    TGX_OK                      = 0,
    TGX_ERR_INVALID_ARGUMENT    = 1,
    TGX_ERR_OUT_OF_MEMORY       = 2,
    TGX_ERR_CUDA                = 3,   /* a CUDA runtime call failed; see tgx_last_error_string */
    TGX_ERR_CAPACITY            = 4,   /* a fixed capacity would be exceeded */
    TGX_ERR_TIMEOUT             = 5,   /* a device loop ran out of its step budget */
    TGX_ERR_NOT_SUPPORTED       = 6,
    TGX_ERR_NO_DEVICE           = 7,
    TGX_ERR_DEVICE_FAULT        = 8    /* a kernel recorded a bounds or consistency error */
} tgx_status;

/* Object record, 96 bytes, identical to tg_object_data_ssbo
 * (tgvk_raytracer.c:35-42, buffers.inc:6-13, std430). */
typedef struct tgx_object
{
    uint32_t n_cluster_pointers_per_dim[3];
    uint32_t first_cluster_pointer;
    float    translation[3];
    uint32_t lut_idx;          /* the reference's `pad` word; the reference always
                                  writes 0 and has one global LUT (tgvk_raytracer.c:1124) */
    float    rotation[16];     /* column-major 4x4, as tg's m4 (tg_math.h:240-275) */
} tgx_object;

/* Camera of one view: tg_camera_ubo (tgvk_raytracer.c:65-74) plus the
 * visibility-buffer size header (tgvk_raytracer.c:76-81).  Corner rays are
 * the normalised directions tg_camera_make_corner_ray_directions computes on
 * the host (tgvk_core.c:435-444); the fourth component is ignored. */
typedef struct tgx_view
{
    float    camera[4];
    float    ray_bl[4];
    float    ray_br[4];
    float    ray_tr[4];
    float    ray_tl[4];
    float    near_plane;
    float    far_plane;
    uint32_t width;
    uint32_t height;
} tgx_view;

/* One LUT entry: linear albedo and roughness (16 bytes). */
typedef struct tgx_material
{
    float albedo[3];
    float roughness;
} tgx_material;

/* Host-side scene store, the arrays of tg_scene (tgvk_raytracer.h:90-108)
 * plus the material grid and LUTs.  tgx_scene_upload copies everything; the
 * caller keeps ownership of its host memory. */
typedef struct tgx_scene_desc
{
    uint32_t             n_objects;
    const tgx_object*    objects;                    /* [n_objects] */
    uint32_t             n_cluster_pointers;
    const uint32_t*      cluster_pointers;           /* [n_cluster_pointers] -> cluster idx */
    uint32_t             n_clusters;
    const uint32_t*      cluster_idx_to_object_idx;  /* [n_clusters] */
    const uint32_t*      voxel_bits;                 /* [n_clusters * 16] */
    const uint8_t*       material_idx;               /* [n_clusters * 512] or NULL */
    uint32_t             n_luts;
    const tgx_material*  luts;                       /* [n_luts * 256] or NULL */
} tgx_scene_desc;

typedef struct tgx_config
{
    int      device;           /* CUDA device ordinal */
    void*    stream;           /* cudaStream_t to run on, or NULL for a context-owned stream */
    uint32_t tile_w;           /* visibility tile width in pixels (0 = default 16); */
    uint32_t tile_h;           /* and height (0 = 16): 32..512 pixels, a whole number of warps */
    uint32_t flags;            /* TGX_FLAG_* bits, 0 for defaults */
    uint32_t trace_steps;      /* SVO traversal: DDA steps a lane runs between refills of the
                                  ray queue (1..256, 0 = default 8); see tgx_set_trace_steps */
} tgx_config;

/* Keeps the visibility bin storage at its minimum (64 entries) so frames
 * overflow it and take the exact record-scan path; for testing that path. */
#define TGX_FLAG_MIN_BIN_CAPACITY       1u
/* Test of the device-side timeout path: the first bitmask batch of every
 * visibility tile waits for 64 bytes more than it copies, so its bounded wait
 * (about one second) runs out.  The tile then stops staging, the frame's
 * pixels are incomplete, and tgx_last_device_error reports TGX_ERR_TIMEOUT
 * (where = 5).  Nothing faults; the context stays usable.  Never set it
 * outside such a test. */
#define TGX_FLAG_TEST_LOST_COPY         2u

typedef struct tgx_device_error
{
    uint32_t code;             /* tgx_status of the first device-side error, 0 if none */
    uint32_t where;            /* kernel-specific location code */
    uint64_t detail;           /* offending index or value */
} tgx_device_error;

typedef struct tgx_ctx   tgx_ctx;
typedef struct tgx_scene tgx_scene;
typedef struct tgx_svo   tgx_svo;

/* ---- context ---- */

uint32_t    tgx_abi_version(void);
const char* tgx_status_string(tgx_status status);
/* Text of the last host-side error of this thread (CUDA message, argument name). */
const char* tgx_last_error_string(void);

tgx_status  tgx_create(const tgx_config* config, tgx_ctx** out_ctx);
void        tgx_destroy(tgx_ctx* ctx);
/* The SVO traversal's DDA steps per lane between refills of its ray queue
 * (1..256): fewer refill idle lanes sooner, more amortise the refill.  The
 * autotuner (tg_gb300/autotune.py) picks it per scene; default 8. */
tgx_status  tgx_set_trace_steps(tgx_ctx* ctx, uint32_t steps);
/* The cudaStream_t the context launches on (as void*). */
void*       tgx_stream(tgx_ctx* ctx);
tgx_status  tgx_sync(tgx_ctx* ctx);
/* Reads and clears the device status word (synchronises the stream). */
tgx_status  tgx_last_device_error(tgx_ctx* ctx, tgx_device_error* out_error);
/* Number of kernels this context has launched so far. */
uint64_t    tgx_launch_count(tgx_ctx* ctx);

/*
 * Per-kernel device timing (tracing).  While enabled, every kernel the context
 * launches is bracketed by CUDA events on its stream.  tgx_trace_get
 * synchronises and returns, for kernel slot `slot` (0 .. tgx_trace_slots()-1),
 * its name, summed device milliseconds and launch count since the last reset.
 * Stands in for tg's QPC frame timer (tg_platform_win32.c:520-570), which has
 * no per-pass GPU timestamps.
 */
tgx_status  tgx_trace_enable(tgx_ctx* ctx, int enable);
tgx_status  tgx_trace_reset(tgx_ctx* ctx);
uint32_t    tgx_trace_slots(void);
tgx_status  tgx_trace_get(tgx_ctx* ctx, uint32_t slot, const char** out_name, double* out_ms,
                          uint64_t* out_launches);

/* ---- scene ---- */

/* Copies a host scene store to the device (blocking).  Replaces the
 * per-object staging uploads of tg_raytracer_create_object
 * (tgvk_raytracer.c:849-978). */
tgx_status  tgx_scene_upload(tgx_ctx* ctx, const tgx_scene_desc* desc, tgx_scene** out_scene);
void        tgx_scene_destroy(tgx_ctx* ctx, tgx_scene* scene);

/* ---- visibility buffer (visibility.vert/.frag + clear.comp) ---- */

/*
 * Renders the visibility buffer of each view: every pixel gets the minimum
 * over all clusters of depth(24)|cluster pointer(31)|voxel(9), exactly as
 * visibility.frag:22-207 computes it per fragment, or TGX_VIS_EMPTY.
 * d_visbuf[i] is a DEVICE pointer to views[i].width*views[i].height u64.
 * The clear of clear.comp is fused in.  Asynchronous on the context stream.
 */
tgx_status  tgx_vis_render(tgx_ctx* ctx, const tgx_scene* scene, const tgx_view* views, uint32_t n_views,
                           uint64_t* const* d_visbuf);

/* Same as tgx_vis_render but h_visbuf[i] are HOST pointers; the call copies
 * the views in and returns when the buffers are on the host.  A buffer in
 * pinned (page-locked) host memory is written by the render directly over the
 * CPU-GPU link, with no device copy; any other goes through a device buffer
 * and a copy. */
tgx_status  tgx_vis_render_host(tgx_ctx* ctx, const tgx_scene* scene, const tgx_view* views, uint32_t n_views,
                                uint64_t* const* h_visbuf);

/* Pipelined form of tgx_vis_render_host for frame loops that read every
 * frame back: enqueues the frame and returns without waiting.  Pinned host
 * buffers are written by the render directly.  Other buffers are copied on a
 * second stream, so frame k's copy overlaps frame k+1's render; the library
 * keeps two device copies of them and holds a render back until the copy two
 * frames before it has finished.  A frame's host buffers must not be touched
 * until tgx_vis_host_wait says the frame is done.  Errors of the call come
 * back from it; device errors from tgx_last_device_error. */
tgx_status  tgx_vis_render_host_async(tgx_ctx* ctx, const tgx_scene* scene, const tgx_view* views, uint32_t n_views,
                                      uint64_t* const* h_visbuf);
/* Waits until at most `max_in_flight` frames of tgx_vis_render_host_async are
 * still being rendered or copied (0: all of them are on the host).  Frames
 * complete in issue order. */
tgx_status  tgx_vis_host_wait(tgx_ctx* ctx, uint32_t max_in_flight);

/*
 * Visibility render that allocates nothing.  No counterpart in the reference:
 * tg always owns its Vulkan buffers.  It exists for callers that cannot call
 * cudaMalloc -- an engine or plugin host that owns every device allocation
 * through its own allocator or a fixed memory budget, or code that must not
 * risk the device-wide synchronisation cudaMalloc/cudaFree can cause.  Needs
 * no tgx_ctx (tgx_create allocates).
 *
 * The caller passes the scene as DEVICE arrays with the tgx_scene_desc layout
 * (objects, cluster pointers, cluster->object map, voxel bits; indices are
 * trusted, not validated), the view on the host, and a DEVICE output of
 * width*height u64.  The result equals tgx_vis_render's bit for bit.  All
 * scratch lives in one fixed device array of about 51 MiB inside the library,
 * which every GPU that loads the library holds until the process exits.
 * Limits: at most 65,536 objects, 524,288 cluster pointers and 32,768 screen
 * tiles of 16x16 pixels (3840x2160 fits); larger inputs are rejected with
 * TGX_ERR_CAPACITY and a message.  The tile bins hold 262,144 (cluster,
 * tile) entries; a frame that needs more is still rendered exactly, but every
 * tile then tests every visible cluster's screen rectangle, which is much
 * slower (tgx_vis_render grows its bins instead).  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress, once per device,
 * with that device current), so make that first call before any stream
 * capture.  The view and the output pointer are handed to the GPU by value in
 * a kernel's arguments: no host buffer is read after the call returns.  Every
 * call shares the one array and reuses what the previous call left in it
 * (what must start at zero is cleared by each call), so calls whose work
 * overlaps on the GPU (other streams, other host threads) race; serialise
 * them.  Runs on `stream` (a cudaStream_t, or NULL for the legacy default
 * stream) and returns without waiting, unless out_error is non-NULL: then it
 * synchronises the stream and reports the device status word.
 */
tgx_status  tgx_vis_render_noalloc(void* stream, const tgx_object* d_objects, uint32_t n_objects,
                                   const uint32_t* d_cluster_pointers, uint32_t n_cluster_pointers,
                                   const uint32_t* d_cluster_idx_to_object_idx, const uint32_t* d_voxel_bits,
                                   const tgx_view* view, uint64_t* d_visbuf, tgx_device_error* out_error);

/* Counters of the last tgx_vis_render on this context (blocking). */
typedef struct tgx_vis_stats
{
    uint32_t visible_clusters;    /* non-empty clusters inside some view's frustum */
    uint32_t bin_entries;         /* (tile, cluster) pairs binned */
    uint32_t tiles;               /* screen tiles over all views */
    uint32_t dda_overruns;        /* DDAs that exceeded their step bound (always 0 unless a bug) */
} tgx_vis_stats;

tgx_status  tgx_vis_get_stats(tgx_ctx* ctx, tgx_vis_stats* out_stats);

/* A device-memory budget for the scene stores of this context (uploaded or
 * generated): an upload or generation that would take the live stores past
 * `bytes` fails with TGX_ERR_OUT_OF_MEMORY and a message, frees what it had
 * allocated, and leaves the context usable, like a real allocation failure.
 * 0 removes the limit (the default).  For an engine that runs under a fixed
 * memory budget; the reference only asserts that an allocation succeeded
 * (tg_memory.c:61).  tgx_get_memory reports the budget and the bytes held. */
tgx_status  tgx_set_memory_budget(tgx_ctx* ctx, uint64_t bytes);
tgx_status  tgx_get_memory(tgx_ctx* ctx, uint64_t* out_budget, uint64_t* out_scene_bytes);

/* Tuning of the visibility pass on this context (0 keeps a default):
 *   depth_buckets  8, 16 (default) or 32 depth buckets per screen tile: a
 *                  tile's clusters are sorted into them near to far, so a
 *                  tile can stop once every pixel is nearer than what is left;
 *   batch          clusters staged per shared-memory batch, 1..48 (48);
 *   drain          (pixel, cluster) pairs a warp collects before its lanes
 *                  run their DDAs, 1..32 (32).
 * The result never depends on them (bit for bit); tg_gb300/autotune.py picks
 * them per workload.  No counterpart in the reference. */
tgx_status  tgx_set_vis_tuning(tgx_ctx* ctx, uint32_t depth_buckets, uint32_t batch, uint32_t drain);

/* Work done by the visibility tile kernel, counted by the kernel itself.  No
 * counterpart in the reference (its GPU work is counted by nobody).  After
 * tgx_vis_count_work(ctx, 1) every tgx_vis_render on the context runs a
 * counting variant of the tile kernel (same results, a little slower) and
 * overwrites these totals; tgx_vis_get_work reads them (blocking).  A
 * (pixel, cluster) pair is one binned cluster evaluated for one pixel. */
typedef struct tgx_vis_work
{
    uint64_t pairs;               /* pairs evaluated: past the per-pixel depth skip */
    uint64_t depth_skips;         /* pairs skipped: the pixel already holds a nearer word */
    uint64_t dir_setups;          /* cluster-space ray directions computed (per pixel and object) */
    uint64_t slab_misses;         /* pairs the conservative slab test rejects */
    uint64_t sure_hits;           /* pairs whose box entry is certain (entry distance only) */
    uint64_t exact_tests;         /* pairs that run the shader's full ray/box test */
    uint64_t ddas;                /* pairs that run the voxel DDA */
    uint64_t dda_steps;           /* voxels visited by those DDAs */
    uint64_t hits;                /* DDAs that found a set voxel */
    uint64_t batches;             /* (pixel, staged batch) visits */
} tgx_vis_work;

tgx_status  tgx_vis_count_work(tgx_ctx* ctx, int enable);
tgx_status  tgx_vis_get_work(tgx_ctx* ctx, tgx_vis_work* out_work);

/* Decodes one visibility-buffer word like tg_raytracer_get_hovered_voxel
 * (tgvk_raytracer.c:1639-1653): returns 1 on hit.  Host-only, no device work. */
int         tgx_vis_decode(uint64_t packed, float* out_depth, uint32_t* out_cluster_pointer, uint32_t* out_voxel_idx);

/* Reads pixel (x, y) of a device visibility buffer of width w and decodes it
 * (tg_raytracer_get_hovered_voxel, tgvk_raytracer.c:1605-1655).  Blocking. */
tgx_status  tgx_pick(tgx_ctx* ctx, const uint64_t* d_visbuf, uint32_t w, uint32_t h, uint32_t x, uint32_t y,
                     float* out_depth, uint32_t* out_cluster_pointer, uint32_t* out_voxel_idx, int* out_hit);

/* ---- shading pass (shading.frag) ---- */

/* Modes of tgx_shade, numbered like the reference's debug views (shading.frag:16-25). */
#define TGX_SHADE_NONE                  0u   /* direct GGX shading with the LUT albedo */
#define TGX_SHADE_OBJECT_INDEX          1u
#define TGX_SHADE_DEPTH                 2u
#define TGX_SHADE_CLUSTER_INDEX         3u
#define TGX_SHADE_VOXEL_INDEX           4u
#define TGX_SHADE_BLOCKS                5u
#define TGX_SHADE_COLOR_LUT_INDEX       6u
#define TGX_SHADE_COLOR                 7u
#define TGX_SHADE_NORMAL                8u
#define TGX_SHADE_SHADING               9u   /* direct shading with white albedo */

/*
 * Shades a visibility buffer the way tg's shading.frag:116-316 does: per pixel
 * the primary surface (face normal from the voxel box), the voxel's LUT
 * albedo, GGX/Smith/Schlick direct light from normalize(0, 0.8, 0.3) with
 * radiance 3, metallic 0.1, roughness 0.8, plus 0.1 * albedo ambient; or one
 * of the debug views.  Sky pixels are magenta.  Writes RGBA, 4 floats per
 * pixel, to d_rgba (DEVICE).  Asynchronous.
 */
tgx_status  tgx_shade(tgx_ctx* ctx, const tgx_scene* scene, const tgx_view* view, const uint64_t* d_visbuf,
                      uint32_t mode, float* d_rgba);

/* ---- batched frames captured as a CUDA graph ---- */

/* One job of a batched frame: n_views views (any resolutions) of one scene. */
typedef struct tgx_vis_job
{
    const tgx_scene*    scene;
    const tgx_view*     views;        /* [n_views] */
    uint32_t            n_views;
    uint64_t* const*    d_visbuf;     /* [n_views] DEVICE outputs, width*height words each */
} tgx_vis_job;

typedef struct tgx_frame_graph tgx_frame_graph;

/*
 * Captures the visibility passes of n_jobs jobs (several scenes, many views of
 * uneven resolution) once into a CUDA graph, so a whole batched frame replays
 * with one tgx_frame_graph_launch.  The graph owns its scratch and its copies
 * of the view tables and output pointers; the scenes and outputs must outlive
 * it.  Creation renders every job once, uncaptured, to size the bins (a
 * replayed frame that still overflows them takes the exact record scan).
 * Synchronous.
 */
tgx_status  tgx_frame_graph_create(tgx_ctx* ctx, const tgx_vis_job* jobs, uint32_t n_jobs,
                                   tgx_frame_graph** out_graph);
/* Replays the frame on the context stream.  Asynchronous. */
tgx_status  tgx_frame_graph_launch(tgx_ctx* ctx, tgx_frame_graph* graph);
/* New cameras for job `job` (same count and resolutions); ordered before later launches. */
tgx_status  tgx_frame_graph_set_views(tgx_ctx* ctx, tgx_frame_graph* graph, uint32_t job, const tgx_view* views);
/* Kernels one launch of the graph runs. */
uint32_t    tgx_frame_graph_kernels(const tgx_frame_graph* graph);
void        tgx_frame_graph_destroy(tgx_ctx* ctx, tgx_frame_graph* graph);

/* ---- one-bit SVO (tg_sparse_voxel_octree.c) ---- */

/*
 * Builds the one-bit voxel set tg_svo_create (tg_sparse_voxel_octree.c:466-542)
 * defines over the cube [min, min + 2^extent_log2)^3 (extent_log2 in 6..14;
 * the reference fixes it at 10): a world voxel is set iff some cluster that
 * passes the reference's recursive OBB/AABB test for every node on the path to
 * the voxel's 32^3 block samples a set bit at the voxel centre.  The result is
 * stored as a dense block table, a pool of 32^3-bit blocks and an occupancy
 * pyramid (see tgx_svo_info).  Asynchronous; the pool capacity is sized from
 * the scene and grown (blocking) when exceeded.
 */
tgx_status  tgx_svo_build(tgx_ctx* ctx, const tgx_scene* scene, const float min[3], uint32_t extent_log2,
                          tgx_svo** out_svo);

/* Leaves out the per-voxel material codes (2 bytes per voxel of every
 * allocated 32^3 block, i.e. 64 KiB per block); GI then shades with grey
 * albedo.  For extents where that grid would not fit. */
#define TGX_SVO_NO_MATERIALS            1u
/* tgx_svo_build with TGX_SVO_* flags. */
tgx_status  tgx_svo_build_flags(tgx_ctx* ctx, const tgx_scene* scene, const float min[3], uint32_t extent_log2,
                                uint32_t flags, tgx_svo** out_svo);
void        tgx_svo_destroy(tgx_ctx* ctx, tgx_svo* svo);

/*
 * Brings an SVO up to date with the scene's current object records after
 * tgx_scene_set_objects moved objects -- the incremental insert the reference
 * intends but leaves commented out (tg_svo_insert_object,
 * tgvk_raytracer.c:982-989; README.md:48).  Objects whose record differs from
 * the one the SVO last saw are "moved"; every 32^3 block one of their
 * non-empty clusters could touch before or after the move is cleared and
 * rebuilt from all clusters, so the voxel set, materials, block counts and
 * pyramid equal those of a fresh tgx_svo_build of the moved scene.  Blocks
 * that end up empty return their slots to a free list the next update reuses;
 * the pool grows (blocking) when it runs out.  `scene` must have the object and
 * cluster-pointer counts of the build.  Blocks the host once for the counts.
 * *out_n_moved (may be NULL) receives the number of moved objects.
 */
tgx_status  tgx_svo_update(tgx_ctx* ctx, tgx_svo* svo, const tgx_scene* scene, uint32_t* out_n_moved);

typedef struct tgx_svo_info
{
    float    min[3];
    uint32_t extent_log2;
    uint32_t blocks_per_axis;     /* 2^(extent_log2-5) */
    uint32_t n_blocks;            /* allocated 32^3 blocks (candidates) */
    uint32_t n_nonempty_blocks;   /* blocks with at least one voxel set */
    uint32_t n_pairs;             /* (cluster, block) pairs the last build or update voxelised */
    uint64_t device_bytes;        /* table + pool + pyramid */
} tgx_svo_info;

tgx_status  tgx_svo_get_info(tgx_ctx* ctx, const tgx_svo* svo, tgx_svo_info* out_info);

/*
 * Copies the non-empty blocks to the host, sorted by block index
 * (bz*B*B + by*B + bx): out_block_xyz[3i..3i+2] = world min corner of block i,
 * out_words[1024i..] its bits (1024z+32y+x).  Returns the block count in
 * *out_n (blocks beyond capacity are counted, not written).  Blocking.
 */
tgx_status  tgx_svo_download(tgx_ctx* ctx, const tgx_svo* svo, int32_t* out_block_xyz, uint32_t* out_words,
                             uint32_t capacity, uint32_t* out_n);

/*
 * Traces n rays (device arrays of float3 origin and direction, world space)
 * through the SVO and writes, per ray, the hit distance t (FLT_MAX on miss)
 * and the world voxel coordinate (int3; undefined on miss).  At most
 * max_steps voxel/node steps per ray; a ray that exhausts them is reported as
 * a miss and counted in the device status word.  Asynchronous.
 */
tgx_status  tgx_svo_trace(tgx_ctx* ctx, const tgx_svo* svo, uint32_t n, const float* d_origins,
                          const float* d_dirs, uint32_t max_steps, float* d_t, int32_t* d_voxel);

/* ---- bounce lighting (new: the reference shades direct light only, shading.frag:285-316) ---- */

typedef struct tgx_gi_params
{
    uint32_t spp;               /* cosine-weighted secondary rays per pixel */
    uint32_t bounces;           /* 1..4 */
    uint32_t max_steps;         /* SVO steps per traced ray, 0 = 256 */
    uint32_t frame;             /* Philox counter word: decorrelates frames */
    uint64_t seed;              /* Philox key */
    float    sun_dir[3];        /* unit vector toward the sun */
    float    sun_radiance[3];
    float    sky_radiance[3];
    float    offset;            /* ray origins move this far (voxels) along the normal */
} tgx_gi_params;

/*
 * Plain GI for one view from its visibility buffer (d_visbuf, DEVICE, as
 * tgx_vis_render wrote it) and the SVO: per pixel, direct sun light with an
 * SVO shadow ray plus `spp` cosine-weighted bounce paths through the SVO
 * (`bounces` deep, a sun shadow ray at every hit), Lambertian albedo from the
 * material LUTs (0.5 grey when the scene has none).  The spp directions of a
 * pixel are a stratified point set (R2 sequence, rotated per pixel and bounce
 * by Philox4x32-10 keyed by `seed`, `frame`).  Writes linear RGB, 3 floats per
 * pixel, to d_rgb (DEVICE).  Rays that run out of max_steps count as misses
 * and are counted in the device status.  Asynchronous; scratch grows in the
 * context (at most 16 M paths in flight).
 */
tgx_status  tgx_gi_render(tgx_ctx* ctx, const tgx_scene* scene, const tgx_svo* svo, const tgx_view* view,
                          const uint64_t* d_visbuf, const tgx_gi_params* params, float* d_rgb);

/* ---- learned radiance cache (new: the reference has no learned component) ---- */

/*
 * A small MLP mapping (position normalised to [0,1]^3, normal, direction) to
 * RGB radiance: 9 inputs -> 216 sin/cos features (12 octaves of pi) -> 4 ReLU
 * layers of 64 -> 3 outputs, no biases.  BF16 weights and activations with
 * FP32 accumulation on the tensor cores, FP32 master weights and Adam.
 * Inputs are n x 9 floats, outputs n x 3 floats, all DEVICE memory.
 */
typedef struct tgx_cache tgx_cache;

uint32_t    tgx_cache_n_params(void);
tgx_status  tgx_cache_create(tgx_ctx* ctx, uint64_t seed, tgx_cache** out_cache);
void        tgx_cache_destroy(tgx_ctx* ctx, tgx_cache* cache);
tgx_status  tgx_cache_infer(tgx_ctx* ctx, tgx_cache* cache, uint32_t n, const float* d_x, float* d_rgb);
/* One Adam step (lr, beta 0.9/0.99) on the relative-L2 loss of a batch. */
tgx_status  tgx_cache_train_step(tgx_ctx* ctx, tgx_cache* cache, uint32_t n, const float* d_x, const float* d_target,
                                 float lr);
/* Batch loss of the last training step or gradient call (blocking). */
tgx_status  tgx_cache_last_loss(tgx_ctx* ctx, const tgx_cache* cache, float* out_loss);
/* The batch gradient without an update, to HOST memory (blocking); for checking. */
tgx_status  tgx_cache_gradient(tgx_ctx* ctx, tgx_cache* cache, uint32_t n, const float* d_x, const float* d_target,
                               float* out_grad, float* out_loss);
/* FP32 master weights as one HOST array of tgx_cache_n_params() floats, in the
 * order W0 [64][216], W1, W2, W3 [64][64], W4 [3][64] (row-major [out][in]). */
tgx_status  tgx_cache_get_weights(tgx_ctx* ctx, const tgx_cache* cache, float* out_w);
tgx_status  tgx_cache_set_weights(tgx_ctx* ctx, tgx_cache* cache, const float* w);
/* Checkpoint and resume: weights, Adam moments and step count. */
tgx_status  tgx_cache_save(tgx_ctx* ctx, const tgx_cache* cache, const char* path);
tgx_status  tgx_cache_load(tgx_ctx* ctx, tgx_cache* cache, const char* path);

/* Online learned-cache GI settings (tgx_gi_render_cached). */
typedef struct tgx_cache_gi_params
{
    uint32_t n_train;           /* training samples per frame (65,536) */
    uint32_t train_spp;         /* SVO paths per training target (16) */
    uint32_t train_steps;       /* Adam steps per frame, n_train / train_steps samples each */
    float    lr;                /* Adam learning rate (1e-2) */
    float    box_min[3];        /* scene box: positions are normalised by it for the cache */
    float    box_max[3];
    float    primary_weight;    /* 0..1: largest share of a pixel's incoming light taken from the
                                   cache's pixel-point network instead of its samples (0: off) */
    uint32_t n_train_primary;   /* training samples of the pixel-point network per frame (0) */
    float    primary_variance_scale; /* multiplies the samples' variance v in the shrinkage weight
                                   (0 = the default, 0.5) */
} tgx_cache_gi_params;

/*
 * GI whose bounce paths end in the learned cache: as tgx_gi_render, but each
 * bounce ray that hits returns the hit voxel's albedo times the cache's
 * prediction of the demodulated radiance (outgoing radiance / albedo) leaving
 * that point toward the shading point, instead of tracing on.  Then trains
 * the cache online on this frame: picks n_train bounce hits, estimates their
 * demodulated outgoing radiance with train_spp plain SVO paths (`bounces` - 1
 * further bounces, direct sun at every hit) and runs train_steps Adam steps.
 * The cache also holds a second network for the pixels' own surface points.
 * It is trained (n_train_primary random pixels per frame, no extra paths) on
 * each pixel's sample mean m of incoming light.  With primary_weight w > 0 a
 * pixel's incoming light becomes m + k (P - m), P the network's prediction.
 * With one sample k = w.  With spp > 1, k = min(w, s v / (s v + b)): b is
 * the network's squared error over the pixel's 13x13 neighbourhood (mean
 * |P - m|^2 less mean variance of m), v the variance of m, its own estimate
 * mixed with the neighbourhood's as (spp - 1) : 1/2, and s =
 * primary_variance_scale; both relative to the pixel's predicted brightness.
 * The prediction counts where the network is accurate around the pixel and
 * the pixel's samples are noisy.  Asynchronous; all buffers DEVICE memory.
 */
tgx_status  tgx_gi_render_cached(tgx_ctx* ctx, const tgx_scene* scene, const tgx_svo* svo, tgx_cache* cache,
                                 const tgx_view* view, const uint64_t* d_visbuf, const tgx_gi_params* params,
                                 const tgx_cache_gi_params* cache_params, float* d_rgb);

/* SVO traversal work of the last tgx_gi_render / tgx_gi_render_cached call on
 * this context, counted by the traversal kernel itself (every ray it traced:
 * bounce, shadow and training rays; one step = one hierarchical-DDA iteration,
 * with the bottom-up start counted like the descent it replaces).  No
 * counterpart in the reference, which has no GI pass.  Blocking. */
typedef struct tgx_gi_work
{
    uint64_t dda_steps;
    uint64_t rays;
} tgx_gi_work;

tgx_status  tgx_gi_get_work(tgx_ctx* ctx, tgx_gi_work* out_work);

/* ---- synthetic scenes (the reference's CPU noise loop, tgvk_raytracer.c:870-978) ---- */

typedef struct tgx_gen_params
{
    uint32_t kind;               /* 0: one object, Bernoulli bits; 1: many objects, value-noise bits */
    uint32_t n_objects;
    uint32_t min_clusters_per_axis;
    uint32_t max_clusters_per_axis;
    float    bernoulli_p;        /* kind 0 */
    float    noise_period;       /* kind 1, lattice spacing in voxels */
    float    noise_threshold;    /* kind 1 */
    uint64_t seed;
    float    box_min[3];         /* translations uniform in [box_min, box_max) (kind 1; kind 0 when not empty) */
    float    box_max[3];
    float    fixed_translation[3]; /* kind 0 with an empty box */
    uint32_t n_luts;
    uint32_t threads;            /* host threads, 0 = all */
} tgx_gen_params;

typedef struct tgx_gen_scene
{
    tgx_scene_desc desc;         /* points into the arrays below */
    tgx_object*    objects;
    uint32_t*      cluster_pointers;
    uint32_t*      cluster_idx_to_object_idx;
    uint32_t*      voxel_bits;
    uint8_t*       material_idx;
    tgx_material*  luts;
} tgx_gen_scene;

tgx_status  tgx_generate_scene(const tgx_gen_params* params, tgx_gen_scene* out_scene);
void        tgx_free_generated_scene(tgx_gen_scene* scene);

/*
 * The same scene built directly in device memory (the reference's "TODO: gen
 * on GPU", tgvk_raytracer.c:868): object records on the host, every cluster's
 * bits and material bytes by one GPU thread per voxel.  Equal byte for byte to
 * tgx_generate_scene + tgx_scene_upload, without the host arrays.  Synchronous.
 */
tgx_status  tgx_generate_scene_device(tgx_ctx* ctx, const tgx_gen_params* params, tgx_scene** out_scene);

/* Sizes of a scene's arrays (any argument may be NULL). */
tgx_status  tgx_scene_counts(const tgx_scene* scene, uint32_t* n_objects, uint32_t* n_cluster_pointers,
                             uint32_t* n_clusters, uint32_t* n_luts);
/*
 * Replaces the records of objects first .. first+n-1 with HOST records that
 * keep each object's cluster layout (first_cluster_pointer and
 * n_cluster_pointers_per_dim) and change its pose (translation, rotation) or
 * LUT: the reference's per-frame object transform write.  Later visibility,
 * shading and GI launches see the new poses; an SVO follows after
 * tgx_svo_update.  Synchronous.
 */
tgx_status  tgx_scene_set_objects(tgx_ctx* ctx, tgx_scene* scene, uint32_t first, uint32_t n, const tgx_object* objects);

/* Copies a scene's arrays back to HOST buffers sized by tgx_scene_counts (NULL skips an array). */
tgx_status  tgx_scene_download(tgx_ctx* ctx, const tgx_scene* scene, tgx_object* objects, uint32_t* cluster_pointers,
                               uint32_t* cluster_idx_to_object_idx, uint32_t* voxel_bits, uint8_t* material_idx,
                               tgx_material* luts);

/* Pinhole view from a position, yaw/pitch (radians) and vertical field of
 * view, with tg's corner-ray construction (tgvk_core.c:382-444): view
 * rotation inverse(euler(pitch, yaw, 0)), projection tgm_m4_perspective,
 * corners inverse(P*R) * (+-1, +-1, 1, 1), normalised. */
tgx_status  tgx_make_view(const float position[3], float pitch, float yaw, float fov_y, uint32_t width,
                          uint32_t height, float near_plane, float far_plane, tgx_view* out_view);

#ifdef __cplusplus
}
#endif

#endif /* TGX_H */
