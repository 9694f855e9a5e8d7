/*
 * Driver around the reference's own CPU code (tg_sparse_voxel_octree.c,
 * tg_physics.c, tg_amanatides_woo.c, tg_math.c), compiled from the reference
 * sources by oracle/build_ref.sh into oracle/_ref/libtgref.so.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests load this library through ctypes to pin the
 * C restatements in oracle/*.c (and through them the CUDA kernels) against
 * the reference's own arithmetic.  Nothing in the product links or calls it.
 *
 * Entry points take flat arrays so Python can drive them:
 *   tgref_svo_build      tg_svo_create   (tg_sparse_voxel_octree.c:466-542)
 *   tgref_svo_traverse   tg_svo_traverse (tg_sparse_voxel_octree.c:558-740)
 *   tgref_angle_axis     tgm_m4_angle_axis (tg_math.c:1870-1910)
 *   tgref_m4_inverse     tgm_m4_inverse  (tg_math.c:2185-2234)
 *   tgref_ray_aabb       tg_intersect_ray_aabb (tg_physics.c:394-406)
 *   tgref_aabb_obb       tg_intersect_aabb_obb_ignore_contact (tg_physics.c:226-392)
 *   tgref_amanatides_woo tg_amanatides_woo (tg_amanatides_woo.c:3-114)
 */
#include "graphics/tg_sparse_voxel_octree.h"
#include "graphics/vulkan/tgvk_raytracer.h"
#include "memory/tg_memory.h"
#include "physics/tg_physics.h"
#include "util/tg_amanatides_woo.h"

#include <setjmp.h>
#include <stdint.h>
#include <string.h>

/* ---- precondition failures of the reference ---- */

static jmp_buf g_assert_jmp;
static int     g_assert_armed = 0;
static char    g_assert_msg[512];

void tgref_assert_fail(const char* condition, const char* file, int line)
{
    snprintf(g_assert_msg, sizeof(g_assert_msg), "%s (%s:%d)", condition, file, line);
    if (g_assert_armed) longjmp(g_assert_jmp, 1);
    fprintf(stderr, "reference assertion failed: %s\n", g_assert_msg);
    abort();
}

/* Message of the last reference precondition that failed. */
const char* tgref_last_assert(void) { return g_assert_msg; }

/* ---- stand-ins for the reference's stack allocator and scene query ---- */

#define TGREF_STACK_DEPTH 4096
static void*   g_stack[TGREF_STACK_DEPTH];
static tg_size g_stack_size[TGREF_STACK_DEPTH];
static int     g_stack_top = 0;

void* tgref_stack_alloc(tg_size size)
{
    TG_ASSERT(g_stack_top < TGREF_STACK_DEPTH);
    void* p = calloc(1, size ? size : 1);
    TG_ASSERT(p != NULL);
    g_stack[g_stack_top] = p;
    g_stack_size[g_stack_top] = size;
    g_stack_top++;
    return p;
}

static void stack_reset(void)
{
    while (g_stack_top > 0) free(g_stack[--g_stack_top]);
}

void tgref_stack_free(tg_size size)
{
    TG_ASSERT(g_stack_top > 0);
    g_stack_top--;
    TG_ASSERT(g_stack_size[g_stack_top] == size);
    free(g_stack[g_stack_top]);
}

void tg_memory_nullify(tg_size size, void* p_memory) { memset(p_memory, 0, size); }

/* Same predicate as tgvk_raytracer.c:1069-1077. */
b32 tg_object_is_initialized(const tg_scene* p_scene, u32 object_idx)
{
    const tg_voxel_object* p = &p_scene->p_objects[object_idx];
    return p->n_cluster_pointers_per_dim.x != 0 && p->n_cluster_pointers_per_dim.y != 0 && p->n_cluster_pointers_per_dim.z != 0;
}

/* ---- helpers ---- */

static void m4_to_array(m4 m, float* out) { memcpy(out, m.p_data, 16 * sizeof(float)); }
static m4 m4_from_array(const float* in) { m4 m; memcpy(m.p_data, in, 16 * sizeof(float)); return m; }

void tgref_angle_axis(float angle, const float axis[3], float out_m4[16])
{
    m4_to_array(tgm_m4_angle_axis(angle, (v3){ axis[0], axis[1], axis[2] }), out_m4);
}

void tgref_m4_inverse(const float in_m4[16], float out_m4[16])
{
    m4_to_array(tgm_m4_inverse(m4_from_array(in_m4)), out_m4);
}

void tgref_m4_mul(const float a[16], const float b[16], float out_m4[16])
{
    m4_to_array(tgm_m4_mul(m4_from_array(a), m4_from_array(b)), out_m4);
}

int tgref_ray_aabb(const float o[3], const float d[3], const float mn[3], const float mx[3], float* enter, float* exit_)
{
    return tg_intersect_ray_aabb((v3){ o[0], o[1], o[2] }, (v3){ d[0], d[1], d[2] },
                                 (v3){ mn[0], mn[1], mn[2] }, (v3){ mx[0], mx[1], mx[2] }, enter, exit_);
}

int tgref_aabb_obb(const float mn[3], const float mx[3], const float corners[24])
{
    v3 c[8];
    for (int i = 0; i < 8; i++) c[i] = (v3){ corners[3 * i], corners[3 * i + 1], corners[3 * i + 2] };
    return tg_intersect_aabb_obb_ignore_contact((v3){ mn[0], mn[1], mn[2] }, (v3){ mx[0], mx[1], mx[2] }, c);
}

int tgref_amanatides_woo(const float hit[3], const float d[3], const float extent[3], const uint32_t* grid, int out_xyz[3])
{
    v3i id;
    b32 r = tg_amanatides_woo((v3){ hit[0], hit[1], hit[2] }, (v3){ d[0], d[1], d[2] },
                              (v3){ extent[0], extent[1], extent[2] }, grid, &id);
    out_xyz[0] = id.x; out_xyz[1] = id.y; out_xyz[2] = id.z;
    return r;
}

/* ---- SVO build ---- */

static tg_scene g_scene;
static float* g_node_min;
static void index_nodes(u32 node_idx, v3 mn, v3 mx);

/*
 * Builds the reference SVO over [mn, mn+1024]^3 from a scene given as the
 * CPU object records (angle/axis form, tg_graphics_core.h:266-273) plus the
 * cluster pointer, cluster->object and voxel bit arrays.  Keeps the SVO in a
 * static so tgref_svo_traverse can query it.  Returns the number of leaf
 * blocks with at least one voxel set, or -1 when one of the reference's own
 * assertions fails for this scene (tgref_last_assert names it).
 */
int tgref_svo_build(uint32_t n_objects, const uint32_t* obj_n_per_dim, const uint32_t* obj_first_ptr,
                    const float* obj_translation, const float* obj_angle, const float* obj_axis,
                    uint32_t n_cluster_pointers, const uint32_t* cluster_pointers,
                    const uint32_t* cluster_idx_to_object_idx, uint32_t n_clusters,
                    const uint32_t* voxel_bits, const float mn[3])
{
    if (g_scene.svo.p_node_buffer) tg_svo_destroy(&g_scene.svo);
    free(g_scene.p_objects);
    free(g_scene.p_cluster_pointers);
    free(g_scene.p_cluster_idx_to_object_idx);
    free(g_scene.p_voxel_cluster_data);
    memset(&g_scene, 0, sizeof(g_scene));

    g_scene.object_capacity = n_objects;
    g_scene.n_objects = n_objects;
    g_scene.p_objects = calloc(n_objects, sizeof(tg_voxel_object));
    for (uint32_t i = 0; i < n_objects; i++)
    {
        tg_voxel_object* p = &g_scene.p_objects[i];
        p->n_cluster_pointers_per_dim = (v3u){ obj_n_per_dim[3 * i], obj_n_per_dim[3 * i + 1], obj_n_per_dim[3 * i + 2] };
        p->first_cluster_pointer = obj_first_ptr[i];
        p->translation = (v3){ obj_translation[3 * i], obj_translation[3 * i + 1], obj_translation[3 * i + 2] };
        p->angle_in_radians = obj_angle[i];
        p->axis = (v3){ obj_axis[3 * i], obj_axis[3 * i + 1], obj_axis[3 * i + 2] };
    }
    g_scene.cluster_pointer_capacity = n_cluster_pointers;
    g_scene.n_cluster_pointers = n_cluster_pointers;
    g_scene.p_cluster_pointers = malloc((size_t)n_cluster_pointers * 4);
    memcpy(g_scene.p_cluster_pointers, cluster_pointers, (size_t)n_cluster_pointers * 4);
    g_scene.p_cluster_idx_to_object_idx = malloc((size_t)n_clusters * 4);
    memcpy(g_scene.p_cluster_idx_to_object_idx, cluster_idx_to_object_idx, (size_t)n_clusters * 4);
    g_scene.p_voxel_cluster_data = malloc((size_t)n_clusters * 64);
    memcpy(g_scene.p_voxel_cluster_data, voxel_bits, (size_t)n_clusters * 64);

    const v3 emin = { mn[0], mn[1], mn[2] };
    const v3 emax = { mn[0] + 1024.0f, mn[1] + 1024.0f, mn[2] + 1024.0f };
    g_assert_msg[0] = 0;
    g_assert_armed = 1;
    if (setjmp(g_assert_jmp))
    {
        /* the reference rejected this scene; its partial SVO is abandoned */
        g_assert_armed = 0;
        stack_reset();
        memset(&g_scene.svo, 0, sizeof(g_scene.svo));
        return -1;
    }
    tg_svo_create(emin, emax, &g_scene, &g_scene.svo);
    g_assert_armed = 0;
    free(g_node_min);
    g_node_min = calloc((size_t)g_scene.svo.node_buffer_count * 3, sizeof(float));

    index_nodes(0, g_scene.svo.min, g_scene.svo.max);
    int n_nonempty = 0;
    for (u32 i = 0; i < g_scene.svo.leaf_node_data_buffer_count; i++)
        n_nonempty += g_scene.svo.p_leaf_node_data_buffer[i].n != 0;
    return n_nonempty;
}

static int g_out_count;
/* g_node_min: world min corner of every node of the last build */

static void index_nodes(u32 node_idx, v3 mn, v3 mx)
{
    g_node_min[3 * node_idx] = mn.x; g_node_min[3 * node_idx + 1] = mn.y; g_node_min[3 * node_idx + 2] = mn.z;
    const tg_svo_inner_node* p = &g_scene.svo.p_node_buffer[node_idx].inner;
    const v3 ce = tgm_v3_mulf(tgm_v3_sub(mx, mn), 0.5f);
    u32 rank = 0;
    for (u32 c = 0; c < 8; c++)
    {
        if (!(p->valid_mask & (1u << c))) continue;
        const u32 child_idx = node_idx + p->child_pointer + rank++;
        const v3 cmn = { mn.x + (f32)(c & 1) * ce.x, mn.y + (f32)((c >> 1) & 1) * ce.y, mn.z + (f32)((c >> 2) & 1) * ce.z };
        if (p->leaf_mask & (1u << c))
        {
            g_node_min[3 * child_idx] = cmn.x; g_node_min[3 * child_idx + 1] = cmn.y; g_node_min[3 * child_idx + 2] = cmn.z;
        }
        else
        {
            index_nodes(child_idx, cmn, tgm_v3_add(cmn, ce));
        }
    }
}

static void walk(u32 node_idx, v3 mn, v3 mx, int32_t* out_block_xyz, uint32_t* out_words, int capacity)
{
    const tg_svo_inner_node* p = &g_scene.svo.p_node_buffer[node_idx].inner;
    const v3 ce = tgm_v3_mulf(tgm_v3_sub(mx, mn), 0.5f);
    u32 rank = 0;
    for (u32 c = 0; c < 8; c++)
    {
        if (!(p->valid_mask & (1u << c))) continue;
        const u32 child_idx = node_idx + p->child_pointer + rank++;
        const v3 cmn = { mn.x + (f32)(c & 1) * ce.x, mn.y + (f32)((c >> 1) & 1) * ce.y, mn.z + (f32)((c >> 2) & 1) * ce.z };
        const v3 cmx = tgm_v3_add(cmn, ce);
        if (p->leaf_mask & (1u << c))
        {
            const u32 dp = g_scene.svo.p_node_buffer[child_idx].leaf.data_pointer;
            if (g_scene.svo.p_leaf_node_data_buffer[dp].n == 0) continue;
            if (g_out_count < capacity)
            {
                out_block_xyz[3 * g_out_count + 0] = (int32_t)cmn.x;
                out_block_xyz[3 * g_out_count + 1] = (int32_t)cmn.y;
                out_block_xyz[3 * g_out_count + 2] = (int32_t)cmn.z;
                memcpy(&out_words[(size_t)g_out_count * 1024], &g_scene.svo.p_voxels_buffer[(size_t)dp * 1024], 4096);
            }
            g_out_count++;
        }
        else
        {
            walk(child_idx, cmn, cmx, out_block_xyz, out_words, capacity);
        }
    }
}

/*
 * Lists the non-empty 32^3 leaf blocks of the last build: world min corner of
 * each block and its 1024 voxel words (bit 1024z+32y+x).  Returns the count
 * (which may exceed capacity; only `capacity` blocks are written).
 */
int tgref_svo_blocks(int32_t* out_block_xyz, uint32_t* out_words, int capacity)
{
    g_out_count = 0;
    if (!g_scene.svo.p_node_buffer) return -1;
    walk(0, g_scene.svo.min, g_scene.svo.max, out_block_xyz, out_words, capacity);
    return g_out_count;
}

void tgref_svo_stats(uint32_t out[3])
{
    out[0] = g_scene.svo.node_buffer_count;
    out[1] = g_scene.svo.leaf_node_data_buffer_count;
    out[2] = g_scene.svo.voxel_buffer_count_in_u32;
}

/*
 * Traverses the last-built SVO for n rays.  out_hit[i] = 1 on hit, -1 when
 * one of the reference's assertions fails for the ray,
 * out_distance = the reference distance, out_world_voxel = world integer
 * coordinate of the hit voxel (from the leaf block origin + voxel index).
 */
void tgref_svo_traverse(uint32_t n, const float* origins, const float* dirs,
                        int32_t* out_hit, float* out_distance, int32_t* out_world_voxel)
{
    for (uint32_t i = 0; i < n; i++)
    {
        f32 dist; u32 node, vox;
        const v3 o = { origins[3 * i], origins[3 * i + 1], origins[3 * i + 2] };
        const v3 d = { dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2] };
        /* tg_svo_traverse treats ray_origin relative to the SVO center
         * (tg_sparse_voxel_octree.c:574) while testing against svo.min/max;
         * callers pass world origins exactly as the reference's probe does
         * (tgvk_raytracer.c:1400). */
        g_assert_armed = 1;
        if (setjmp(g_assert_jmp))
        {
            /* one of the reference's assertions failed for this ray */
            g_assert_armed = 0;
            out_hit[i] = -1;
            out_distance[i] = 0.0f;
            out_world_voxel[3 * i] = out_world_voxel[3 * i + 1] = out_world_voxel[3 * i + 2] = 0;
            continue;
        }
        const b32 hit = tg_svo_traverse(&g_scene.svo, o, d, &dist, &node, &vox);
        g_assert_armed = 0;
        out_hit[i] = hit;
        out_distance[i] = dist;
        out_world_voxel[3 * i] = out_world_voxel[3 * i + 1] = out_world_voxel[3 * i + 2] = 0;
        if (hit)
        {
            const u32 dp = g_scene.svo.p_node_buffer[node].leaf.data_pointer;
            const u32 rel = vox - dp * 32768u;
            out_world_voxel[3 * i + 0] = (int32_t)g_node_min[3 * node + 0] + (int32_t)(rel % 32u);
            out_world_voxel[3 * i + 1] = (int32_t)g_node_min[3 * node + 1] + (int32_t)((rel / 32u) % 32u);
            out_world_voxel[3 * i + 2] = (int32_t)g_node_min[3 * node + 2] + (int32_t)(rel / 1024u);
        }
    }
}
