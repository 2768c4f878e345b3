/*
 * qbo — CPU oracle for the qubatron octree ray-cast path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * fragment shader `src/qubatron/shaders/octree_fsh.c` (ray generation, the
 * joint static+dynamic `cube_trace_line` traversal, shadow bit, shading and
 * light flare), of the node-array producer in `src/qubatron/octree.c`
 * (`octree_insert_point`, `octree_insert_path`, `octree_remove_point`) and of
 * the per-frame uniform derivation in `src/qubatron/octree_glc.c:249-305`.
 * It exists to check the CUDA library; nothing in the library calls it.
 *
 * Parity anchor: the static-tree part of the traversal is pinned against the
 * reference's own `octree_trace_line` (`octree.c:341-537`) and the node arrays
 * against its `octree_insert_point`, compiled from the reference sources into
 * oracle/_ref by oracle/build_ref.sh; fixtures from that build are committed
 * under tests/golden/. The GLSL shader itself cannot run here (no graphics
 * stack), so the dynamic-tree, shading and flare parts are restated from the
 * shader text and checked by the GPU kernel's bit-exact agreement only.
 *
 * Arithmetic: FP32 in the shader's operation order, compiled with
 * -ffp-contract=off so no multiply-add is fused; division and sqrt are IEEE.
 */
#ifndef QBO_H
#define QBO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One tree in the reference layout: 12 int32 per node (8 children, model
 * index, 3 pad), node 0 = root, child index 0 = empty (octree.c:11-14).
 * cbox / box_depth: leaf-box records of qbo_build_boxes (16 words per node)
 * and the depth they were built for; NULL (the default) walks as the shader,
 * with no pruning. */
typedef struct qbo_tree
{
    const int32_t*  nodes;
    int64_t         n_nodes;
    const uint32_t* cbox;
    int32_t         box_depth;
} qbo_tree;

/* Per-point float3 attribute arrays (model.c:14-25). */
typedef struct qbo_model
{
    const float* col;
    const float* nrm;
    int64_t      n_points;
} qbo_model;

/* [0] = static, [1] = dynamic (octree_fsh.c:33-40). */
typedef struct qbo_scene
{
    qbo_tree  tree[2];
    qbo_model model[2];
} qbo_scene;

/* Uniforms of one frame, derived on the host exactly once
 * (octree_glc.c:263-284 plus the per-frame constants of octree_fsh.c:401-418). */
typedef struct qbo_view
{
    float   camfp[3];      /* camera position (uniform camfp) */
    float   light[3];      /* uniform light */
    float   basecube[4];   /* (0, S, S, S) */
    float   dim[2];        /* uniform dimensions (ow, oh) */
    float   cfp[3];        /* screen-space focus point */
    float   qz[4];         /* yaw quaternion */
    float   qx[4];         /* pitch quaternion */
    float   ncamlight[3];  /* normalize(light - camfp) */
    float   flare_cos;     /* largest float <= cos(0.02f) */
    float   coord_scale[2];/* ow / width_px, oh / height_px */
    int32_t width_px;
    int32_t height_px;
    int32_t maxlevel;
    int32_t shoot;
} qbo_view;

/* Status of one traversal. */
enum
{
    QBO_MISS    = 0, /* traversal emptied its stack (octree_fsh.c:374) */
    QBO_LEAF    = 1, /* reached level == maxlevel (octree_fsh.c:218) */
    QBO_DISCARD = 2  /* fewer than 2 basecube faces or both behind (octree_fsh.c:195-198) */
};

typedef struct qbo_hit
{
    float   isp[4];       /* entry point of the leaf cell, w = t */
    float   col[4];
    float   nrm[4];
    float   tlf[4];       /* leaf cube */
    int32_t leaf[2];      /* node index at the leaf in static / dynamic tree */
    int32_t model[2];     /* slot-8 model index after the empty rule */
    int32_t status;
    int32_t faces;        /* number of basecube faces that passed the entry test */
    int32_t visits[2];    /* subnode tests run with a non-empty node, per tree */
    int32_t steps;        /* loop iterations */
    int32_t oob;          /* an index fell outside an uploaded array */
} qbo_hit;

/* Per-pixel status bits written by qbo_render. */
enum
{
    QBO_PX_PRIMARY_LEAF = 1u << 0,
    QBO_PX_DISCARD      = 1u << 1, /* some traversal discarded: pixel not written */
    QBO_PX_SHADED       = 1u << 2, /* res.isp.w > 0: shadow ray traced */
    QBO_PX_SHADOW_LEAF  = 1u << 3,
    QBO_PX_LIT          = 1u << 4, /* step(sqr, 15.0) == 1 */
    QBO_PX_FLARE_TEST   = 1u << 5, /* camangle < 0.02 */
    QBO_PX_FLARE_WHITE  = 1u << 6,
    QBO_PX_OOB          = 1u << 7
};

/* Per-pixel outputs; every pointer may be NULL. Row 0 is the bottom row. */
typedef struct qbo_frame
{
    float*    rgba;    /* 4 floats per pixel */
    uint8_t*  rgba8;   /* 4 bytes per pixel, GL unorm8 conversion */
    uint32_t* flags;   /* QBO_PX_* */
    int32_t*  leaf;    /* 4 per pixel: primary leaf s, d; shadow leaf s, d (-1 when none) */
    float*    isp;     /* 4 per pixel: primary isp (x, y, z, t) */
    uint32_t* visits;  /* 4 per pixel: primary visits s, d; shadow visits s, d */
} qbo_frame;

/* Traversal: cube_trace_line(pos, dir) (octree_fsh.c:138-379). */
void qbo_trace(const qbo_scene* sc, const float basecube[4], int maxlevel, const float pos[3], const float dir[3], qbo_hit* out);

/* qbo_trace over n rays on `threads` host threads (0: all); per ray status,
 * leaf[2], model[2], visits[2] (any output may be NULL). */
void qbo_trace_rays(const qbo_scene* sc, const float basecube[4], int maxlevel, const float* pos, const float* dir,
                    int64_t n, int32_t* status, int32_t* leaf, int32_t* model, int32_t* visits, int threads);

/* One fragment: main() (octree_fsh.c:399-464) at pixel (i, j), j from the bottom. */
void qbo_shade_pixel(const qbo_scene* sc, const qbo_view* v, int i, int j, float rgba[4], uint32_t* flags, int32_t leaf[4], float isp[4], uint32_t visits[4]);

/* Shading of a primary hit (octree_fsh.c:431-449): col (the hit texel,
 * alpha kept) is shaded in place; sqr is the squared distance from the
 * shadow ray's first leaf to the hit. */
void qbo_shade(const float isp[3], const float nrm[3], const float csv[3], const float light[3], float sqr, int shoot, float col[4]);

/* Camera ray of pixel (i, j) (octree_fsh.c:401-418): out = (csv, cosine of
 * the angle between csv and light - camfp). */
void qbo_camera_ray(const qbo_view* v, int i, int j, float out[4]);

/* A whole frame, OpenMP over 8x8 pixel tiles; threads <= 0 uses all. */
void qbo_render(const qbo_scene* sc, const qbo_view* v, const qbo_frame* out, int threads);

/* A pixel subset (for size-independent checks of big frames). */
void qbo_render_pixels(const qbo_scene* sc, const qbo_view* v, const int32_t* px, const int32_t* py, int64_t n, const qbo_frame* out, int threads);

/* Uniform derivation of octree_glc_update (octree_glc.c:263-270) plus the
 * frame-constant parts of main() (octree_fsh.c:403-418). focal <= 0 selects
 * the reference focal length (dim.x/2)/tan(PI/4). */
void qbo_view_setup(float width, float height, const float position[3], const float angle[3], float lighta, int quality, int maxlevel, float basesize, int shoot, float focal, qbo_view* out);

/* Leaf-box pruning of the CUDA library (no reference counterpart), restated
 * to check the pruned walk's visit counts; see qbo_boxes.c.
 * qbo_build_boxes fills rec (16 words per node) and returns the tree's depth,
 * or -1 when the array is not usable (a node reached twice, a child index
 * outside the array, deeper than 17 levels). */
typedef struct qbo_box_frame_t
{
    float a0[3], a1[3], u[3];
} qbo_box_frame_t;
int32_t qbo_build_boxes(const int32_t* nodes, int64_t n, uint32_t* rec);
void    qbo_box_frame(const float cube[4], const float p[3], const float inv[3], float m, qbo_box_frame_t* f);
int     qbo_box_hit(uint32_t rx, uint32_t ry, int o, const qbo_box_frame_t* f);
int     qbo_box_ray_ok(const float bc[4], int maxlevel, const float p[3], const float d[3]);

/* GL float -> unorm8 conversion used for the RGBA8 target (octree_glc.c:237). */
uint8_t qbo_unorm8(float f);

/* Node-array producer (octree.c:95-218). Nodes are 12 int32 each; *len is the
 * node count, cap the capacity in nodes. Returns 0, or -1 when cap is hit. */
int  qbo_insert_point(int32_t* nodes, int64_t* len, int64_t cap, float basesize, int levels, int64_t modind, const float pnt[3], int32_t* octindarr);
int  qbo_insert_path(int32_t* nodes, int64_t* len, int64_t cap, int levels, int64_t modind, const int32_t* octets);
void qbo_remove_point(int32_t* nodes, float basesize, int levels, const float pnt[3], int32_t* modind, int32_t* octind);
/* qbo_remove_point for n points (3 floats each) in order. */
void qbo_remove_points(int32_t* nodes, float basesize, int levels, const float* pnts, int64_t n, int32_t* modind,
                       int32_t* octind);
void qbo_point_octets(float basesize, int levels, const float pnt[3], int32_t* octets);
/* All n points in order into an empty tree; returns the node count or -1. */
int64_t qbo_build_tree(const float* pnts, int64_t n, float basesize, int levels, int32_t* nodes, int64_t cap);

/* Seeded synthetic scenes of the benchmark workloads (qbo_scene.c; kind 0
 * floor, 1 room, 2 house): n float3 points, normals and colours in
 * octree-path order. Returns 0, or a negative value on bad arguments. */
int qbo_scene_generate(int kind, int levels, int64_t n, uint64_t seed, float basesize, int n_boxes, float box_min, float box_max, int n_spheres, float sphere_min, float sphere_max, float color_noise, float* pnts, float* nrms, float* cols);

#ifdef __cplusplus
}
#endif

#endif
