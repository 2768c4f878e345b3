/*
 * libqbcuda — GB300 (sm_103a) implementation of qubatron's octree ray-cast
 * path behind a plain C ABI.
 *
 * It replaces the GL connector of the reference, src/qubatron/octree_glc.c
 * (interface at octree_glc.c:65-85): the same buffers are uploaded with the
 * same (data, type, size, itemsize, start, end, buftype) arguments, and one
 * render call draws a frame the way octree_glc_update does, into a headless
 * RGBA buffer instead of a GL framebuffer. The per-pixel work is the fragment
 * shader src/qubatron/shaders/octree_fsh.c (primary ray, shadow ray, shading,
 * light flare), reproduced bit for bit in FP32.
 *
 * Conventions
 *  - Every call returns 0 on success or a negative QBC_E_* code; the message
 *    of the last failure on the calling thread is qbc_last_error().
 *  - One context drives one GPU and is not thread-safe, like the single GL
 *    context of the reference.
 *  - Output rows run bottom-up (row 0 is the bottom row), as glReadPixels
 *    returns a GL framebuffer.
 */
#ifndef QBCUDA_H
#define QBCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---- */
#define QBC_OK 0
#define QBC_E_ARG -1      /* bad argument (range, itemsize, type, size) */
#define QBC_E_CUDA -2     /* a CUDA runtime call failed */
#define QBC_E_NOMEM -3    /* device or host allocation failed */
#define QBC_E_STATE -4    /* call not valid in this state */
#define QBC_E_TIMEOUT -5  /* a bounded wait inside a kernel gave up */
#define QBC_E_IO -6       /* a file could not be opened or read */

/* ---- GL enums the reference passes as `type` (GL/gl.h values) ---- */
#define QBC_GL_INT 0x1404
#define QBC_GL_FLOAT 0x1406

/* Buffer ids: same order and meaning as octree_glc_buffer_t (octree_glc.c:16-24). */
typedef enum qbc_buffer
{
    QBC_STATIC_COLOR   = 0,
    QBC_STATIC_NORMAL  = 1,
    QBC_STATIC_OCTREE  = 2,
    QBC_DYNAMIC_COLOR  = 3,
    QBC_DYNAMIC_NORMAL = 4,
    QBC_DYNAMIC_OCTREE = 5
} qbc_buffer;

typedef struct qbc_ctx qbc_ctx;

/*
 * Uniforms of one frame. qbc_view_setup derives them from the arguments of
 * octree_glc_update (octree_glc.c:263-284) and from the frame-constant part of
 * the shader's main() (octree_fsh.c:401-418); everything per pixel is done on
 * the GPU. Filling the struct directly renders with exactly these values.
 */
typedef struct qbc_view
{
    float   camfp[3];       /* camera position (uniform camfp) */
    float   light[3];       /* uniform light */
    float   basecube[4];    /* (0, S, S, S) */
    float   dim[2];         /* uniform dimensions: (ow, oh) */
    float   cfp[3];         /* screen-space focus point (ow/2, oh/2, focal) */
    float   qz[4];          /* yaw quaternion, about +y by -angle.x */
    float   qx[4];          /* pitch quaternion, about the rotated -x by -angle.y */
    float   ncamlight[3];   /* normalize(light - camfp) */
    float   flare_cos;      /* largest float <= cos(0.02f): camangle < 0.02 test */
    float   coord_scale[2]; /* ow / width_px, oh / height_px (1.0 for whole sizes) */
    int32_t width_px;       /* (int) ow: the GL viewport width */
    int32_t height_px;
    int32_t maxlevel;       /* uniform maxlevel, 0..QBC_MAX_LEVEL */
    int32_t shoot;          /* uniform shoot */
} qbc_view;

#define QBC_MAX_LEVEL 17 /* the shader's stack holds 18 levels (octree_fsh.c:151) */

/* Per-pixel status bits (qbc_outputs.flags). */
#define QBC_PX_PRIMARY_LEAF (1u << 0) /* primary ray reached a leaf */
#define QBC_PX_DISCARD (1u << 1)      /* a traversal discarded the fragment: pixel left at 0 */
#define QBC_PX_SHADED (1u << 2)       /* res.isp.w > 0: shadow ray traced and pixel shaded */
#define QBC_PX_SHADOW_LEAF (1u << 3)  /* shadow ray reached a leaf */
#define QBC_PX_LIT (1u << 4)          /* step(sqr, 15.0) == 1 */
#define QBC_PX_FLARE_TEST (1u << 5)   /* camangle < 0.02: flare ray traced */
#define QBC_PX_FLARE_WHITE (1u << 6)  /* flare turned the pixel white */
#define QBC_PX_OOB (1u << 7)          /* a node or point index fell outside the uploaded arrays */

/*
 * Output buffers of one view; any pointer may be NULL. All are width_px *
 * height_px pixels, row 0 at the bottom.
 *   rgba8   4 bytes per pixel, the RGBA8 target of the reference (octree_glc.c:237)
 *   rgba32f 4 floats per pixel, the fragment colour before quantisation
 *   flags   QBC_PX_* bits
 *   leaf    4 int32 per pixel: primary leaf node (static, dynamic), shadow
 *           leaf node (static, dynamic); -1 where no leaf was reached
 *   isp     4 floats per pixel: primary intersection (x, y, z, t)
 *   visits  4 uint32 per pixel: node visits of the primary ray (static,
 *           dynamic) and of the shadow ray (static, dynamic)
 */
typedef struct qbc_outputs
{
    uint8_t*  rgba8;
    float*    rgba32f;
    uint32_t* flags;
    int32_t*  leaf;
    float*    isp;
    uint32_t* visits;
} qbc_outputs;

/* Library version string. */
const char* qbc_version(void);

/* Message of the last failed call on this thread ("" when none). */
const char* qbc_last_error(void);

/*
 * Create a context on CUDA device `device` (replaces octree_glc_init,
 * octree_glc.c:93-247: no shaders to compile, six empty buffers).
 */
int qbc_create(int device, qbc_ctx** out);
int qbc_destroy(qbc_ctx* ctx);

/*
 * Upload a range of a host buffer (replaces octree_glc_upload_texbuffer_data,
 * octree_glc.c:361-498), same argument meaning:
 *   data      base of the WHOLE host array (the copy reads data + start)
 *   type      QBC_GL_FLOAT for colour/normal, QBC_GL_INT for octrees
 *   size      bytes of the whole array; the device buffer grows to hold it and
 *             is then refilled from [0, size), as the reference re-creates its
 *             texture (octree_glc.c:412-428)
 *   itemsize  12 (one float3 point) for colour/normal; 16 (one RGBA32I texel,
 *             3 per node) or 48 (one node) for octrees
 *   start,end byte range [start, end) to copy; an octree range is widened to
 *             whole nodes [start/48, ceil(end/48))
 * Octree nodes (12 int32: 8 children, model index, 3 pad; octree.c:11-14) are
 * repacked on the device into 32-byte child blocks plus a model-index array.
 * The host array may be reused as soon as the call returns.
 */
int qbc_upload(qbc_ctx* ctx, const void* data, int type, size_t size, size_t itemsize, size_t start, size_t end, int buftype);

/*
 * qbc_upload with `data` in device memory of the context's GPU (for example
 * the output of a skinning kernel), same argument meaning. Keeps the data on
 * the device instead of a host round trip per frame (the reference reads the
 * skinned paths back and re-uploads the dynamic tree and normals each frame,
 * skeleton_glc.c:238-245, qubatron.c:508-529).
 */
int qbc_upload_device(qbc_ctx* ctx, const void* data, int type, size_t size, size_t itemsize, size_t start, size_t end, int buftype);

/*
 * Rigid skinning on the GPU: point i moves with bone[i], p' = R p + t and
 * n' = R n, with bones[b] = {R row-major (9 floats), t (3 floats)}. Arrays
 * are device memory; rest_nrms/out_nrms may both be NULL. A stand-in for the
 * reference's skeleton shader (skeleton_vsh.c, gameplay) that drives the
 * per-frame dynamic rebuild: skin, then qbc_build_tree(ctx, 1, out_pnts, ...,
 * on_device = 1) and qbc_upload_device of the normals.
 */
#define QBC_MAX_BONES 64
int qbc_skin_rigid(qbc_ctx* ctx, const float* rest_pnts, const float* rest_nrms, const int32_t* bone, int64_t n, const float* bones, int n_bones, float* out_pnts, float* out_nrms);

/*
 * The per-frame update of the dynamic basecube as one call: rigid skinning
 * of the rest points with the bone set in DEVICE memory (read when the work
 * runs), the dynamic tree rebuilt on the GPU from the skinned points
 * (octree_reset + octree_insert_point in point order, octree.c:89-147, model
 * indices 0..n-1), and the skinned normals taken as the dynamic model's
 * normals. The reference does this on the host each frame, reading the
 * skinned paths back from its skeleton shader and uploading the dynamic
 * octree and normals again (qubatron.c:439-452, 508-529; skeleton_glc.c:238-245).
 * All arrays are device memory of the context's GPU; pnts / nrms receive the
 * skinned points and normals. The call queues the work on the context's
 * stream and returns: no host synchronisation, and no allocation once the
 * buffers have this update's size (the first call of a size allocates). A
 * bone index outside the set skins with bone 0; a skinned point that is
 * negative or not finite is left out of the tree; either is reported by the
 * next qbc_synchronize / qbc_tree_nodes / qbc_download_tree. The colours of
 * the dynamic model are uploaded once, as the reference does.
 */
typedef struct qbc_dynamic_update
{
    const float*   rest_pnts; /* n float3 */
    const float*   rest_nrms; /* n float3, or NULL (then nrms NULL) */
    const int32_t* bone;      /* n bone indices */
    const float*   bones;     /* n_bones x 12 floats: R row-major, t; p' = R p + t */
    float*         pnts;      /* n float3 out */
    float*         nrms;      /* n float3 out, or NULL */
    int64_t        n;
    int32_t        n_bones;   /* 1..QBC_MAX_BONES */
    int32_t        levels;    /* tree depth, 0..21 */
    float          basesize;  /* basecube edge of the dynamic tree */
    int32_t        pad;
} qbc_dynamic_update;

int qbc_dynamic_update_run(qbc_ctx* ctx, const qbc_dynamic_update* update);

/*
 * Derive the uniforms of one frame from the arguments of octree_glc_update
 * (octree_glc.c:249-284). focal <= 0 selects the reference's focal length
 * (ow/2)/tan(pi/4) (octree_fsh.c:403); a positive value sets cfp.z directly.
 */
int qbc_view_setup(float width, float height, const float position[3], const float angle[3], float lighta, int quality, int maxlevel, float basesize, int shoot, float focal, qbc_view* out);

/*
 * Render one frame with the reference's arguments (replaces
 * octree_glc_update, octree_glc.c:249-352, without the window blit):
 * width_px x height_px RGBA8 pixels into the host buffer rgba8_out. Blocks
 * until the pixels are in host memory.
 */
int qbc_render(qbc_ctx* ctx, float width, float height, const float position[3], const float angle[3], float lighta, int quality, int maxlevel, float basesize, int shoot, uint8_t* rgba8_out);

/*
 * Render n views in one batch. outs[i] holds the outputs of views[i]; the
 * pointers are host memory when outputs_on_device is 0 (pinned memory gives
 * the fastest copy) and device memory of this context's GPU otherwise. With
 * device outputs the call returns once the work is queued on the context's
 * stream; with host outputs it returns when the pixels are on the host.
 */
int qbc_render_views(qbc_ctx* ctx, const qbc_view* views, const qbc_outputs* outs, int n, int outputs_on_device);

/*
 * Batched ray queries through the same traversal (cube_trace_line,
 * octree_fsh.c:138-379): the reference's CPU callers of octree_trace_line
 * (qubatron.c:214-240, zombie.c:296-486) and the particle collision shader
 * (particle_vsh.c:122-374) ask exactly this. Per ray i, any pointer may be NULL:
 *   status  0 miss, 1 leaf reached, 2 discarded (fewer than 2 basecube faces)
 *   leaf    2 int32: node index at the leaf (static, dynamic), -1 when none
 *   model   2 int32: slot-8 model index at the leaf (static, dynamic)
 *   isp     4 floats: entry point of the leaf cell (x, y, z, t)
 *   col,nrm 4 floats each: colour and normal the shader fetches at the leaf
 *   visits  2 uint32: node visits (static, dynamic)
 * pos and dir are n float3; all arrays are host memory when on_device is 0,
 * device memory otherwise.
 */
typedef struct qbc_ray_hits
{
    int32_t*  status;
    int32_t*  leaf;
    int32_t*  model;
    float*    isp;
    float*    col;
    float*    nrm;
    uint32_t* visits;
} qbc_ray_hits;

int qbc_trace_rays(qbc_ctx* ctx, const float* pos, const float* dir, int64_t n, const float basecube[4], int maxlevel, const qbc_ray_hits* out, int on_device);

/*
 * Camera rays of selected pixels of one view, exactly as the render kernels
 * generate them (octree_fsh.c:401-418: ctp = pixel centre in the render's
 * coordinate space, csv = qx * (qz * (ctp - cfp)), and the flare test's
 * argument dot(normalize(light - camfp), normalize(csv))). Per pixel k,
 * out[4k..4k+3] = (csv.x, csv.y, csv.z, cosine). px, py and out are host
 * arrays (on_device = 0) or device arrays of the context's GPU. Lets a caller
 * check the per-pixel ray against its own camera math (the reference's
 * mt_quat.c quaternions) and find pixels on the flare threshold.
 */
int qbc_camera_rays(qbc_ctx* ctx, const qbc_view* view, const int32_t* px, const int32_t* py, int64_t n, float* out, int on_device);

/*
 * Render without allocating anything (no counterpart in the reference).
 *
 * For callers that cannot call cudaMalloc while they render: a frame loop
 * that must not stall on an allocation (cudaMalloc and cudaFree can
 * synchronize the device), a process whose device memory is already handed
 * to another allocator or a fixed budget, or code that must keep the
 * device's allocation state unchanged between frames. Same pixels as
 * qbc_render_views with device outputs; the caller passes the views and
 * DEVICE output buffers on the context's GPU, the scene comes from earlier
 * qbc_upload calls, and the work is queued on the context's stream.
 *
 * The only scratch the kernel needs, its work-queue counters, lives in a
 * fixed array of QBC_NOALLOC_MAX_LAUNCHES counters in the library's static
 * device memory, held by every GPU that loads the library until exit. A call
 * takes one counter per 32 views, so at most QBC_NOALLOC_MAX_VIEWS views per
 * call; more is rejected with QBC_E_ARG. The counters are cleared on the
 * stream before each use. All calls share them: two calls whose work
 * overlaps on the GPU (different streams, different contexts on one device)
 * race and must be ordered by the caller. The first call on a context loads
 * the render kernels' code (lazy module loading can otherwise place it in
 * device memory during a later frame) and sets their shared-memory limit;
 * make that first call before any stream capture. Every call looks up the
 * array's device address with the context's device current, so the address
 * stays right after a reset of the device's primary context. Host output
 * pointers are rejected with QBC_E_ARG. Building leaf
 * boxes (QBC_OPT_BOX_PRUNE) allocates, so this call never builds them: it
 * prunes with the boxes an earlier allocating render built for the current
 * trees, and walks a tree changed since then unpruned (same pixels). The
 * frame always runs on the persistent fused kernel: QBC_OPT_PERSISTENT 0 and
 * QBC_OPT_SPLIT_TREES 1 (whose record queue this call would have to
 * allocate) do not apply to it.
 */
#define QBC_NOALLOC_MAX_LAUNCHES 8
#define QBC_NOALLOC_MAX_VIEWS (QBC_NOALLOC_MAX_LAUNCHES * 32)
int qbc_render_views_noalloc(qbc_ctx* ctx, const qbc_view* views, const qbc_outputs* outs, int n);

/*
 * Options of qbc_render_views_ex.
 *   two_pass        0: one fused kernel (as qbc_render_views). 1: a primary
 *                   pass that queues the shaded and flare pixels (compacted
 *                   with warp-aggregated atomics), then a shade pass over the
 *                   queue: shadow ray, shading, flare.
 *   proposals       (two_pass only) cells to test before the plain shadow
 *                   walk: QBC_PROPOSE_NONE, QBC_PROPOSE_MLP (the occluder
 *                   network of qbc_proposal_*), QBC_PROPOSE_LOGGED (the first
 *                   leaf a previous logged render of the same views found),
 *                   QBC_PROPOSE_RANDOM (seeded, for tests).
 *   log             (two_pass only) record, per queued pixel, the t of the
 *                   plain shadow walk's first leaf and its lit bit.
 *   proposal_level  level of the proposed cells (0: QBC_OPT_PROPOSAL_LEVEL,
 *                   default 8).
 *   seed            QBC_PROPOSE_RANDOM seed.
 * A proposal is a point on the shadow ray; its level-`proposal_level` cell is
 * entered exactly as the plain walk would enter it (same candidates, same
 * entry point) and only its subtree is walked. A leaf found there more than
 * 4 units before the primary hit proves the pixel unlit: the plain walk's
 * first leaf is at least as early along the ray. Otherwise the plain walk
 * runs. Every pixel's colour, flags, primary leaf and intersection are thus
 * identical to the plain result; for proven pixels the shadow-leaf output is
 * -2 (not computed) and the shadow visit counts are the proposal walks'.
 */
#define QBC_PROPOSE_NONE 0
#define QBC_PROPOSE_MLP 1
#define QBC_PROPOSE_LOGGED 2
#define QBC_PROPOSE_RANDOM 3
typedef struct qbc_render_opts
{
    int32_t  two_pass;
    int32_t  proposals;
    int32_t  log;
    int32_t  proposal_level;
    uint64_t seed;
} qbc_render_opts;

/* Counters of the last qbc_render_views_ex call. The first six count the
 * shade pass of a two_pass render (0 otherwise; in a fused frame that runs
 * split, QBC_OPT_SPLIT_TREES, queued counts the pixels the one-tree kernel
 * handed to the two-tree kernel); box_words counts the 8-byte
 * leaf-box words (QBC_OPT_BOX_PRUNE) read by all walks of a render in which a
 * view has a visits output (0 otherwise). */
typedef struct qbc_render_stats
{
    uint64_t queued;            /* pixels in the shade pass */
    uint64_t shadow_rays;       /* plain shadow walks */
    uint64_t shadow_visits;     /* node visits of plain shadow walks */
    uint64_t proposals_tried;   /* proposal walks */
    uint64_t proposals_proven;  /* shadow rays settled by a proposal */
    uint64_t proposal_visits;   /* node visits of proposal walks */
    uint64_t box_words;         /* leaf-box words read (instrumented renders) */
} qbc_render_stats;

int qbc_render_views_ex(qbc_ctx* ctx, const qbc_view* views, const qbc_outputs* outs, int n, int outputs_on_device, const qbc_render_opts* opts, qbc_render_stats* stats);

/*
 * Static edits on the device. The reference edits its host octree with
 * octree_remove_point (src/qubatron/octree.c:182-218) and re-uploads each
 * edited node as a one-node range (modelutil.c:345-440). qbc_tree_remove_points
 * edits the tree held on the device directly, as n octree_remove_point calls
 * in input order would: per point, walk its octets (basesize, levels as the
 * tree was built); at the leaf, zero the parent's link to it and report the
 * leaf's model index (modind) and the parent node (octind). A point whose walk
 * meets an empty link reports -1 for both (the reference leaves the caller's
 * values as they were); of several points of one leaf, the first in input
 * order removes it and the rest report -1. A point with x <= -size at some
 * level (the reference would read outside the node there) or a non-finite
 * coordinate reports -1 and changes nothing. pts, modind and octind are host
 * or device arrays per on_device; modind / octind may be null. Captured frame
 * graphs see the edit (no buffer moves).
 */
int qbc_tree_remove_points(qbc_ctx* ctx, int tree, const float* pts, int64_t n, float basesize, int levels, int on_device, int32_t* modind, int32_t* octind, int64_t* removed);

/*
 * qmc flat model files, the reference's on-disk scene format (read by
 * model_load_flat, src/qubatron/model.c:53-111; written by qmc,
 * src/qubatron/qmc.c:275-327): .pnt, .nrm and .col hold one float3 per
 * point, .rng holds int triples (first point index of a column, x index,
 * y index).
 *
 * qbc_flat_read (host only, no GPU): the point count is the .pnt size in
 * whole float3 (trailing bytes ignored); colours and normals are read for
 * that many points (a shorter file leaves the rest 0); the range count is the
 * .rng size in whole ints. Null arrays return only the counts; arrays are
 * filled when their capacity (points, ints) suffices, else QBC_E_ARG.
 * rng_path may be null (no ranges). A file that cannot be opened or read
 * gives QBC_E_IO (the reference crashes on a missing .pnt).
 *
 * qbc_load_flat: qbc_flat_read, then what the reference's static model load
 * does with it (modelutil.c:180-255): octree_insert_point of every point in
 * file order into an empty tree (levels, basecube (0, S, S, S)), here built
 * on the GPU, and the colours and normals uploaded as that tree's model.
 * tree: 0 static, 1 dynamic. Counts out (any may be null); ranges as in
 * qbc_flat_read.
 */
int qbc_flat_read(const char* pnt_path, const char* col_path, const char* nrm_path, const char* rng_path, float* pnts, float* cols, float* nrms, int64_t point_cap, int64_t* points, int32_t* ranges, int64_t range_cap, int64_t* range_ints);
int qbc_load_flat(qbc_ctx* ctx, int tree, const char* pnt_path, const char* col_path, const char* nrm_path, const char* rng_path, float basesize, int levels, int64_t* points, int64_t* nodes, int32_t* ranges, int64_t range_cap, int64_t* range_ints);

/*
 * Autotuner (not part of the reference). Times frames of these views
 * (device outputs, these render options) on the context's stream under
 * candidate tuning options, one option after another with the others kept
 * at their best so far. With QBC_PROPOSE_MLP first the network's proposals:
 * the gate (1000 = off, 900, 700, 500, 300, 0 per mille), then, unless off,
 * the proposal count (1..3) and, when opts->proposal_level is 0, the cell
 * level (5..8), so that a network whose tries cost more than they save is
 * switched off and the frame is never slower than the plain two-pass
 * frame; then the service threshold (1..16), the warp tile width (2, 4, 8,
 * 16, 32) and the render blocks per SM (0, 2..8). Each candidate gets
 * one untimed frame, then `reps` (1..101) frames timed with CUDA events; its
 * time is their median. The fastest setting stays set on the context (the
 * initial one on error). The options change only the time of a frame, never
 * its pixels.
 */
typedef struct qbc_tune_result
{
    int32_t tile_width;
    int32_t blocks_per_sm;
    int32_t service_min;
    int32_t candidates;  /* settings timed */
    float   ms_initial;  /* median frame time under the options found */
    float   ms_best;     /* ... under the options left set */
    int32_t proposal_gate;  /* QBC_PROPOSE_MLP frames: gate left set (1000: proposals off) */
    int32_t proposal_count;
    int32_t proposal_level;
    int32_t split_trees;    /* two-tree fused frames: QBC_OPT_SPLIT_TREES left set */
} qbc_tune_result;

int qbc_autotune(qbc_ctx* ctx, const qbc_view* views, const qbc_outputs* dev_outs, int n, const qbc_render_opts* opts, int reps, qbc_tune_result* result);

/*
 * A frame as a CUDA graph (not part of the reference: the GL connector
 * redraws through the driver each frame). qbc_graph_capture renders the
 * views once into the device outputs, then captures the same frame (every
 * memset and kernel qbc_render_views_ex enqueues with these options) on the
 * context's stream as a CUDA graph and instantiates it. qbc_graph_launch
 * replays the frame with one launch call on the context's stream;
 * qbc_graph_update re-captures it for new uniforms of the same view sizes
 * (camera, light, quality) and updates the instantiated graph in place.
 * The graph holds the device addresses and sizes of the trees, models and
 * work buffers, the stream and the tuning options as they were at capture:
 * after an upload, build, qbc_set_stream or qbc_set_option that changes any
 * of them, qbc_graph_launch fails with QBC_E_STATE until qbc_graph_update.
 * Render statistics are not collected. qbc_destroy detaches the context's
 * graphs: afterwards they only accept qbc_graph_destroy.
 */
typedef struct qbc_graph qbc_graph;
int qbc_graph_capture(qbc_ctx* ctx, const qbc_view* views, const qbc_outputs* dev_outs, int n, const qbc_render_opts* opts, qbc_graph** graph);
/*
 * The same with the frame's dynamic update captured in front of the render
 * (qbc_dynamic_update_run: skin with the bones in device memory, rebuild the
 * dynamic tree, take the normals): one replay then re-skins, rebuilds and
 * renders, with no host round trip. Write the next frame's bones into
 * update->bones (on the context's stream, or before the launch) and call
 * qbc_graph_launch. The update's arrays and sizes are held by the graph; the
 * dynamic tree's buffers are sized for the update's node bound, so replays
 * never reallocate. qbc_graph_update re-captures both parts.
 */
int qbc_graph_capture_dynamic(qbc_ctx* ctx, const qbc_dynamic_update* update, const qbc_view* views, const qbc_outputs* dev_outs, int n, const qbc_render_opts* opts, qbc_graph** graph);
int qbc_graph_update(qbc_graph* graph, const qbc_view* views, int n);
int qbc_graph_launch(qbc_graph* graph);
int qbc_graph_destroy(qbc_graph* graph);

/*
 * Occluder-proposal network (QBC_PROPOSE_MLP; not part of the reference).
 * A 45 -> 128 -> 128 -> 128 -> 4 GELU network, BF16 weights and activations
 * on the tensor cores with FP32 accumulation, trained on the GPU. Input of a
 * shaded pixel: its hit point normalised to the basecube, unit normal, unit
 * direction to the light and sin/cos of pi times the normalised hit point
 * scaled by 4, 8, ..., 128 (6 frequencies). Output: 3 points t along the
 * shadow ray (light at 0, hit at 1; outside (0, 1) means "no proposal") and
 * the logit of "occluded before the hit" that gates them.
 *
 * qbc_proposal_collect: render views (at most 32) with the plain shadow walk
 *   and append one sample per shaded pixel to the context's training set:
 *   the features and the t of the walk's first leaf (occluded) or "lit".
 * qbc_proposal_train: minibatch Adam over the training set (initialises the
 *   network from opts->seed on first use).
 * Parameters are QBC_PROPOSAL_PARAMS floats: W1 [128][48], b1, W2 [128][128],
 * b2, W3 [128][128], b3, W4 [16][128], b4 [16] (W as [out][in]; input
 * columns 45..47 and output rows 3..15 are padding).
 */
#define QBC_PROPOSAL_PARAMS 41360
typedef struct qbc_train_opts
{
    int32_t  steps;
    int32_t  batch;
    float    lr;
    int32_t  pad;
    uint64_t seed;
} qbc_train_opts;

typedef struct qbc_train_stats
{
    uint64_t samples;   /* training-set size */
    uint64_t occluded;  /* samples with an occluder */
    float    loss_first;
    float    loss_last; /* mean of the last 10 steps */
} qbc_train_stats;

int qbc_proposal_collect(qbc_ctx* ctx, const qbc_view* views, int n, int64_t* samples);
int qbc_proposal_train(qbc_ctx* ctx, const qbc_train_opts* opts, qbc_train_stats* stats);
int qbc_proposal_clear(qbc_ctx* ctx);
int qbc_proposal_get_params(qbc_ctx* ctx, float* params);
int qbc_proposal_set_params(qbc_ctx* ctx, const float* params);
/* Network outputs for m host feature rows (45 floats each) -> out (4 per
 * row: the 3 proposed t, the occlusion logit). */
int qbc_proposal_eval(qbc_ctx* ctx, const float* x, int64_t m, float* out);
/* Mean training loss and its gradient (QBC_PROPOSAL_PARAMS floats) for m host
 * rows: features x (45 each), target t and kind (1 occluded at t, 0 lit). */
int qbc_proposal_gradient(qbc_ctx* ctx, const float* x, const float* t, const int8_t* kind, int64_t m, float* loss, float* grad);

/* Run the context's work on this CUDA stream (a cudaStream_t; NULL = the
 * context's own stream). */
int qbc_set_stream(qbc_ctx* ctx, void* stream);
int qbc_synchronize(qbc_ctx* ctx);

/*
 * Tuning options of a context (performance only; results do not change).
 *   QBC_OPT_SERVICE_MIN  1..32, default 4: in the persistent render kernel a
 *   lane whose ray ended waits until this many lanes of its warp wait (or no
 *   ray runs) before the warp starts their next rays together.
 *   QBC_OPT_PROPOSAL_GATE  0..1000 per mille, default 500: QBC_PROPOSE_MLP
 *   tries a pixel's proposals only when the network's occlusion probability
 *   is at least this (0: always; 1000: never, and the network is not run:
 *   the frame is the plain two-pass frame).
 *   QBC_OPT_PROPOSAL_LEVEL  1..QBC_MAX_LEVEL, default 8: level of the
 *   proposed cells when a render's opts->proposal_level is 0.
 *   QBC_OPT_PROPOSAL_COUNT  1..3, default 3: network proposals tried per
 *   pixel, earliest first.
 *   QBC_OPT_BOX_PRUNE  1 (default) or 0: the walk skips a child whose
 *   subtree's leaf box (widened by 2^-14 of the basecube edge) the ray
 *   misses. Pixels never change; only the per-pixel visit counts (the
 *   `visits` stream) fall below the shader's. 0 walks exactly as the
 *   shader, visit counts included.
 *   QBC_OPT_TILE_WIDTH  2, 4, 8 (default), 16 or 32: width of the 32-pixel warp
 *   tiles the render kernels take from their queue (height 32 / width).
 *   QBC_OPT_BLOCKS_PER_SM  0 (default: as many as fit) .. 32: resident
 *   render blocks per SM of the persistent grid.
 *   QBC_OPT_PERSISTENT  1 (default) or 0: the fused frame runs on the
 *   persistent kernel (warps take tiles of all views from a work queue and
 *   start new rays in batches), or, with 0, on the plain schedule: one
 *   thread per pixel for the pixel's whole life, one warp per 32-pixel tile,
 *   one launch of tiles_total / 4 blocks. Same pixels; the plain schedule is
 *   the baseline the persistent kernel is measured against. Two-pass renders
 *   always run persistent.
 *   QBC_OPT_SPLIT_TREES  0 (default) or 1: with 1, a persistent fused frame
 *   with a dynamic tree whose leaf boxes are built (QBC_OPT_BOX_PRUNE 1,
 *   exactly representable cubes) runs as two launches: a one-tree kernel
 *   walks every ray that misses the leaf boxes of the dynamic root's
 *   children and hands each pixel whose next ray may not to a two-tree
 *   kernel, which finishes it (and, should the record queue fill, the tiles
 *   the one-tree kernel then left). Same pixels; the queue takes 32 bytes
 *   per pixel of the largest launch. It pays on large frames in which the
 *   character covers little (32 4K views of a house: -8 %), not on a view
 *   aimed at the character (+5 %); qbc_autotune decides it.
 */
#define QBC_OPT_SERVICE_MIN 1
#define QBC_OPT_PROPOSAL_GATE 2
#define QBC_OPT_TILE_WIDTH 3
#define QBC_OPT_BLOCKS_PER_SM 4
#define QBC_OPT_PROPOSAL_COUNT 5
#define QBC_OPT_BOX_PRUNE 6
#define QBC_OPT_PERSISTENT 7
#define QBC_OPT_PROPOSAL_LEVEL 8
#define QBC_OPT_SPLIT_TREES 9
int qbc_set_option(qbc_ctx* ctx, int option, int value);
int qbc_get_option(qbc_ctx* ctx, int option, int* value);

/* Node and point counts currently held for a tree / model (0 static, 1 dynamic). */
int qbc_tree_nodes(qbc_ctx* ctx, int tree, int64_t* n_nodes);
int qbc_model_points(qbc_ctx* ctx, int model, int64_t* n_points);

/* Kernel launches issued by this context since creation. */
int qbc_launch_count(qbc_ctx* ctx, int64_t* count);

/*
 * GPU tree build into the context's static (tree 0) or dynamic (tree 1)
 * octree: the node array that inserting the n points in order into an empty
 * tree gives (octree_reset + octree_insert_point, octree.c:89-147, model
 * indices first_index + i), numbering included, built with sorts and prefix
 * sums instead of one walk per point. The result replaces the tree exactly
 * as a whole-array qbc_upload of that array would. pnts is n float3 on the
 * host (on_device = 0) or on the context's GPU.
 */
int qbc_build_tree(qbc_ctx* ctx, int tree, const float* pnts, int64_t n, float basesize, int levels, int64_t first_index, int on_device);
/* The same from per-point octet paths, `levels` int32 per point in 0..7
 * (octree_insert_path, octree.c:149-180; the per-frame dynamic rebuild of
 * qubatron.c:439-452 from the paths of skeleton_vsh.c:188-213). */
int qbc_build_tree_paths(qbc_ctx* ctx, int tree, const int32_t* octets, int64_t n, int levels, int64_t first_index, int on_device);
/* Copy a tree back to the host in the reference layout (12 int32 per node:
 * 8 children, model index, 3 zero). nodes may be NULL to query the count. */
int qbc_download_tree(qbc_ctx* ctx, int tree, int32_t* nodes, int64_t cap, int64_t* n_nodes);

/* ---- node-array producer (octree.c:95-218) ---- */

/* A growable host node array (12 int32 per node, node 0 = root). */
typedef struct qbc_octree qbc_octree;

/* New tree holding only the root (octree_create, octree.c:55-67). */
int qbc_octree_create(float basesize, int levels, qbc_octree** out);
int qbc_octree_free(qbc_octree* tree);
/* Back to the root alone (octree_reset, octree.c:89-93). */
int qbc_octree_reset(qbc_octree* tree);
/* octree_insert_point (octree.c:95-147) for n points in order, model indices
 * first_index + i. */
int qbc_octree_insert_points(qbc_octree* tree, const float* pnts, int64_t n, int64_t first_index);
/* octree_insert_path (octree.c:149-180): octets holds `levels` octets per point. */
int qbc_octree_insert_paths(qbc_octree* tree, const int32_t* octets, int64_t n, int64_t first_index);
/* octree_remove_point (octree.c:182-218). */
int qbc_octree_remove_point(qbc_octree* tree, const float pnt[3], int32_t* modind, int32_t* octind);
/* Node array and node count (valid until the tree changes). */
int qbc_octree_nodes(qbc_octree* tree, const int32_t** nodes, int64_t* n_nodes);

/* ---- seeded synthetic scenes ---- */

#define QBC_SCENE_FLOOR 0 /* floor plane + boxes + spheres */
#define QBC_SCENE_ROOM 1  /* closed room (floor, 4 walls, ceiling) + boxes + spheres */
#define QBC_SCENE_HOUSE 2 /* 3 floors x 6 closed rooms; each box / sphere in a seeded room */

typedef struct qbc_scene_desc
{
    int32_t  kind;
    int32_t  levels;
    int64_t  n_points;
    uint64_t seed;
    float    basesize;
    int32_t  n_boxes;
    float    box_min, box_max;
    int32_t  n_spheres;
    float    sphere_min, sphere_max;
    float    color_noise; /* uniform +- per channel around the primitive colour */
} qbc_scene_desc;

/*
 * Generate n_points float3 points, normals and colours. Points are emitted in
 * octree-path order (a stable sort by the 3-bit octets of octree.c:100-109,
 * root first), the order a voxel-sorted asset has, so that inserting them in
 * order builds the tree front to back. Only +, -, *, / and sqrt are used, so
 * every machine generates the same bits.
 */
int qbc_scene_generate(const qbc_scene_desc* desc, float* pnts, float* nrms, float* cols);

#ifdef __cplusplus
}
#endif

#endif
