/* octree_cuda.c — octree_glc_* on top of libqbcuda. Link with -lqbcuda. */
#include "mt_vector_3d.c" /* v3_t, included the way qubatron's other sources do */
#include "qbcuda.h"
#include <stdio.h>
#include <stdlib.h>

typedef struct octree_glc_t { qbc_ctx* ctx; uint8_t* frame; size_t frame_bytes; } octree_glc_t;
typedef qbc_buffer octree_glc_buffer_t;           /* same enum values */

octree_glc_t octree_glc_init(char* path)
{
    (void) path;                                     /* no shaders to load */
    octree_glc_t rc = {0};
    if (qbc_create(0, &rc.ctx)) fprintf(stderr, "qbc_create: %s\n", qbc_last_error());
    return rc;
}

void octree_glc_upload_texbuffer_data(octree_glc_t* rc, void* data, int type, size_t size,
                                      size_t itemsize, size_t start, size_t end,
                                      octree_glc_buffer_t buftype)
{
    if (qbc_upload(rc->ctx, data, type, size, itemsize, start, end, buftype))
        fprintf(stderr, "qbc_upload: %s\n", qbc_last_error());
}

void octree_glc_update(octree_glc_t* rc, float width, float height, v3_t position, v3_t angle,
                       float lighta, uint8_t quality, int maxlevel, float basesize, int shoot)
{
    qbc_view v;
    float pos[3] = {position.x, position.y, position.z}, ang[3] = {angle.x, angle.y, 0.0f};
    if (qbc_view_setup(width, height, pos, ang, lighta, quality, maxlevel, basesize, shoot, 0.0f, &v)) return;
    size_t need = (size_t) v.width_px * v.height_px * 4;
    if (need > rc->frame_bytes) { rc->frame = realloc(rc->frame, need); rc->frame_bytes = need; }
    qbc_outputs out = {0};
    out.rgba8 = rc->frame;                           /* row 0 = bottom, like glReadPixels */
    if (qbc_render_views(rc->ctx, &v, &out, 1, 0))
        fprintf(stderr, "qbc_render_views: %s\n", qbc_last_error());
    /* present rc->frame: SDL_UpdateTexture / write a file / hand to an encoder */
}
