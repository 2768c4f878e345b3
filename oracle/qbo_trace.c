/*
 * CPU oracle (test infrastructure only): restatement of the fragment shader
 * src/qubatron/shaders/octree_fsh.c and the frame-uniform setup of
 * src/qubatron/octree_glc.c:249-305. Build with -ffp-contract=off.
 */
#include "qbo.h"

#include <float.h>
#include <math.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define QBO_STACK 18 /* stck_t stck[18] (octree_fsh.c:151) */

/* Bound on node entries per ray. A valid tree needs far fewer; a corrupt one
 * whose child indices repeat could make the walk exponential. Past the bound
 * the ray ends as a miss with the out-of-range flag set (the CUDA kernel
 * applies the same bound to the same count). */
#define QBO_MAX_PUSHES (1 << 22)

typedef struct v4
{
    float x, y, z, w;
} v4;

/* octet shift tables and octet pairs (octree_fsh.c:25-31) */
static const float k_xsft[8] = {0.0f, 1.0f, 0.0f, 1.0f, 0.0f, 1.0f, 0.0f, 1.0f};
static const float k_ysft[8] = {0.0f, 0.0f, 1.0f, 1.0f, 0.0f, 0.0f, 1.0f, 1.0f};
static const float k_zsft[8] = {0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 1.0f, 1.0f, 1.0f};
static const int   k_hor[8]  = {1, 0, 3, 2, 5, 4, 7, 6};
static const int   k_ver[8]  = {2, 3, 0, 1, 6, 7, 4, 5};
static const int   k_dep[8]  = {4, 5, 6, 7, 0, 1, 2, 3};

/* is_cube_xplane / yplane / zplane (octree_fsh.c:62-99). A ray parallel to
 * the plane returns FLT_MAX in every component. */
static v4 hit_xplane(float x, const float* p, const float* d)
{
    v4 r = {FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX};
    if (d[0] != 0.0f)
    {
        r.w = (x - p[0]) / d[0];
        r.y = p[1] + d[1] * r.w;
        r.z = p[2] + d[2] * r.w;
        r.x = x;
    }
    return r;
}

static v4 hit_yplane(float y, const float* p, const float* d)
{
    v4 r = {FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX};
    if (d[1] != 0.0f)
    {
        r.w = (y - p[1]) / d[1];
        r.x = p[0] + d[0] * r.w;
        r.z = p[2] + d[2] * r.w;
        r.y = y;
    }
    return r;
}

static v4 hit_zplane(float z, const float* p, const float* d)
{
    v4 r = {FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX};
    if (d[2] != 0.0f)
    {
        r.w = (z - p[2]) / d[2];
        r.x = p[0] + d[0] * r.w;
        r.y = p[1] + d[1] * r.w;
        r.z = z;
    }
    return r;
}

/* Half-open face tests of octree_fsh.c:166-192 (the same forms are used for
 * the bisecting planes at :263-271). tlf = top-left-front, brb = bottom-right-back. */
static int in_zface(v4 a, v4 tlf, v4 brb) { return tlf.x < a.x && a.x <= brb.x && tlf.y > a.y && a.y >= brb.y; }
static int in_xface(v4 a, v4 tlf, v4 brb) { return tlf.y > a.y && a.y >= brb.y && tlf.z > a.z && a.z >= brb.z; }
static int in_yface(v4 a, v4 tlf, v4 brb) { return tlf.x < a.x && a.x <= brb.x && tlf.z > a.z && a.z >= brb.z; }

/* oct_from_octets_for_index (octree_fsh.c:127-136): node i slot k, with node 0
 * below the root meaning "no node". An index outside the uploaded array reads
 * as 0 and is reported; a tree that was never uploaded reads as all zero. */
static int32_t node_slot(const qbo_tree* t, int32_t node, int slot, int level, int32_t* oob)
{
    if (node == 0 && level > 0) return 0;
    if (t->n_nodes == 0) return 0;
    if (node < 0 || (int64_t) node >= t->n_nodes)
    {
        *oob = 1;
        return 0;
    }
    return t->nodes[(int64_t) node * 12 + slot];
}

/* texelFetch of an RGB32F point texture (octree_fsh.c:226-241): alpha reads 1. */
static void attr_fetch(const float* arr, int64_t n, int32_t idx, float out[4], int32_t* oob)
{
    if (n == 0)
    {
        out[0] = out[1] = out[2] = out[3] = 0.0f;
        return;
    }
    if (idx < 0 || (int64_t) idx >= n)
    {
        *oob   = 1;
        out[0] = out[1] = out[2] = out[3] = 0.0f;
        return;
    }
    out[0] = arr[(int64_t) idx * 3 + 0];
    out[1] = arr[(int64_t) idx * 3 + 1];
    out[2] = arr[(int64_t) idx * 3 + 2];
    out[3] = 1.0f;
}

typedef struct level_t
{
    v4      cube;    /* cube of this stack level */
    v4      isps[4]; /* candidate entry points, isps[0] = entry point of the cube */
    int     octs[4]; /* octet of each candidate */
    int     ispsi;   /* 128 | next << 4 | remaining, 0 = not yet tested */
    int32_t node[2]; /* node index in the static and dynamic tree */
} level_t;

void qbo_trace(const qbo_scene* sc, const float bc[4], int maxlevel, const float pos[3], const float dir[3], qbo_hit* out)
{
    memset(out, 0, sizeof(*out));
    out->leaf[0] = out->leaf[1] = -1;
    out->model[0] = out->model[1] = -1;
    out->status                   = QBO_MISS;

    level_t stk[QBO_STACK];
    int     level = 0;

    v4 tlf = {bc[0], bc[1], bc[2], bc[3]};
    v4 brb = {tlf.x + tlf.w, tlf.y - tlf.w, tlf.z - tlf.w, 0.0f};

    /* basecube entry (octree_fsh.c:161-208); room for all 6 faces so a ray
     * through an edge or corner keeps the first two candidates */
    v4  hitp[6];
    int hitc = 0;
    v4  act;

    act = hit_zplane(tlf.z, pos, dir); /* front */
    if (in_zface(act, tlf, brb)) hitp[hitc++] = act;
    act = hit_zplane(brb.z, pos, dir); /* back */
    if (in_zface(act, tlf, brb)) hitp[hitc++] = act;
    act = hit_xplane(tlf.x, pos, dir); /* left */
    if (in_xface(act, tlf, brb)) hitp[hitc++] = act;
    act = hit_xplane(brb.x, pos, dir); /* right */
    if (in_xface(act, tlf, brb)) hitp[hitc++] = act;
    act = hit_yplane(tlf.y, pos, dir); /* top */
    if (in_yface(act, tlf, brb)) hitp[hitc++] = act;
    act = hit_yplane(brb.y, pos, dir); /* bottom */
    if (in_yface(act, tlf, brb)) hitp[hitc++] = act;

    out->faces = hitc;

    if (hitc < 2 || (hitp[0].w < 0.0f && hitp[1].w < 0.0f))
    {
        out->status = QBO_DISCARD;
        return;
    }

    if (hitp[1].w < hitp[0].w) hitp[0] = hitp[1];
    if (hitp[0].w < 0.0f)
    {
        hitp[0].x = pos[0];
        hitp[0].y = pos[1];
        hitp[0].z = pos[2];
        hitp[0].w = 0.0f;
    }

    stk[0].cube    = tlf;
    stk[0].isps[0] = hitp[0];
    stk[0].ispsi   = 0;
    stk[0].node[0] = 0;
    stk[0].node[1] = 0;

    const qbo_tree* ts = &sc->tree[0];
    const qbo_tree* td = &sc->tree[1];
    int64_t         pushes = 0;

    /* leaf-box pruning of the CUDA library, when the scene carries boxes
     * (qbo_boxes.c; off by default): the ray conditions, the reciprocal
     * direction and the margin 2^-14 S */
    const int box_ray = (ts->cbox || td->cbox) && qbo_box_ray_ok(bc, maxlevel, pos, dir);
    const int box_s   = box_ray && ts->cbox && maxlevel >= ts->box_depth;
    const int box_d   = box_ray && td->cbox && td->n_nodes > 0 && maxlevel >= td->box_depth;
    float     inv[3]  = {0.0f, 0.0f, 0.0f};
    if (box_ray)
        for (int k = 0; k < 3; ++k) inv[k] = 1.0f / dir[k];
    const float box_m = bc[3] * 6.1035156e-05f;

    /* a ray that misses the leaf box of every child of the dynamic root can
     * reach no dynamic leaf: the library walks such a ray on the static tree
     * alone (no dynamic lookups, no dynamic visits); the pixels are the same */
    int use_d = 1;
    if (box_d && td->box_depth > 1)
    {
        qbo_box_frame_t bf0;
        qbo_box_frame(bc, pos, inv, box_m, &bf0);
        int near = 0;
        for (int o = 0; o < 8; ++o)
        {
            int32_t dummy = 0;
            int32_t c     = node_slot(td, 0, o, 0, &dummy);
            if (c > 0 && qbo_box_hit(td->cbox[2 * o], td->cbox[2 * o + 1], o, &bf0)) near = 1;
        }
        use_d = near;
    }

    for (;;)
    {
        out->steps++;
        level_t* L = &stk[level];
        tlf        = L->cube;

        if (level == maxlevel)
        {
            /* leaf: model indices, colour and normal (octree_fsh.c:218-247) */
            int32_t ms = node_slot(ts, L->node[0], 8, level, &out->oob);
            int32_t md = use_d ? node_slot(td, L->node[1], 8, level, &out->oob) : 0;

            out->isp[0] = L->isps[0].x;
            out->isp[1] = L->isps[0].y;
            out->isp[2] = L->isps[0].z;
            out->isp[3] = L->isps[0].w;
            out->tlf[0] = tlf.x;
            out->tlf[1] = tlf.y;
            out->tlf[2] = tlf.z;
            out->tlf[3] = tlf.w;

            attr_fetch(sc->model[0].col, sc->model[0].n_points, ms, out->col, &out->oob);
            attr_fetch(sc->model[0].nrm, sc->model[0].n_points, ms, out->nrm, &out->oob);
            if (md > 0)
            {
                attr_fetch(sc->model[1].col, sc->model[1].n_points, md, out->col, &out->oob);
                attr_fetch(sc->model[1].nrm, sc->model[1].n_points, md, out->nrm, &out->oob);
            }
            out->leaf[0]  = L->node[0];
            out->leaf[1]  = L->node[1];
            out->model[0] = ms;
            out->model[1] = md;
            out->status   = QBO_LEAF;
            return;
        }

        if (L->ispsi == 0)
        {
            /* subnode test (octree_fsh.c:251-329) */
            L->ispsi = 128;

            /* a visit reads the node's child block: counted when the node
             * exists and lies inside the uploaded array */
            if (!(L->node[0] == 0 && level > 0) && L->node[0] >= 0 && L->node[0] < ts->n_nodes) out->visits[0]++;
            if (use_d && !(L->node[1] == 0 && level > 0) && L->node[1] >= 0 && L->node[1] < td->n_nodes)
                out->visits[1]++;

            v4 cb = {tlf.x + tlf.w, tlf.y - tlf.w, tlf.z - tlf.w, 0.0f};
            v4 hlf;
            hlf.x = cb.x + (tlf.x - cb.x) * 0.5f;
            hlf.y = cb.y + (tlf.y - cb.y) * 0.5f;
            hlf.z = cb.z + (tlf.z - cb.z) * 0.5f;
            hlf.w = cb.w + (tlf.w - cb.w) * 0.5f;

            hitc    = 1;
            hitp[0] = L->isps[0];

            /* pruning: a level whose children are not all leaf cells */
            const int lev_s = box_s && level + 1 < ts->box_depth;
            const int lev_d = box_d && level + 1 < td->box_depth;
            qbo_box_frame_t bf;
            if (lev_s || lev_d)
            {
                const float cube4[4] = {tlf.x, tlf.y, tlf.z, tlf.w};
                qbo_box_frame(cube4, pos, inv, box_m, &bf);
            }

            act = hit_zplane(hlf.z, pos, dir);
            if (act.w > 0.0f && in_zface(act, tlf, cb)) hitp[hitc++] = act;
            act = hit_xplane(hlf.x, pos, dir);
            if (act.w > 0.0f && in_xface(act, tlf, cb)) hitp[hitc++] = act;
            act = hit_yplane(hlf.y, pos, dir);
            if (act.w > 0.0f && in_yface(act, tlf, cb)) hitp[hitc++] = act;

            int pre = -1;
            for (int i = 0; i < hitc; ++i)
            {
                /* selection by swapping, exactly as the shader orders them */
                for (int j = i + 1; j < hitc; ++j)
                {
                    if (hitp[j].w < hitp[i].w)
                    {
                        v4 tmp  = hitp[i];
                        hitp[i] = hitp[j];
                        hitp[j] = tmp;
                    }
                }

                act     = hitp[i];
                int oct = 0;
                if (act.x > hlf.x) oct = 1;
                if (act.y < hlf.y) oct += 2;
                if (act.z < hlf.z) oct += 4;

                /* a point on a bisecting plane lands in the same octet as the
                 * previous one: take its neighbour across that plane */
                if (oct == pre)
                {
                    if (act.x == hlf.x)
                        oct = k_hor[oct];
                    else if (act.y == hlf.y)
                        oct = k_ver[oct];
                    else if (act.z == hlf.z)
                        oct = k_dep[oct];
                }
                pre = oct;

                int32_t cs = node_slot(ts, L->node[0], oct, level, &out->oob);
                int32_t cd = use_d ? node_slot(td, L->node[1], oct, level, &out->oob) : 0;
                int     keep = cs > 0 || cd > 0;
                if (keep && (lev_s || lev_d))
                {
                    /* a child is kept while a tree holding it may have a
                     * leaf near the ray */
                    const uint32_t* rs = lev_s ? ts->cbox + (int64_t) L->node[0] * 16 : NULL;
                    const uint32_t* rd = lev_d ? td->cbox + (int64_t) L->node[1] * 16 : NULL;
                    const int hs = cs > 0 && (!rs || qbo_box_hit(rs[2 * oct], rs[2 * oct + 1], oct, &bf));
                    const int hd = cd > 0 && (!rd || qbo_box_hit(rd[2 * oct], rd[2 * oct + 1], oct, &bf));
                    keep = hs || hd;
                }
                if (keep)
                {
                    int len      = L->ispsi & 0x0F;
                    L->octs[len] = oct;
                    L->isps[len] = act;
                    L->ispsi     = (L->ispsi & 0xF0) | (len + 1);
                }
            }
        }

        int cur_len = L->ispsi & 0x0F;
        if (cur_len > 0)
        {
            /* descend into the next candidate (octree_fsh.c:334-367) */
            int nxt_ind = (L->ispsi >> 4) & 7;
            v4  nxt_isp = L->isps[nxt_ind];
            int nxt_oct = L->octs[nxt_ind];

            float halfs = tlf.w / 2.0f;
            tlf.x += k_xsft[nxt_oct] * halfs;
            tlf.y -= k_ysft[nxt_oct] * halfs;
            tlf.z -= k_zsft[nxt_oct] * halfs;
            tlf.w = halfs;

            nxt_ind++;
            cur_len--;
            L->ispsi = 128 | (nxt_ind << 4) | cur_len;

            int32_t cs = node_slot(ts, L->node[0], nxt_oct, level, &out->oob);
            int32_t cd = use_d ? node_slot(td, L->node[1], nxt_oct, level, &out->oob) : 0;

            if (++pushes > QBO_MAX_PUSHES)
            {
                out->oob = 1;
                return; /* QBO_MISS */
            }
            level += 1;
            level_t* N = &stk[level];
            N->cube    = tlf;
            N->ispsi   = 0;
            N->node[0] = cs;
            N->node[1] = cd;
            N->isps[0] = nxt_isp;
        }
        else
        {
            /* pop (octree_fsh.c:368-375) */
            L->ispsi = 0;
            level -= 1;
            if (level < 0) return; /* QBO_MISS, isp = col = 0 */
        }
    }
}

/* ---- main() helpers (octree_fsh.c:381-395 and GLSL built-ins) ---- */

static float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static void normalize3(const float* v, float* o)
{
    float len = sqrtf(dot3(v, v));
    o[0]      = v[0] / len;
    o[1]      = v[1] / len;
    o[2]      = v[2] / len;
}

/* GLSL max(x, y) = x < y ? y : x */
static float glsl_max(float x, float y) { return x < y ? y : x; }

static void quat_rotate(const float* q, float* v)
{
    /* v + 2.0 * cross(q.xyz, cross(q.xyz, v) + q.w * v) */
    float c1[3] = {q[1] * v[2] - q[2] * v[1], q[2] * v[0] - q[0] * v[2], q[0] * v[1] - q[1] * v[0]};
    float a[3]  = {c1[0] + q[3] * v[0], c1[1] + q[3] * v[1], c1[2] + q[3] * v[2]};
    float c2[3] = {q[1] * a[2] - q[2] * a[1], q[2] * a[0] - q[0] * a[2], q[0] * a[1] - q[1] * a[0]};
    v[0]        = v[0] + 2.0f * c2[0];
    v[1]        = v[1] + 2.0f * c2[1];
    v[2]        = v[2] + 2.0f * c2[2];
}

static void quat_axis_angle(const float* axis, float angle, float* q)
{
    float half = angle * 0.5f;
    q[0]       = axis[0] * sinf(half);
    q[1]       = axis[1] * sinf(half);
    q[2]       = axis[2] * sinf(half);
    q[3]       = cosf(half);
}

uint8_t qbo_unorm8(float f)
{
    if (!(f > 0.0f)) return 0;
    if (f >= 1.0f) return 255;
    return (uint8_t) (f * 255.0f + 0.5f);
}

void qbo_view_setup(float width, float height, const float position[3], const float angle[3], float lighta, int quality, int maxlevel, float basesize, int shoot, float focal, qbo_view* v)
{
    memset(v, 0, sizeof(*v));

    /* octree_glc.c:263-270; the light and size expressions mix float and
     * double exactly as the C source does before storing into GLfloat */
    v->basecube[0] = 0.0f;
    v->basecube[1] = basesize;
    v->basecube[2] = basesize;
    v->basecube[3] = basesize;

    float sl    = sinf(lighta);
    v->light[0] = 420.0f;
    v->light[1] = (float) ((double) 200.0f - (double) sl * 20.0);
    v->light[2] = (float) ((double) 680.0f - (double) sl * 200.0);

    double div = 6.0 - (double) (float) quality / 2.0;
    float  ow  = (float) ((double) width / div);
    float  oh  = (float) ((double) height / div);

    v->dim[0]    = ow;
    v->dim[1]    = oh;
    v->width_px  = (int32_t) ow; /* glViewport takes GLint */
    v->height_px = (int32_t) oh;
    v->coord_scale[0] = v->width_px > 0 ? ow / (float) v->width_px : 1.0f;
    v->coord_scale[1] = v->height_px > 0 ? oh / (float) v->height_px : 1.0f;

    v->camfp[0] = position[0];
    v->camfp[1] = position[1];
    v->camfp[2] = position[2];

    /* octree_fsh.c:403 */
    const float pi = 3.1415926535897932384626433832795f;
    v->cfp[0]      = ow / 2.0f;
    v->cfp[1]      = oh / 2.0f;
    v->cfp[2]      = focal > 0.0f ? focal : (ow / 2.0f) / tanf(pi / 4.0f);

    /* octree_fsh.c:406-408 */
    const float yaxis[3] = {0.0f, 1.0f, 0.0f};
    quat_axis_angle(yaxis, -angle[0], v->qz);
    float vx[3] = {-1.0f, 0.0f, 0.0f};
    quat_rotate(v->qz, vx);
    quat_axis_angle(vx, -angle[1], v->qx);

    /* octree_fsh.c:417-418: camangle < 0.02 is evaluated as
     * dot > cos(0.02f) with dot <= 1 (acos is decreasing and NaN above 1) */
    float camlight[3] = {v->light[0] - v->camfp[0], v->light[1] - v->camfp[1], v->light[2] - v->camfp[2]};
    normalize3(camlight, v->ncamlight);
    double c  = cos((double) 0.02f);
    float  cf = (float) c;
    if ((double) cf > c) cf = nextafterf(cf, -2.0f);
    v->flare_cos = cf;

    v->maxlevel = maxlevel;
    v->shoot    = shoot;
}

void qbo_shade(const float isp[3], const float nrm[3], const float csv[3], const float light[3], float sqr, int shoot, float col[4])
{
    /* octree_fsh.c:431-449 */
    float lghtv[3] = {isp[0] - light[0], isp[1] - light[1], isp[2] - light[2]};
    float nl[3], nn[3], nc[3];
    float neg_l[3] = {-lghtv[0], -lghtv[1], -lghtv[2]};
    float neg_c[3] = {-csv[0], -csv[1], -csv[2]};
    normalize3(neg_l, nl);
    normalize3(nrm, nn);
    normalize3(neg_c, nc);
    float lght_nrm_ang = glsl_max(dot3(nl, nn), 0.0f);
    float camv_nrm_ang = glsl_max(dot3(nc, nn), 0.0f);

    float lit = (15.0f < sqr) ? 0.0f : 1.0f; /* step(sqr, 15.0) */
    float k   = 0.1f + 0.2f * camv_nrm_ang + lght_nrm_ang * lit * 0.7f;
    col[0]    = col[0] * k;
    col[1]    = col[1] * k;
    col[2]    = col[2] * k;
    col[2] *= 0.7f;
    float g = (float) shoot * camv_nrm_ang * 0.1f;
    col[0] += g;
    col[1] += g;
    col[2] += g;
}

void qbo_camera_ray(const qbo_view* v, int i, int j, float out[4])
{
    /* ray generation (octree_fsh.c:402-413); coord is the pixel centre */
    float cx     = ((float) i + 0.5f) * v->coord_scale[0];
    float cy     = ((float) j + 0.5f) * v->coord_scale[1];
    float csv[3] = {cx - v->cfp[0], cy - v->cfp[1], 0.0f - v->cfp[2]};
    quat_rotate(v->qz, csv);
    quat_rotate(v->qx, csv);
    /* camangle's argument (octree_fsh.c:416-417) */
    float ncsv[3];
    normalize3(csv, ncsv);
    out[0] = csv[0];
    out[1] = csv[1];
    out[2] = csv[2];
    out[3] = dot3(v->ncamlight, ncsv);
}

void qbo_shade_pixel(const qbo_scene* sc, const qbo_view* v, int i, int j, float rgba[4], uint32_t* flags, int32_t leaf[4], float isp[4], uint32_t visits[4])
{
    uint32_t f = 0;
    leaf[0] = leaf[1] = leaf[2] = leaf[3] = -1;
    isp[0] = isp[1] = isp[2] = isp[3] = 0.0f;
    visits[0] = visits[1] = visits[2] = visits[3] = 0;
    rgba[0] = rgba[1] = rgba[2] = rgba[3] = 0.0f;

    float ray[4];
    qbo_camera_ray(v, i, j, ray);
    float csv[3]  = {ray[0], ray[1], ray[2]};
    float cosang = ray[3];
    int   flare  = cosang > v->flare_cos && cosang <= 1.0f;

    qbo_hit res;
    qbo_trace(sc, v->basecube, v->maxlevel, v->camfp, csv, &res);
    visits[0] = (uint32_t) res.visits[0];
    visits[1] = (uint32_t) res.visits[1];
    if (res.oob) f |= QBO_PX_OOB;
    if (res.status == QBO_DISCARD)
    {
        *flags = f | QBO_PX_DISCARD;
        return;
    }
    if (res.status == QBO_LEAF)
    {
        f |= QBO_PX_PRIMARY_LEAF;
        leaf[0] = res.leaf[0];
        leaf[1] = res.leaf[1];
    }
    isp[0] = res.isp[0];
    isp[1] = res.isp[1];
    isp[2] = res.isp[2];
    isp[3] = res.isp[3];

    float col[4] = {res.col[0], res.col[1], res.col[2], res.col[3]};

    if (res.isp[3] > 0.0f)
    {
        /* shadow ray and shading (octree_fsh.c:431-449) */
        f |= QBO_PX_SHADED;
        float   lghtv[3] = {res.isp[0] - v->light[0], res.isp[1] - v->light[1], res.isp[2] - v->light[2]};
        qbo_hit lc;
        qbo_trace(sc, v->basecube, v->maxlevel, v->light, lghtv, &lc);
        visits[2] = (uint32_t) lc.visits[0];
        visits[3] = (uint32_t) lc.visits[1];
        if (lc.oob) f |= QBO_PX_OOB;
        if (lc.status == QBO_DISCARD)
        {
            rgba[0] = rgba[1] = rgba[2] = rgba[3] = 0.0f;
            *flags = f | QBO_PX_DISCARD;
            return;
        }
        if (lc.status == QBO_LEAF)
        {
            f |= QBO_PX_SHADOW_LEAF;
            leaf[2] = lc.leaf[0];
            leaf[3] = lc.leaf[1];
        }
        float ispv[3] = {lc.isp[0] - res.isp[0], lc.isp[1] - res.isp[1], lc.isp[2] - res.isp[2]};
        float sqr     = ispv[0] * ispv[0] + ispv[1] * ispv[1] + ispv[2] * ispv[2];

        if (!(15.0f < sqr)) f |= QBO_PX_LIT; /* step(sqr, 15.0) */
        qbo_shade(res.isp, res.nrm, csv, v->light, sqr, v->shoot, col);
    }

    if (flare)
    {
        /* light flare (octree_fsh.c:452-459) */
        f |= QBO_PX_FLARE_TEST;
        float   lghtv[3] = {v->light[0] - v->camfp[0], v->light[1] - v->camfp[1], v->light[2] - v->camfp[2]};
        qbo_hit lc;
        qbo_trace(sc, v->basecube, v->maxlevel, v->camfp, lghtv, &lc);
        if (lc.oob) f |= QBO_PX_OOB;
        if (lc.status == QBO_DISCARD)
        {
            *flags = f | QBO_PX_DISCARD;
            return;
        }
        float resv_x = lc.isp[0] - v->camfp[0];
        if (resv_x / lghtv[0] > 1.0f)
        {
            f |= QBO_PX_FLARE_WHITE;
            col[0] = col[1] = col[2] = col[3] = 1.0f;
        }
    }

    rgba[0] = col[0];
    rgba[1] = col[1];
    rgba[2] = col[2];
    rgba[3] = col[3];
    *flags  = f;
}

static void write_pixel(const qbo_scene* sc, const qbo_view* v, int i, int j, int64_t o, const qbo_frame* out)
{
    float    rgba[4], isp[4];
    uint32_t flags, visits[4];
    int32_t  leaf[4];
    qbo_shade_pixel(sc, v, i, j, rgba, &flags, leaf, isp, visits);
    if (out->rgba) memcpy(out->rgba + o * 4, rgba, sizeof(rgba));
    if (out->rgba8)
        for (int c = 0; c < 4; c++) out->rgba8[o * 4 + c] = qbo_unorm8(rgba[c]);
    if (out->flags) out->flags[o] = flags;
    if (out->leaf) memcpy(out->leaf + o * 4, leaf, sizeof(leaf));
    if (out->isp) memcpy(out->isp + o * 4, isp, sizeof(isp));
    if (out->visits) memcpy(out->visits + o * 4, visits, sizeof(visits));
}

void qbo_render(const qbo_scene* sc, const qbo_view* v, const qbo_frame* out, int threads)
{
    const int W  = v->width_px, H = v->height_px;
    const int tx = (W + 7) / 8, ty = (H + 7) / 8;
    const int nt = tx * ty;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
#endif
    for (int t = 0; t < nt; t++)
    {
        int x0 = (t % tx) * 8, y0 = (t / tx) * 8;
        for (int j = y0; j < y0 + 8 && j < H; j++)
            for (int i = x0; i < x0 + 8 && i < W; i++) write_pixel(sc, v, i, j, (int64_t) j * W + i, out);
    }
    (void) threads;
}

void qbo_render_pixels(const qbo_scene* sc, const qbo_view* v, const int32_t* px, const int32_t* py, int64_t n, const qbo_frame* out, int threads)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; k++) write_pixel(sc, v, px[k], py[k], k, out);
    (void) threads;
}

/* A batch of ray queries, rays k = 0..n-1 (pos, dir: 3 floats each), on
 * `threads` host threads (0: all): per ray its status, leaf node indices,
 * model indices and visits (any output may be NULL). The CPU side of the
 * library's batched queries (qbc_trace_rays); each ray is qbo_trace. */
void qbo_trace_rays(const qbo_scene* sc, const float basecube[4], int maxlevel, const float* pos, const float* dir,
                    int64_t n, int32_t* status, int32_t* leaf, int32_t* model, int32_t* visits, int threads)
{
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; k++)
    {
        qbo_hit h;
        qbo_trace(sc, basecube, maxlevel, pos + 3 * k, dir + 3 * k, &h);
        if (status) status[k] = h.status;
        if (leaf)
        {
            leaf[2 * k]     = h.leaf[0];
            leaf[2 * k + 1] = h.leaf[1];
        }
        if (model)
        {
            model[2 * k]     = h.model[0];
            model[2 * k + 1] = h.model[1];
        }
        if (visits)
        {
            visits[2 * k]     = h.visits[0];
            visits[2 * k + 1] = h.visits[1];
        }
    }
    (void) threads;
}
