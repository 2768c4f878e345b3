/*
 * CPU oracle (test infrastructure only): the leaf-box pruning of the CUDA
 * library, restated so that the visit counts of a pruned walk can be checked
 * as well as its pixels. The reference shader has no such filter; a scene
 * without boxes (the default) is walked exactly as the shader walks it.
 *
 * qbo_build_boxes restates the library's box build (qubatron_gb300/csrc/
 * boxes.cu: integer work, same rules for refusing an array), and
 * qbo_box_frame / qbo_box_hit restate its float test (trace.cuh: BoxFrame,
 * child_box_hit) operation for operation: built with -ffp-contract=off, the
 * one fused multiply-add per bound is an explicit fmaf, so every pruning
 * decision matches the GPU's.
 */
#include "qbo.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define QBO_BOX_MAX_LEVEL 17 /* deepest render level (the shader's stack holds 18) */

int32_t qbo_build_boxes(const int32_t* nodes, int64_t n, uint32_t* rec)
{
    if (n <= 0) return -1;
    memset(rec, 0, (size_t) n * 16 * sizeof(uint32_t));
    int32_t* order = (int32_t*) malloc((size_t) n * sizeof(int32_t));
    uint8_t* seen  = (uint8_t*) calloc((size_t) n, 1);
    int32_t* box   = (int32_t*) malloc((size_t) n * 6 * sizeof(int32_t));
    int64_t  off[QBO_BOX_MAX_LEVEL + 4];
    int      depth = -1;
    if (!order || !seen || !box) goto done;

    /* breadth first from the root: level L holds order[off[L], off[L+1]);
     * the expansion runs for levels 0 .. QBO_BOX_MAX_LEVEL + 1 */
    order[0] = 0;
    seen[0]  = 1;
    off[0]   = 0;
    off[1]   = 1;
    int nlev = 1; /* levels with an end in off */
    for (int L = 0; L <= QBO_BOX_MAX_LEVEL + 1; ++L)
    {
        const int64_t b = off[L], e = off[L + 1];
        if (e == b) break;
        int64_t total = e;
        for (int64_t j = b; j < e; ++j)
        {
            const int32_t* nd = nodes + (int64_t) order[j] * 12;
            for (int o = 0; o < 8; ++o)
            {
                const int32_t c = nd[o];
                if (c > 0 && c < n)
                {
                    if (seen[c]) goto done; /* reached twice: not a tree */
                    seen[c]          = 1;
                    order[total++]   = c;
                }
                else if (c != 0)
                    goto done; /* an index outside the array */
            }
        }
        off[L + 2] = total;
        nlev       = L + 2;
    }
    /* the deepest level with nodes */
    int D = 0;
    while (D + 2 <= nlev && off[D + 2] > off[D + 1]) ++D;
    if (D > QBO_BOX_MAX_LEVEL) goto done;

    /* exact boxes in leaf cells relative to each node's cube, bottom up */
    for (int L = D; L >= 0; --L)
    {
        const int32_t half = L == D ? 0 : (int32_t) 1 << (D - L - 1);
        for (int64_t j = off[L]; j < off[L + 1]; ++j)
        {
            const int32_t  node = order[j];
            int32_t*       r    = box + (int64_t) node * 6;
            if (L == D)
            {
                for (int k = 0; k < 6; ++k) r[k] = 0;
                continue;
            }
            r[0] = r[2] = r[4] = INT_MAX;
            r[1] = r[3] = r[5] = -1;
            for (int o = 0; o < 8; ++o)
            {
                const int32_t c = nodes[(int64_t) node * 12 + o];
                if (!(c > 0 && c < n)) continue;
                const int32_t* cb = box + (int64_t) c * 6;
                if (cb[1] < cb[0]) continue; /* no leaves below */
                const int32_t sh[3] = {(o & 1) ? half : 0, (o & 2) ? half : 0, (o & 4) ? half : 0};
                for (int k = 0; k < 3; ++k)
                {
                    if (cb[2 * k] + sh[k] < r[2 * k]) r[2 * k] = cb[2 * k] + sh[k];
                    if (cb[2 * k + 1] + sh[k] > r[2 * k + 1]) r[2 * k + 1] = cb[2 * k + 1] + sh[k];
                }
            }
        }
    }
    /* records: each child's box rounded outward to 1/256 of its edge */
    for (int L = 0; L < D; ++L)
    {
        const int64_t cells = (int64_t) 1 << (D - L - 1);
        for (int64_t j = off[L]; j < off[L + 1]; ++j)
        {
            const int32_t node = order[j];
            uint32_t*     w    = rec + (int64_t) node * 16;
            for (int o = 0; o < 8; ++o)
            {
                uint32_t      q[6] = {255u, 0u, 255u, 0u, 255u, 0u}; /* empty */
                const int32_t c    = nodes[(int64_t) node * 12 + o];
                if (c > 0 && c < n)
                {
                    const int32_t* cb = box + (int64_t) c * 6;
                    if (cb[0] <= cb[1])
                    {
                        for (int k = 0; k < 3; ++k)
                        {
                            const int64_t lo = cb[2 * k], hi1 = (int64_t) cb[2 * k + 1] + 1;
                            const int64_t ql = lo * 256 / cells;
                            const int64_t qh = (hi1 * 256 + cells - 1) / cells - 1;
                            q[2 * k]         = (uint32_t) (ql < 0 ? 0 : (ql > 255 ? 255 : ql));
                            q[2 * k + 1]     = (uint32_t) (qh < 0 ? 0 : (qh > 255 ? 255 : qh));
                        }
                    }
                }
                w[2 * o]     = q[0] | (q[1] << 8) | (q[2] << 16) | (q[3] << 24);
                w[2 * o + 1] = q[4] | (q[5] << 8);
            }
        }
    }
    depth = D;
done:
    if (depth < 0) memset(rec, 0, (size_t) n * 16 * sizeof(uint32_t));
    free(order);
    free(seen);
    free(box);
    return depth;
}

void qbo_box_frame(const float cube[4], const float p[3], const float inv[3], float m, qbo_box_frame_t* f)
{
    const float unit = cube[3] * 0.001953125f; /* 1/512 of the node's edge */
    const float ax = (cube[0] - p[0]) * inv[0], mx = m * inv[0];
    const float ay = (cube[1] - p[1]) * inv[1], my = m * inv[1];
    const float az = (cube[2] - p[2]) * inv[2], mz = m * inv[2];
    f->a0[0] = ax - mx;
    f->a1[0] = ax + mx;
    f->u[0]  = unit * inv[0];
    f->a0[1] = ay - my;
    f->a1[1] = ay + my;
    f->u[1]  = -(unit * inv[1]);
    f->a0[2] = az - mz;
    f->a1[2] = az + mz;
    f->u[2]  = -(unit * inv[2]);
}

/* byte k of w as a float: bits 0x4B0000kk are 2^23 + k */
static float byte_float(uint32_t w, int k)
{
    const uint32_t bits = 0x4B000000u | ((w >> (8 * k)) & 0xFFu);
    float          f;
    memcpy(&f, &bits, sizeof(f));
    return f;
}

int qbo_box_hit(uint32_t rx, uint32_t ry, int o, const qbo_box_frame_t* f)
{
    const float kx = (o & 1) ? 8388352.0f : 8388608.0f, ky = (o & 2) ? 8388352.0f : 8388608.0f,
                kz = (o & 4) ? 8388352.0f : 8388608.0f;
    const float xlo = byte_float(rx, 0) - kx, xhi = byte_float(rx, 1) - (kx - 1.0f);
    const float ylo = byte_float(rx, 2) - ky, yhi = byte_float(rx, 3) - (ky - 1.0f);
    const float zlo = byte_float(ry, 0) - kz, zhi = byte_float(ry, 1) - (kz - 1.0f);
    float t0 = fmaf(xlo, f->u[0], f->a0[0]), t1 = fmaf(xhi, f->u[0], f->a1[0]);
    float tn = fminf(t0, t1), tf = fmaxf(t0, t1);
    t0 = fmaf(yhi, f->u[1], f->a0[1]);
    t1 = fmaf(ylo, f->u[1], f->a1[1]);
    tn = fmaxf(tn, fminf(t0, t1));
    tf = fminf(tf, fmaxf(t0, t1));
    t0 = fmaf(zhi, f->u[2], f->a0[2]);
    t1 = fmaf(zlo, f->u[2], f->a1[2]);
    tn = fmaxf(tn, fminf(t0, t1));
    tf = fminf(tf, fmaxf(t0, t1));
    return (xlo < xhi) && (tn <= tf) && (tf >= 0.0f);
}

/* The per-ray conditions of the library's filter: a basecube (+0, S, S, S)
 * whose cube coordinates stay exact to maxlevel, operands for which the
 * division by reciprocal is exact, every direction component nonzero and the
 * origin within 8 basecube edges. */
static int odd_bits(float s)
{
    int      e = 0;
    float    f = frexpf(s, &e);
    uint32_t m = (uint32_t) ldexpf(f, 24);
    if (m == 0) return 0;
    while ((m & 1u) == 0) m >>= 1;
    int b = 0;
    while (m)
    {
        ++b;
        m >>= 1;
    }
    return b;
}

int qbo_box_ray_ok(const float bc[4], int maxlevel, const float p[3], const float d[3])
{
    const float s = bc[3];
    if (!(s > 0.0f) || !isfinite(s) || !isnormal(s)) return 0;
    if (bc[0] != 0.0f || signbit(bc[0])) return 0;
    if (bc[1] != s || bc[2] != s) return 0;
    if (ldexpf(s, -maxlevel) < 1.17549435e-38f) return 0;
    if (odd_bits(s) + maxlevel > 24) return 0;
    for (int k = 0; k < 3; ++k)
    {
        const float a = fabsf(d[k]), b = fabsf(p[k]);
        if (!((a == 0.0f) || (a >= 9.094947e-13f && a <= 1.0995116e12f))) return 0;
        if (!((b == 0.0f) || (b >= 2.1684043e-19f && b <= 1.8446744e19f))) return 0;
    }
    if (!(s >= 9.536743e-07f && s <= 1.0995116e12f)) return 0;
    const float r8 = 8.0f * s;
    for (int k = 0; k < 3; ++k)
        if (d[k] == 0.0f || !(fabsf(p[k]) <= r8)) return 0;
    return 1;
}
