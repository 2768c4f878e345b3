/*
 * Flat entry points over the reference's own src/qubatron/octree.c and
 * src/qubatron/model.c, compiled from the reference sources by
 * oracle/build_ref.sh into oracle/_ref. Test infrastructure only: it pins the
 * oracle's restatement (qbo_octree.c, qbo_trace.c) to the reference's CPU
 * insertion and static-tree traversal, and the library's flat-file reader to
 * the reference's model_load_flat.
 */
#include "octree.c" /* declarations only: included below level 0 */
#include "model.c"
#include "mt_quat.c"

#include <string.h>

/* Build a static tree with octree_insert_point (octree.c:95-147) for points in
 * order; returns the node count, copying nodes into out when they fit. */
long qbref_build(const float* pts, long n, float basesize, int levels, int* out, long cap)
{
    octree_t tree = octree_create((v4_t){0.0f, basesize, basesize, basesize}, levels);
    for (long i = 0; i < n; i++)
        octree_insert_point(&tree, 0, (size_t) i, (v3_t){pts[i * 3 + 0], pts[i * 3 + 1], pts[i * 3 + 2]}, NULL);
    long len = (long) tree.len;
    if (out != NULL && len <= cap) memcpy(out, tree.octs, (size_t) len * sizeof(octets_t));
    octree_delete(&tree);
    return len;
}

/* Build with octree_insert_path (octree.c:149-180) from per-point octets
 * (levels <= 12, one row of 12 per point). */
long qbref_build_paths(const int* octets, long n, float basesize, int levels, int* out, long cap)
{
    octree_t tree = octree_create((v4_t){0.0f, basesize, basesize, basesize}, levels);
    for (long i = 0; i < n; i++)
    {
        int o14[4], o54[4], o94[4];
        for (int k = 0; k < 4; k++)
        {
            o14[k] = octets[i * 12 + k];
            o54[k] = octets[i * 12 + 4 + k];
            o94[k] = octets[i * 12 + 8 + k];
        }
        octree_insert_path(&tree, 0, (size_t) i, o14, o54, o94);
    }
    long len = (long) tree.len;
    if (out != NULL && len <= cap) memcpy(out, tree.octs, (size_t) len * sizeof(octets_t));
    octree_delete(&tree);
    return len;
}

/* octree_remove_point (octree.c:182-218) on a caller-owned node array. */
void qbref_remove(int* nodes, long n_nodes, float basesize, int levels, const float* pnt, int* modind, int* octind)
{
    octree_t tree;
    tree.basecube = (v4_t){0.0f, basesize, basesize, basesize};
    tree.octs     = (octets_t*) nodes;
    tree.size     = (size_t) n_nodes;
    tree.len      = (size_t) n_nodes;
    tree.levels   = levels;
    octree_remove_point(&tree, (v3_t){pnt[0], pnt[1], pnt[2]}, modind, octind);
}

/* octree_trace_line (octree.c:341-537) for n rays; out_tlf gets the leaf cube,
 * w = -1 when no leaf was reached. */
void qbref_trace(const int* nodes, long n_nodes, float basesize, int levels, const float* pos, const float* dir, long n, int* out_model, float* out_tlf)
{
    octree_t tree;
    tree.basecube = (v4_t){0.0f, basesize, basesize, basesize};
    tree.octs     = (octets_t*) nodes;
    tree.size     = (size_t) n_nodes;
    tree.len      = (size_t) n_nodes;
    tree.levels   = levels;
    for (long i = 0; i < n; i++)
    {
        v4_t tlf       = {0.0f, 0.0f, 0.0f, -1.0f};
        out_model[i]   = octree_trace_line(&tree, (v3_t){pos[i * 3], pos[i * 3 + 1], pos[i * 3 + 2]}, (v3_t){dir[i * 3], dir[i * 3 + 1], dir[i * 3 + 2]}, &tlf);
        out_tlf[i * 4 + 0] = tlf.x;
        out_tlf[i * 4 + 1] = tlf.y;
        out_tlf[i * 4 + 2] = tlf.z;
        out_tlf[i * 4 + 3] = tlf.w;
    }
}

/* model_load_flat (model.c:53-111) on the four paths; returns the point count
 * and copies the float3 arrays (3 floats per point) and the range ints when
 * they fit. */
long qbref_load_flat(const char* pnt, const char* col, const char* nrm, const char* rng, float* vtx, float* cols,
                     float* nrms, long cap, int* ranges, long rcap, long* range_count)
{
    model_t m = model_init();
    model_load_flat(&m, (char*) pnt, (char*) col, (char*) nrm, (char*) rng);
    long n = m.point_count;
    if (vtx != NULL && n <= cap)
    {
        memcpy(vtx, m.vertexes, (size_t) n * 3 * sizeof(float));
        memcpy(cols, m.colors, (size_t) n * 3 * sizeof(float));
        memcpy(nrms, m.normals, (size_t) n * 3 * sizeof(float));
    }
    *range_count = m.range_count;
    if (ranges != NULL && m.range_count <= rcap) memcpy(ranges, m.ranges, (size_t) m.range_count * sizeof(int));
    return n;
}

/* The frame quaternions of the shader's main() (octree_fsh.c:406-408) with the
 * reference's C quaternion functions (mt_quat.c:14-29, the same formulas as
 * the shader's quat_from_axis_angle / quat_rotate at octree_fsh.c:381-395):
 * qz about +y by -angle.x, qx about qz-rotated -x by -angle.y. */
void qbref_frame_quats(float angle_x, float angle_y, float* qz, float* qx)
{
    v4_t z  = quat_from_axis_angle((v3_t){0.0f, 1.0f, 0.0f}, -angle_x);
    v3_t vx = quat_rotate(z, (v3_t){-1.0f, 0.0f, 0.0f});
    v4_t x  = quat_from_axis_angle(vx, -angle_y);
    qz[0] = z.x, qz[1] = z.y, qz[2] = z.z, qz[3] = z.w;
    qx[0] = x.x, qx[1] = x.y, qx[2] = x.z, qx[3] = x.w;
}

/* csv = quat_rotate(qx, quat_rotate(qz, ctp - cfp)) (octree_fsh.c:402-413)
 * for n screen points ctp (x, y; z = 0). */
void qbref_camera_dirs(const float* qz, const float* qx, const float* cfp, const float* ctp, long n, float* out)
{
    v4_t z = {qz[0], qz[1], qz[2], qz[3]}, x = {qx[0], qx[1], qx[2], qx[3]};
    for (long i = 0; i < n; i++)
    {
        v3_t csv = v3_sub((v3_t){ctp[2 * i], ctp[2 * i + 1], 0.0f}, (v3_t){cfp[0], cfp[1], cfp[2]});
        csv      = quat_rotate(z, csv);
        csv      = quat_rotate(x, csv);
        out[3 * i + 0] = csv.x;
        out[3 * i + 1] = csv.y;
        out[3 * i + 2] = csv.z;
    }
}

/* The shading of octree_fsh.c:431-449 written with the reference's own C
 * vector helpers (mt_vector_3d.c: v3_sub, v3_scale, v3_normalize, v3_dot).
 * v3_normalize multiplies by 1 / sqrt where the shader restatement divides,
 * so this twin agrees with it to within a few ulps, not bit for bit; it pins
 * the formula. col is shaded in place. */
void qbref_shade(const float* isp, const float* nrm, const float* csv, const float* light, float sqr, int shoot, float* col)
{
    v3_t  ispv  = {isp[0], isp[1], isp[2]};
    v3_t  lghtv = v3_sub(ispv, (v3_t){light[0], light[1], light[2]});
    v3_t  n     = v3_normalize((v3_t){nrm[0], nrm[1], nrm[2]});
    float lght  = v3_dot(v3_normalize(v3_scale(lghtv, -1.0f)), n);
    float camv  = v3_dot(v3_normalize(v3_scale((v3_t){csv[0], csv[1], csv[2]}, -1.0f)), n);
    float lght_nrm_ang = lght > 0.0f ? lght : 0.0f;
    float camv_nrm_ang = camv > 0.0f ? camv : 0.0f;
    float lit = 15.0f < sqr ? 0.0f : 1.0f; /* step(sqr, 15.0) */
    float k   = 0.1f + 0.2f * camv_nrm_ang + lght_nrm_ang * lit * 0.7f;
    v3_t  c   = v3_scale((v3_t){col[0], col[1], col[2]}, k);
    c.z *= 0.7f;
    float g = (float) shoot * camv_nrm_ang * 0.1f;
    col[0]  = c.x + g;
    col[1]  = c.y + g;
    col[2]  = c.z + g;
}
