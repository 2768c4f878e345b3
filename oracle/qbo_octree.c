/*
 * CPU oracle (test infrastructure only): restatement of the node-array
 * producer in src/qubatron/octree.c. Nodes are 12 int32: 8 child indices,
 * the model index of the point that created the node, 3 pad (octree.c:11-14).
 */
#include "qbo.h"

#include <string.h>

/* Octet of a point at each level (octree.c:100-109): size halves from the
 * basecube edge, x picks bit 0, y below the midline picks bit 1 and z behind
 * it picks bit 2, all from the float quotient truncated to int. */
void qbo_point_octets(float basesize, int levels, const float pnt[3], int32_t* octets)
{
    float size = basesize;
    for (int level = 0; level < levels; level++)
    {
        size /= 2.0f;
        int octet = (int) (pnt[0] / size) % 2;
        int yi    = (int) (pnt[1] / size) % 2;
        int zi    = (int) (pnt[2] / size) % 2;
        if (yi == 0) octet += 2;
        if (zi == 0) octet += 4;
        octets[level] = octet;
    }
}

static int append_node(int32_t* nodes, int64_t* len, int64_t cap, int64_t parent, int octet, int64_t modind)
{
    if (*len >= cap) return -1;
    nodes[parent * 12 + octet] = (int32_t) *len;
    memset(&nodes[*len * 12], 0, 12 * sizeof(int32_t));
    nodes[*len * 12 + 8] = (int32_t) modind;
    (*len)++;
    return 0;
}

/* octree_insert_point (octree.c:95-147), starting at the root. octindarr, when
 * given, receives the parent and new node of the first level that grew. */
int qbo_insert_point(int32_t* nodes, int64_t* len, int64_t cap, float basesize, int levels, int64_t modind, const float pnt[3], int32_t* octindarr)
{
    int32_t octets[32];
    qbo_point_octets(basesize, levels, pnt, octets);
    int64_t index = 0;
    for (int level = 0; level < levels; level++)
    {
        int octet = octets[level];
        if (nodes[index * 12 + octet] == 0)
        {
            if (octindarr != NULL)
            {
                octindarr[level]     = (int32_t) index;
                octindarr[level + 1] = (int32_t) *len;
            }
            if (append_node(nodes, len, cap, index, octet, modind)) return -1;
        }
        index = nodes[index * 12 + octet];
    }
    return 0;
}

/* octree_insert_path (octree.c:149-180) with the octets in one array instead
 * of the three 4-wide transform-feedback buffers. */
int qbo_insert_path(int32_t* nodes, int64_t* len, int64_t cap, int levels, int64_t modind, const int32_t* octets)
{
    int64_t index = 0;
    for (int level = 0; level < levels; level++)
    {
        int octet = octets[level];
        if (nodes[index * 12 + octet] == 0)
            if (append_node(nodes, len, cap, index, octet, modind)) return -1;
        index = nodes[index * 12 + octet];
    }
    return 0;
}

/* octree_remove_point (octree.c:182-218): zero the parent's pointer to the
 * leaf holding pnt and report the leaf's model index and the parent node. */
void qbo_remove_point(int32_t* nodes, float basesize, int levels, const float pnt[3], int32_t* modind, int32_t* octind)
{
    float   size   = basesize;
    int32_t index  = 0;
    int32_t lindex = 0;
    int     loctet = 0;
    for (int level = 0; level < levels + 1; level++)
    {
        size /= 2.0f;
        int octet = (int) (pnt[0] / size) % 2;
        int yi    = (int) (pnt[1] / size) % 2;
        int zi    = (int) (pnt[2] / size) % 2;
        if (yi == 0) octet += 2;
        if (zi == 0) octet += 4;

        if (level == levels)
        {
            *modind                            = nodes[(int64_t) index * 12 + 8];
            *octind                            = lindex;
            nodes[(int64_t) lindex * 12 + loctet] = 0;
        }
        lindex = index;
        loctet = octet;
        index  = nodes[(int64_t) index * 12 + octet];
        if (index == 0) return;
    }
}

/* n qbo_remove_point calls in input order (the reference's sequence of
 * octree_remove_point calls); a point whose walk meets an empty link leaves
 * its modind / octind entries as they were. */
void qbo_remove_points(int32_t* nodes, float basesize, int levels, const float* pnts, int64_t n, int32_t* modind,
                       int32_t* octind)
{
    for (int64_t k = 0; k < n; k++) qbo_remove_point(nodes, basesize, levels, pnts + 3 * k, modind + k, octind + k);
}
