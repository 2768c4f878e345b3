/*
 * CPU oracle (test infrastructure only): the seeded synthetic scenes of the
 * benchmark workloads, restated in plain C so that the benchmark's reference
 * arm builds the same scene without loading any part of the CUDA library.
 *
 * The reference's own assets (the res/ point, normal and colour files) are absent, so every
 * workload is a procedural scene: axis-aligned rectangles (floor, room walls,
 * five faces per box) and spheres, points drawn in proportion to surface
 * area, exact normals, per-primitive colours with optional uniform noise, all
 * from a splitmix64 stream. Points are returned in octree-path order (a
 * stable sort by the octets of src/qubatron/octree.c:100-109, root level most
 * significant), the order a voxel-sorted asset has.
 *
 * The definition is the one the library's qbc_scene_generate implements; a
 * CPU test requires both to give identical bits. Only +, -, *, / and sqrt
 * touch the floats (compiled with -ffp-contract=off), so the bits are the
 * same on every machine.
 */
#include "qbo.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct
{
    uint64_t state;
} qs_rng;

static uint64_t qs_next(qs_rng* r)
{
    uint64_t z = (r->state += 0x9E3779B97F4A7C15ull);
    z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* uniform in [0, 1): 24 bits as float, 53 bits as double */
static float  qs_unit(qs_rng* r) { return (float) (qs_next(r) >> 40) * (1.0f / 16777216.0f); }
static double qs_unit_d(qs_rng* r) { return (double) (qs_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static float  qs_between(qs_rng* r, float a, float b) { return a + (b - a) * qs_unit(r); }

static float qs_minf(float a, float b) { return b < a ? b : a; }
static float qs_maxf(float a, float b) { return a < b ? b : a; }

/* A surface: rectangle origin + a*edge0 + b*edge1 (a, b in [0, 1)), or a
 * sphere (centre, radius). */
typedef struct
{
    int    is_sphere;
    float  origin[3], edge0[3], edge1[3], normal[3];
    float  centre[3], radius;
    float  rgb[3];
    double area;
} qs_surface;

typedef struct
{
    qs_surface* s;
    size_t      n, cap;
} qs_list;

static qs_surface* qs_push(qs_list* l)
{
    if (l->n == l->cap)
    {
        l->cap = l->cap ? 2 * l->cap : 64;
        l->s   = (qs_surface*) realloc(l->s, l->cap * sizeof(qs_surface));
    }
    qs_surface* s = &l->s[l->n++];
    memset(s, 0, sizeof(*s));
    return s;
}

static void qs_rect(qs_list* l, float ox, float oy, float oz, const float e0[3], const float e1[3], float nx, float ny, float nz, const float rgb[3])
{
    qs_surface* s = qs_push(l);
    s->origin[0] = ox, s->origin[1] = oy, s->origin[2] = oz;
    s->normal[0] = nx, s->normal[1] = ny, s->normal[2] = nz;
    for (int k = 0; k < 3; k++)
    {
        s->edge0[k] = e0[k];
        s->edge1[k] = e1[k];
        s->rgb[k]   = rgb[k];
    }
    double l0 = sqrt((double) e0[0] * e0[0] + (double) e0[1] * e0[1] + (double) e0[2] * e0[2]);
    double l1 = sqrt((double) e1[0] * e1[0] + (double) e1[1] * e1[1] + (double) e1[2] * e1[2]);
    s->area   = l0 * l1;
}

/* The five visible faces of a box standing on y = y0: top, +z, -z, -x, +x. */
static void qs_box(qs_list* l, float x0, float y0, float z0, float sx, float sy, float sz, const float rgb[3])
{
    const float ex[3] = {sx, 0.0f, 0.0f}, ey[3] = {0.0f, sy, 0.0f}, ez[3] = {0.0f, 0.0f, sz};
    qs_rect(l, x0, y0 + sy, z0, ex, ez, 0.0f, 1.0f, 0.0f, rgb);
    qs_rect(l, x0, y0, z0 + sz, ex, ey, 0.0f, 0.0f, 1.0f, rgb);
    qs_rect(l, x0, y0, z0, ex, ey, 0.0f, 0.0f, -1.0f, rgb);
    qs_rect(l, x0, y0, z0, ey, ez, -1.0f, 0.0f, 0.0f, rgb);
    qs_rect(l, x0 + sx, y0, z0, ey, ez, 1.0f, 0.0f, 0.0f, rgb);
}

static void qs_sphere(qs_list* l, float cx, float cy, float cz, float r, const float rgb[3])
{
    qs_surface* s = qs_push(l);
    s->is_sphere  = 1;
    s->centre[0] = cx, s->centre[1] = cy, s->centre[2] = cz;
    s->radius = r;
    for (int k = 0; k < 3; k++) s->rgb[k] = rgb[k];
    s->area = 4.0 * 3.14159265358979323846 * (double) r * (double) r;
}

static void qs_colour(qs_rng* r, float rgb[3])
{
    rgb[0] = qs_unit(r);
    rgb[1] = qs_unit(r);
    rgb[2] = qs_unit(r);
}

/* A closed room: floor, ceiling (one colour) and four walls (another). */
static void qs_house_room(qs_list* l, qs_rng* r, float x0, float y0, float z0, float rw, float fh, float rd)
{
    float rgb[3];
    const float ex[3] = {rw, 0.0f, 0.0f}, ey[3] = {0.0f, fh, 0.0f}, ez[3] = {0.0f, 0.0f, rd};
    qs_colour(r, rgb);
    qs_rect(l, x0, y0, z0, ex, ez, 0.0f, 1.0f, 0.0f, rgb);
    qs_rect(l, x0, y0 + fh, z0, ex, ez, 0.0f, -1.0f, 0.0f, rgb);
    qs_colour(r, rgb);
    qs_rect(l, x0, y0, z0, ey, ez, 1.0f, 0.0f, 0.0f, rgb);
    qs_rect(l, x0 + rw, y0, z0, ey, ez, -1.0f, 0.0f, 0.0f, rgb);
    qs_rect(l, x0, y0, z0, ex, ey, 0.0f, 0.0f, 1.0f, rgb);
    qs_rect(l, x0, y0, z0 + rd, ex, ey, 0.0f, 0.0f, -1.0f, rgb);
}

/* Stable LSD radix sort of perm by key (11-bit digits). */
static int qs_sort(uint64_t* key, uint32_t* perm, size_t n, int key_bits)
{
    uint64_t* k2 = (uint64_t*) malloc(n * sizeof(uint64_t));
    uint32_t* p2 = (uint32_t*) malloc(n * sizeof(uint32_t));
    if (!k2 || !p2)
    {
        free(k2);
        free(p2);
        return -1;
    }
    enum { D = 11, B = 1 << D };
    size_t* count = (size_t*) malloc(B * sizeof(size_t));
    for (int sh = 0; sh < key_bits; sh += D)
    {
        memset(count, 0, B * sizeof(size_t));
        for (size_t i = 0; i < n; i++) count[(key[i] >> sh) & (B - 1)]++;
        size_t run = 0;
        for (int b = 0; b < B; b++)
        {
            size_t c = count[b];
            count[b] = run;
            run += c;
        }
        for (size_t i = 0; i < n; i++)
        {
            size_t at = count[(key[i] >> sh) & (B - 1)]++;
            k2[at]    = key[i];
            p2[at]    = perm[i];
        }
        memcpy(key, k2, n * sizeof(uint64_t));
        memcpy(perm, p2, n * sizeof(uint32_t));
    }
    free(count);
    free(k2);
    free(p2);
    return 0;
}

int qbo_scene_generate(int kind, int levels, int64_t n, uint64_t seed, float S, int n_boxes, float box_min, float box_max, int n_spheres, float sphere_min, float sphere_max, float noise, float* pnts, float* nrms, float* cols)
{
    if (n <= 0 || n > 0xFFFFFFFFll || levels < 1 || levels > 21 || !(S > 0.0f)) return -1;
    qs_rng  rng = {seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
    qs_list L   = {0};
    float   rgb[3];

    /* placement bounds of boxes and spheres in a single-room scene */
    float floor_y = 0.0f, ceil_y = S, lo = 0.0f, hi = S;
    const float m = 0.02f * S; /* wall inset of the room and house */
    if (kind == 0)
    {
        floor_y = 0.05f * S;
        qs_colour(&rng, rgb);
        const float ex[3] = {S, 0.0f, 0.0f}, ez[3] = {0.0f, 0.0f, S};
        qs_rect(&L, 0.0f, floor_y, 0.0f, ex, ez, 0.0f, 1.0f, 0.0f, rgb);
    }
    else if (kind == 1)
    {
        const float h = 0.6f * S, w = S - 2.0f * m;
        floor_y = m, ceil_y = m + h, lo = m, hi = S - m;
        const float ew[3] = {w, 0.0f, 0.0f}, eh[3] = {0.0f, h, 0.0f}, ed[3] = {0.0f, 0.0f, w};
        qs_colour(&rng, rgb);
        qs_rect(&L, m, m, m, ew, ed, 0.0f, 1.0f, 0.0f, rgb); /* floor */
        qs_colour(&rng, rgb);
        qs_rect(&L, m, m + h, m, ew, ed, 0.0f, -1.0f, 0.0f, rgb); /* ceiling */
        qs_colour(&rng, rgb);
        qs_rect(&L, m, m, m, eh, ed, 1.0f, 0.0f, 0.0f, rgb); /* x = m */
        qs_colour(&rng, rgb);
        qs_rect(&L, S - m, m, m, eh, ed, -1.0f, 0.0f, 0.0f, rgb); /* x = S - m */
        qs_colour(&rng, rgb);
        qs_rect(&L, m, m, m, ew, eh, 0.0f, 0.0f, 1.0f, rgb); /* z = m */
        qs_colour(&rng, rgb);
        qs_rect(&L, m, m, S - m, ew, eh, 0.0f, 0.0f, -1.0f, rgb); /* z = S - m */
    }
    else if (kind == 2)
    {
        const float fh = (S - 2.0f * m) / 3.0f, rw = (S - 2.0f * m) / 3.0f, rd = (S - 2.0f * m) / 2.0f;
        for (int f = 0; f < 3; f++)
            for (int rx = 0; rx < 3; rx++)
                for (int rz = 0; rz < 2; rz++) qs_house_room(&L, &rng, m + rx * rw, m + f * fh, m + rz * rd, rw, fh, rd);
    }
    else
    {
        return -1;
    }

    /* x0 x1 y0 y1 z0 z1 of the room a box or sphere goes into */
    float rb[6];
#define QS_ROOM()                                                                                               \
    do {                                                                                                        \
        if (kind != 2)                                                                                          \
        {                                                                                                       \
            rb[0] = lo, rb[1] = hi, rb[2] = floor_y, rb[3] = ceil_y, rb[4] = lo, rb[5] = hi;                    \
        }                                                                                                       \
        else                                                                                                    \
        {                                                                                                       \
            const float fh = (S - 2.0f * m) / 3.0f, rw = (S - 2.0f * m) / 3.0f, rd = (S - 2.0f * m) / 2.0f;     \
            const int   room = (int) (qs_next(&rng) % 18u);                                                     \
            rb[0] = m + (room / 2) % 3 * rw, rb[1] = rb[0] + rw;                                                \
            rb[2] = m + room / 6 * fh, rb[3] = rb[2] + fh;                                                      \
            rb[4] = m + room % 2 * rd, rb[5] = rb[4] + rd;                                                      \
        }                                                                                                       \
    } while (0)

    for (int b = 0; b < n_boxes; b++)
    {
        QS_ROOM();
        float sx = qs_between(&rng, box_min, box_max);
        float sy = qs_between(&rng, box_min, box_max);
        float sz = qs_between(&rng, box_min, box_max);
        sx       = qs_minf(sx, 0.9f * (rb[1] - rb[0]));
        sz       = qs_minf(sz, 0.9f * (rb[5] - rb[4]));
        sy       = qs_minf(sy, 0.9f * (rb[3] - rb[2]));
        float x0 = qs_between(&rng, rb[0], rb[1] - sx);
        float z0 = qs_between(&rng, rb[4], rb[5] - sz);
        qs_colour(&rng, rgb);
        qs_box(&L, x0, rb[2], z0, sx, sy, sz, rgb);
    }
    for (int s = 0; s < n_spheres; s++)
    {
        QS_ROOM();
        float r  = qs_between(&rng, sphere_min, sphere_max);
        r        = qs_minf(r, 0.45f * qs_minf(qs_minf(rb[1] - rb[0], rb[5] - rb[4]), rb[3] - rb[2]));
        float cx = qs_between(&rng, rb[0] + r, rb[1] - r);
        float cy = qs_between(&rng, rb[2] + r, rb[3] - r);
        float cz = qs_between(&rng, rb[4] + r, rb[5] - r);
        qs_colour(&rng, rgb);
        qs_sphere(&L, cx, cy, cz, r, rgb);
    }
#undef QS_ROOM

    /* cumulative area: a point picks the first surface whose running sum
     * exceeds u * total */
    double* cum   = (double*) malloc(L.n * sizeof(double));
    double  total = 0.0;
    for (size_t i = 0; i < L.n; i++)
    {
        total += L.s[i].area;
        cum[i] = total;
    }

    uint64_t* key  = (uint64_t*) malloc((size_t) n * sizeof(uint64_t));
    uint32_t* perm = (uint32_t*) malloc((size_t) n * sizeof(uint32_t));
    int       rc   = (key && perm && cum) ? 0 : -1;
    for (int64_t i = 0; i < n && rc == 0; i++)
    {
        const double u = qs_unit_d(&rng) * total;
        size_t       a = 0, b = L.n; /* first cum[k] > u */
        while (a < b)
        {
            size_t mid = (a + b) / 2;
            if (cum[mid] > u)
                b = mid;
            else
                a = mid + 1;
        }
        if (a >= L.n) a = L.n - 1;
        const qs_surface* s  = &L.s[a];
        float*            p  = pnts + 3 * i;
        float*            nn = nrms + 3 * i;
        for (int tries = 0;; tries++)
        {
            if (!s->is_sphere)
            {
                const float ua = qs_unit(&rng), ub = qs_unit(&rng);
                for (int c = 0; c < 3; c++)
                {
                    p[c]  = s->origin[c] + ua * s->edge0[c] + ub * s->edge1[c];
                    nn[c] = s->normal[c];
                }
            }
            else
            {
                float x, y, z, q;
                do
                {
                    x = 2.0f * qs_unit(&rng) - 1.0f;
                    y = 2.0f * qs_unit(&rng) - 1.0f;
                    z = 2.0f * qs_unit(&rng) - 1.0f;
                    q = x * x + y * y + z * z;
                } while (!(q > 1.0e-6f && q <= 1.0f));
                const float len = sqrtf(q);
                nn[0]           = x / len;
                nn[1]           = y / len;
                nn[2]           = z / len;
                for (int c = 0; c < 3; c++) p[c] = s->centre[c] + s->radius * nn[c];
            }
            if (p[0] >= 0.0f && p[0] < S && p[1] >= 0.0f && p[1] < S && p[2] >= 0.0f && p[2] < S) break;
            if (tries > 64)
            {
                rc = -2;
                break;
            }
        }
        if (rc) break;
        float* cc = cols + 3 * i;
        for (int c = 0; c < 3; c++)
        {
            float v = s->rgb[c];
            if (noise > 0.0f) v = v + noise * (2.0f * qs_unit(&rng) - 1.0f);
            cc[c] = qs_minf(1.0f, qs_maxf(0.0f, v));
        }
        int32_t oct[32];
        qbo_point_octets(S, levels, p, oct);
        uint64_t k = 0;
        for (int lv = 0; lv < levels; lv++) k = (k << 3) | (uint64_t) oct[lv];
        key[i]  = k;
        perm[i] = (uint32_t) i;
    }
    if (rc == 0) rc = qs_sort(key, perm, (size_t) n, 3 * levels);
    if (rc == 0)
    {
        float* tmp = (float*) malloc((size_t) n * 3 * sizeof(float));
        if (!tmp) rc = -1;
        float* arrays[3] = {pnts, nrms, cols};
        for (int a = 0; a < 3 && rc == 0; a++)
        {
            for (int64_t i = 0; i < n; i++) memcpy(tmp + 3 * i, arrays[a] + 3 * (int64_t) perm[i], 3 * sizeof(float));
            memcpy(arrays[a], tmp, (size_t) n * 3 * sizeof(float));
        }
        free(tmp);
    }
    free(key);
    free(perm);
    free(cum);
    free(L.s);
    return rc;
}

/* octree_insert_point (octree.c:95-147) of n points in order into an empty
 * tree (model indices 0..n-1): the whole producer in one call. Returns the
 * node count, or -1 when cap nodes do not suffice. */
int64_t qbo_build_tree(const float* pnts, int64_t n, float basesize, int levels, int32_t* nodes, int64_t cap)
{
    if (cap < 1) return -1;
    memset(nodes, 0, 12 * sizeof(int32_t));
    int64_t len = 1;
    for (int64_t i = 0; i < n; i++)
        if (qbo_insert_point(nodes, &len, cap, basesize, levels, i, pnts + 3 * i, NULL)) return -1;
    return len;
}
