// Host side of libqbcuda that needs no GPU: error reporting, the per-frame
// uniform derivation of octree_glc_update, the node-array producer of
// src/qubatron/octree.c and the seeded synthetic scenes.
//
// Compiled with -ffp-contract=off: the uniforms feed a bit-exact traversal
// and the scenes must come out the same on every machine.

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "qbcuda.h"
#include "qbc_internal.h"

namespace {
thread_local std::string g_last_error;
}

namespace qbc {

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

// Odd-mantissa bit count of a positive finite float: S = m * 2^e, m odd.
static int odd_mantissa_bits(float s) {
  int e = 0;
  float f = std::frexp(s, &e);  // f in [0.5, 1)
  uint32_t m = (uint32_t)std::ldexp(f, 24);
  if (m == 0) return 0;
  while ((m & 1u) == 0) m >>= 1;
  int b = 0;
  while (m) {
    ++b;
    m >>= 1;
  }
  return b;
}

bool cube_shift_exact(const qbc_view& v) {
  // With basecube (0, S, S, S) every cube coordinate down to maxlevel is
  // k * S / 2^L with 0 <= k <= 2^L; all of them, and so every child shift,
  // are exact when the odd part of S has at most 24 - maxlevel bits.
  float s = v.basecube[3];
  if (!(s > 0.0f) || !std::isfinite(s) || !std::isnormal(s)) return false;
  if (v.basecube[0] != 0.0f || std::signbit(v.basecube[0])) return false;
  if (v.basecube[1] != s || v.basecube[2] != s) return false;
  if (std::ldexp(s, -v.maxlevel) < 1.17549435e-38f) return false;  // stays normal
  return odd_mantissa_bits(s) + v.maxlevel <= 24;
}

}  // namespace qbc

using qbc::fail;

extern "C" const char* qbc_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* qbc_version(void) { return "qbcuda 0.1.0 (sm_103a)"; }

// ---------------------------------------------------------------------------
// Uniform derivation
// ---------------------------------------------------------------------------

namespace {

void rotate_by_quat(const float* q, float* v) {
  // v + 2.0 * cross(q.xyz, cross(q.xyz, v) + q.w * v)  (octree_fsh.c:392-395)
  float c1x = q[1] * v[2] - q[2] * v[1];
  float c1y = q[2] * v[0] - q[0] * v[2];
  float c1z = q[0] * v[1] - q[1] * v[0];
  float ax = c1x + q[3] * v[0];
  float ay = c1y + q[3] * v[1];
  float az = c1z + q[3] * v[2];
  float c2x = q[1] * az - q[2] * ay;
  float c2y = q[2] * ax - q[0] * az;
  float c2z = q[0] * ay - q[1] * ax;
  v[0] = v[0] + 2.0f * c2x;
  v[1] = v[1] + 2.0f * c2y;
  v[2] = v[2] + 2.0f * c2z;
}

void axis_angle_quat(const float* axis, float angle, float* q) {
  // quat_from_axis_angle (octree_fsh.c:381-390)
  float half = angle * 0.5f;
  q[0] = axis[0] * sinf(half);
  q[1] = axis[1] * sinf(half);
  q[2] = axis[2] * sinf(half);
  q[3] = cosf(half);
}

}  // namespace

extern "C" int qbc_view_setup(float width, float height, const float position[3], const float angle[3],
                              float lighta, int quality, int maxlevel, float basesize, int shoot, float focal,
                              qbc_view* out) {
  if (!position || !angle || !out) return fail(QBC_E_ARG, "qbc_view_setup: null pointer");
  if (maxlevel < 0 || maxlevel > QBC_MAX_LEVEL)
    return fail(QBC_E_ARG, "qbc_view_setup: maxlevel %d outside 0..%d", maxlevel, QBC_MAX_LEVEL);
  if (quality < 0 || quality > 255) return fail(QBC_E_ARG, "qbc_view_setup: quality %d is not a uint8", quality);
  qbc_view v;
  std::memset(&v, 0, sizeof(v));

  // octree_glc.c:263-264: GLfloat arrays filled from float/double expressions
  v.basecube[0] = 0.0f;
  v.basecube[1] = basesize;
  v.basecube[2] = basesize;
  v.basecube[3] = basesize;
  float sl = sinf(lighta);
  v.light[0] = 420.0f;
  v.light[1] = (float)((double)200.0f - (double)sl * 20.0);
  v.light[2] = (float)((double)680.0f - (double)sl * 200.0);

  // octree_glc.c:268-270, 288: render size and the integer viewport
  double div = 6.0 - (double)(float)quality / 2.0;
  float ow = (float)((double)width / div);
  float oh = (float)((double)height / div);
  if (!(ow >= 1.0f) || !(oh >= 1.0f) || ow > 65536.0f || oh > 65536.0f)
    return fail(QBC_E_ARG, "qbc_view_setup: render size %gx%g outside 1..65536", ow, oh);
  v.dim[0] = ow;
  v.dim[1] = oh;
  v.width_px = (int32_t)ow;
  v.height_px = (int32_t)oh;
  v.coord_scale[0] = ow / (float)v.width_px;
  v.coord_scale[1] = oh / (float)v.height_px;

  v.camfp[0] = position[0];
  v.camfp[1] = position[1];
  v.camfp[2] = position[2];

  // octree_fsh.c:403: cfp = (dim.x/2, dim.y/2, (dim.x/2)/tan(PI/4))
  const float pi = 3.1415926535897932384626433832795f;
  v.cfp[0] = ow / 2.0f;
  v.cfp[1] = oh / 2.0f;
  v.cfp[2] = focal > 0.0f ? focal : (ow / 2.0f) / tanf(pi / 4.0f);

  // octree_fsh.c:406-408
  const float yaxis[3] = {0.0f, 1.0f, 0.0f};
  axis_angle_quat(yaxis, -angle[0], v.qz);
  float vx[3] = {-1.0f, 0.0f, 0.0f};
  rotate_by_quat(v.qz, vx);
  axis_angle_quat(vx, -angle[1], v.qx);

  // octree_fsh.c:417-418 and :452: acos(c) < 0.02 <=> c > cos(0.02) for
  // c <= 1 (acos falls monotonically and is NaN above 1)
  float cl[3] = {v.light[0] - v.camfp[0], v.light[1] - v.camfp[1], v.light[2] - v.camfp[2]};
  float len = sqrtf(cl[0] * cl[0] + cl[1] * cl[1] + cl[2] * cl[2]);
  v.ncamlight[0] = cl[0] / len;
  v.ncamlight[1] = cl[1] / len;
  v.ncamlight[2] = cl[2] / len;
  double c = std::cos((double)0.02f);
  float cf = (float)c;
  if ((double)cf > c) cf = std::nextafter(cf, -2.0f);
  v.flare_cos = cf;

  v.maxlevel = maxlevel;
  v.shoot = shoot;
  *out = v;
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Node-array producer (octree.c:55-218)
// ---------------------------------------------------------------------------

struct qbc_octree {
  std::vector<int32_t> nodes;  // 12 per node
  int64_t len = 0;
  float basesize = 0.0f;
  int levels = 0;
};

namespace {

// octree.c:100-109
inline int octet_at(const float* p, float size) {
  int octet = (int)(p[0] / size) % 2;
  int yi = (int)(p[1] / size) % 2;
  int zi = (int)(p[2] / size) % 2;
  if (yi == 0) octet += 2;
  if (zi == 0) octet += 4;
  return octet;
}

inline bool point_ok(const float* p) {
  // (int)(x / size) % 2 is only defined for 0 <= x / size < 2^31
  for (int k = 0; k < 3; ++k)
    if (!(p[k] >= 0.0f) || !(p[k] < 1.0e30f)) return false;
  return true;
}

int reserve_nodes(qbc_octree* t, int64_t need) {
  size_t want = (size_t)need * 12;
  if (t->nodes.size() >= want) return QBC_OK;
  size_t cap = std::max(want, t->nodes.size() + t->nodes.size() / 2);
  try {
    t->nodes.resize(cap, 0);
  } catch (const std::bad_alloc&) {
    return fail(QBC_E_NOMEM, "octree: cannot grow to %lld nodes", (long long)need);
  }
  return QBC_OK;
}

inline int append(qbc_octree* t, int64_t parent, int octet, int64_t modind) {
  if (t->len >= INT32_MAX) return fail(QBC_E_NOMEM, "octree: node index overflows int32");
  if (t->len + 1 > (int64_t)(t->nodes.size() / 12)) {
    int rc = reserve_nodes(t, t->len + 1);
    if (rc) return rc;
  }
  int32_t* n = t->nodes.data();
  n[parent * 12 + octet] = (int32_t)t->len;
  std::memset(n + t->len * 12, 0, 12 * sizeof(int32_t));
  n[t->len * 12 + 8] = (int32_t)modind;
  ++t->len;
  return QBC_OK;
}

}  // namespace

extern "C" int qbc_octree_create(float basesize, int levels, qbc_octree** out) {
  if (!out) return fail(QBC_E_ARG, "qbc_octree_create: null out");
  if (levels < 0 || levels > 21) return fail(QBC_E_ARG, "qbc_octree_create: levels %d outside 0..21", levels);
  if (!(basesize > 0.0f) || !std::isfinite(basesize)) return fail(QBC_E_ARG, "qbc_octree_create: bad basesize");
  qbc_octree* t = new (std::nothrow) qbc_octree();
  if (!t) return fail(QBC_E_NOMEM, "qbc_octree_create: out of memory");
  t->basesize = basesize;
  t->levels = levels;
  int rc = reserve_nodes(t, 1024);
  if (rc) {
    delete t;
    return rc;
  }
  t->len = 1;  // root, all zero (octree.c:63-64)
  *out = t;
  return QBC_OK;
}

extern "C" int qbc_octree_free(qbc_octree* t) {
  delete t;
  return QBC_OK;
}

extern "C" int qbc_octree_reset(qbc_octree* t) {
  if (!t) return fail(QBC_E_ARG, "qbc_octree_reset: null tree");
  std::memset(t->nodes.data(), 0, 12 * sizeof(int32_t));
  t->len = 1;
  return QBC_OK;
}

extern "C" int qbc_octree_insert_points(qbc_octree* t, const float* pnts, int64_t n, int64_t first_index) {
  if (!t || (n > 0 && !pnts)) return fail(QBC_E_ARG, "qbc_octree_insert_points: null argument");
  for (int64_t i = 0; i < n; ++i) {
    const float* p = pnts + 3 * i;
    if (!point_ok(p))
      return fail(QBC_E_ARG, "qbc_octree_insert_points: point %lld is negative or not finite", (long long)i);
    float size = t->basesize;
    int64_t index = 0;
    for (int level = 0; level < t->levels; ++level) {
      size /= 2.0f;
      int octet = octet_at(p, size);
      if (t->nodes[index * 12 + octet] == 0) {
        int rc = append(t, index, octet, first_index + i);
        if (rc) return rc;
      }
      index = t->nodes[index * 12 + octet];
    }
  }
  return QBC_OK;
}

extern "C" int qbc_octree_insert_paths(qbc_octree* t, const int32_t* octets, int64_t n, int64_t first_index) {
  if (!t || (n > 0 && !octets)) return fail(QBC_E_ARG, "qbc_octree_insert_paths: null argument");
  for (int64_t i = 0; i < n; ++i) {
    const int32_t* o = octets + (int64_t)t->levels * i;
    int64_t index = 0;
    for (int level = 0; level < t->levels; ++level) {
      int octet = o[level];
      if (octet < 0 || octet > 7)
        return fail(QBC_E_ARG, "qbc_octree_insert_paths: octet %d of path %lld", octet, (long long)i);
      if (t->nodes[index * 12 + octet] == 0) {
        int rc = append(t, index, octet, first_index + i);
        if (rc) return rc;
      }
      index = t->nodes[index * 12 + octet];
    }
  }
  return QBC_OK;
}

extern "C" int qbc_octree_remove_point(qbc_octree* t, const float pnt[3], int32_t* modind, int32_t* octind) {
  if (!t || !pnt || !modind || !octind) return fail(QBC_E_ARG, "qbc_octree_remove_point: null argument");
  if (!point_ok(pnt)) return fail(QBC_E_ARG, "qbc_octree_remove_point: point is negative or not finite");
  float size = t->basesize;
  int32_t index = 0, lindex = 0;
  int loctet = 0;
  int32_t* n = t->nodes.data();
  for (int level = 0; level < t->levels + 1; ++level) {
    size /= 2.0f;
    int octet = octet_at(pnt, size);
    if (level == t->levels) {
      *modind = n[(int64_t)index * 12 + 8];
      *octind = lindex;
      n[(int64_t)lindex * 12 + loctet] = 0;
    }
    lindex = index;
    loctet = octet;
    index = n[(int64_t)index * 12 + octet];
    if (index == 0) return QBC_OK;
  }
  return QBC_OK;
}

extern "C" int qbc_octree_nodes(qbc_octree* t, const int32_t** nodes, int64_t* n_nodes) {
  if (!t || !nodes || !n_nodes) return fail(QBC_E_ARG, "qbc_octree_nodes: null argument");
  *nodes = t->nodes.data();
  *n_nodes = t->len;
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// Seeded synthetic scenes
// ---------------------------------------------------------------------------

namespace {

struct Rng {
  uint64_t s;
  uint64_t next() {  // splitmix64
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  float uf() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }       // [0, 1)
  double ud() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
  float range(float a, float b) { return a + (b - a) * uf(); }
};

// An axis-aligned rectangle o + a*u + b*v (a, b in [0, 1)) or a sphere.
struct Prim {
  int sphere;
  float o[3], u[3], v[3], n[3];
  float c[3], r;
  float col[3];
  double area;
};

void rect(std::vector<Prim>& out, const float o[3], const float u[3], const float v[3], const float n[3],
          const float col[3]) {
  Prim p{};
  p.sphere = 0;
  for (int k = 0; k < 3; ++k) {
    p.o[k] = o[k];
    p.u[k] = u[k];
    p.v[k] = v[k];
    p.n[k] = n[k];
    p.col[k] = col[k];
  }
  double lu = std::sqrt((double)u[0] * u[0] + (double)u[1] * u[1] + (double)u[2] * u[2]);
  double lv = std::sqrt((double)v[0] * v[0] + (double)v[1] * v[1] + (double)v[2] * v[2]);
  p.area = lu * lv;
  out.push_back(p);
}

// Five faces of a box standing on y = y0 (its bottom face is hidden).
void box(std::vector<Prim>& out, float x0, float y0, float z0, float sx, float sy, float sz, const float col[3]) {
  float ux[3] = {sx, 0, 0}, uy[3] = {0, sy, 0}, uz[3] = {0, 0, sz};
  {
    float o[3] = {x0, y0 + sy, z0}, n[3] = {0, 1, 0};
    rect(out, o, ux, uz, n, col);
  }
  {
    float o[3] = {x0, y0, z0 + sz}, n[3] = {0, 0, 1};
    rect(out, o, ux, uy, n, col);
  }
  {
    float o[3] = {x0, y0, z0}, n[3] = {0, 0, -1};
    rect(out, o, ux, uy, n, col);
  }
  {
    float o[3] = {x0, y0, z0}, n[3] = {-1, 0, 0};
    rect(out, o, uy, uz, n, col);
  }
  {
    float o[3] = {x0 + sx, y0, z0}, n[3] = {1, 0, 0};
    rect(out, o, uy, uz, n, col);
  }
}

void sphere(std::vector<Prim>& out, float cx, float cy, float cz, float r, const float col[3]) {
  Prim p{};
  p.sphere = 1;
  p.c[0] = cx;
  p.c[1] = cy;
  p.c[2] = cz;
  p.r = r;
  for (int k = 0; k < 3; ++k) p.col[k] = col[k];
  p.area = 4.0 * 3.14159265358979323846 * (double)r * (double)r;
  out.push_back(p);
}

// LSD radix sort of (key, index) pairs by key, stable, 12 bits per pass.
void radix_sort(std::vector<uint64_t>& key, std::vector<uint32_t>& idx, int key_bits) {
  size_t n = key.size();
  std::vector<uint64_t> k2(n);
  std::vector<uint32_t> i2(n);
  std::vector<size_t> cnt(4096);
  for (int shift = 0; shift < key_bits; shift += 12) {
    std::fill(cnt.begin(), cnt.end(), 0);
    for (size_t i = 0; i < n; ++i) ++cnt[(key[i] >> shift) & 4095];
    size_t sum = 0;
    for (size_t b = 0; b < 4096; ++b) {
      size_t c = cnt[b];
      cnt[b] = sum;
      sum += c;
    }
    for (size_t i = 0; i < n; ++i) {
      size_t d = cnt[(key[i] >> shift) & 4095]++;
      k2[d] = key[i];
      i2[d] = idx[i];
    }
    key.swap(k2);
    idx.swap(i2);
  }
}

}  // namespace

extern "C" int qbc_scene_generate(const qbc_scene_desc* d, float* pnts, float* nrms, float* cols) {
  if (!d || !pnts || !nrms || !cols) return fail(QBC_E_ARG, "qbc_scene_generate: null argument");
  if (d->n_points <= 0 || d->n_points > 0xFFFFFFFFll)
    return fail(QBC_E_ARG, "qbc_scene_generate: n_points %lld outside 1..2^32-1", (long long)d->n_points);
  if (d->levels < 1 || d->levels > 21) return fail(QBC_E_ARG, "qbc_scene_generate: levels outside 1..21");
  const float S = d->basesize;
  if (!(S > 0.0f)) return fail(QBC_E_ARG, "qbc_scene_generate: basesize must be positive");

  Rng rng{d->seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
  std::vector<Prim> prims;
  auto color = [&](float* c) {
    c[0] = rng.uf();
    c[1] = rng.uf();
    c[2] = rng.uf();
  };

  float lo = 0.0f, floor_y = 0.0f, hi_y = S;  // placement bounds for boxes / spheres
  float xlo = 0.0f, xhi = S;
  if (d->kind == QBC_SCENE_FLOOR) {
    floor_y = 0.05f * S;
    float c[3];
    color(c);
    float o[3] = {0.0f, floor_y, 0.0f}, u[3] = {S, 0, 0}, v[3] = {0, 0, S}, n[3] = {0, 1, 0};
    rect(prims, o, u, v, n, c);
  } else if (d->kind == QBC_SCENE_ROOM) {
    float m = 0.02f * S;        // wall inset
    float h = 0.6f * S;         // room height
    float w = S - 2.0f * m;     // room width and depth
    floor_y = m;
    hi_y = m + h;
    xlo = m;
    xhi = S - m;
    float c[3];
    color(c);
    {
      float o[3] = {m, m, m}, u[3] = {w, 0, 0}, v[3] = {0, 0, w}, n[3] = {0, 1, 0};
      rect(prims, o, u, v, n, c);  // floor
    }
    color(c);
    {
      float o[3] = {m, m + h, m}, u[3] = {w, 0, 0}, v[3] = {0, 0, w}, n[3] = {0, -1, 0};
      rect(prims, o, u, v, n, c);  // ceiling
    }
    color(c);
    {
      float o[3] = {m, m, m}, u[3] = {0, h, 0}, v[3] = {0, 0, w}, n[3] = {1, 0, 0};
      rect(prims, o, u, v, n, c);  // left wall
    }
    color(c);
    {
      float o[3] = {S - m, m, m}, u[3] = {0, h, 0}, v[3] = {0, 0, w}, n[3] = {-1, 0, 0};
      rect(prims, o, u, v, n, c);  // right wall
    }
    color(c);
    {
      float o[3] = {m, m, m}, u[3] = {w, 0, 0}, v[3] = {0, h, 0}, n[3] = {0, 0, 1};
      rect(prims, o, u, v, n, c);  // back wall
    }
    color(c);
    {
      float o[3] = {m, m, S - m}, u[3] = {w, 0, 0}, v[3] = {0, h, 0}, n[3] = {0, 0, -1};
      rect(prims, o, u, v, n, c);  // front wall
    }
  } else if (d->kind == QBC_SCENE_HOUSE) {
    // 3 floors of 3 x 2 closed rooms (floor, ceiling, 4 walls each)
    const float m = 0.02f * S, fh = (S - 2.0f * m) / 3.0f, rw = (S - 2.0f * m) / 3.0f, rd = (S - 2.0f * m) / 2.0f;
    for (int f = 0; f < 3; ++f)
      for (int rx = 0; rx < 3; ++rx)
        for (int rz = 0; rz < 2; ++rz) {
          const float x0 = m + rx * rw, y0 = m + f * fh, z0 = m + rz * rd;
          float c[3];
          color(c);
          {
            float o[3] = {x0, y0, z0}, u[3] = {rw, 0, 0}, v[3] = {0, 0, rd}, n[3] = {0, 1, 0};
            rect(prims, o, u, v, n, c);  // floor
          }
          {
            float o[3] = {x0, y0 + fh, z0}, u[3] = {rw, 0, 0}, v[3] = {0, 0, rd}, n[3] = {0, -1, 0};
            rect(prims, o, u, v, n, c);  // ceiling
          }
          color(c);
          {
            float o[3] = {x0, y0, z0}, u[3] = {0, fh, 0}, v[3] = {0, 0, rd}, n[3] = {1, 0, 0};
            rect(prims, o, u, v, n, c);
          }
          {
            float o[3] = {x0 + rw, y0, z0}, u[3] = {0, fh, 0}, v[3] = {0, 0, rd}, n[3] = {-1, 0, 0};
            rect(prims, o, u, v, n, c);
          }
          {
            float o[3] = {x0, y0, z0}, u[3] = {rw, 0, 0}, v[3] = {0, fh, 0}, n[3] = {0, 0, 1};
            rect(prims, o, u, v, n, c);
          }
          {
            float o[3] = {x0, y0, z0 + rd}, u[3] = {rw, 0, 0}, v[3] = {0, fh, 0}, n[3] = {0, 0, -1};
            rect(prims, o, u, v, n, c);
          }
        }
  } else {
    return fail(QBC_E_ARG, "qbc_scene_generate: unknown scene kind %d", d->kind);
  }
  (void)lo;

  // where boxes and spheres go: the single room (floor / room scenes, x and z
  // share bounds), or a seeded room of the house
  auto room_bounds = [&](float* b) {  // x0 x1 y0 y1 z0 z1
    if (d->kind != QBC_SCENE_HOUSE) {
      b[0] = xlo, b[1] = xhi, b[2] = floor_y, b[3] = hi_y, b[4] = xlo, b[5] = xhi;
      return;
    }
    const float m = 0.02f * S, fh = (S - 2.0f * m) / 3.0f, rw = (S - 2.0f * m) / 3.0f, rd = (S - 2.0f * m) / 2.0f;
    const int r = (int)(rng.next() % 18u), f = r / 6, rx = (r / 2) % 3, rz = r % 2;
    b[0] = m + rx * rw, b[1] = b[0] + rw, b[2] = m + f * fh, b[3] = b[2] + fh, b[4] = m + rz * rd, b[5] = b[4] + rd;
  };
  for (int b = 0; b < d->n_boxes; ++b) {
    float rb[6];
    room_bounds(rb);
    float sx = rng.range(d->box_min, d->box_max);
    float sy = rng.range(d->box_min, d->box_max);
    float sz = rng.range(d->box_min, d->box_max);
    sx = std::min(sx, 0.9f * (rb[1] - rb[0]));
    sz = std::min(sz, 0.9f * (rb[5] - rb[4]));
    sy = std::min(sy, 0.9f * (rb[3] - rb[2]));
    float x0 = rng.range(rb[0], rb[1] - sx);
    float z0 = rng.range(rb[4], rb[5] - sz);
    float c[3];
    color(c);
    box(prims, x0, rb[2], z0, sx, sy, sz, c);
  }
  for (int s = 0; s < d->n_spheres; ++s) {
    float rb[6];
    room_bounds(rb);
    float r = rng.range(d->sphere_min, d->sphere_max);
    r = std::min(r, 0.45f * std::min(std::min(rb[1] - rb[0], rb[5] - rb[4]), rb[3] - rb[2]));
    float cx = rng.range(rb[0] + r, rb[1] - r);
    float cy = rng.range(rb[2] + r, rb[3] - r);
    float cz = rng.range(rb[4] + r, rb[5] - r);
    float c[3];
    color(c);
    sphere(prims, cx, cy, cz, r, c);
  }

  std::vector<double> cdf(prims.size());
  double tot = 0.0;
  for (size_t i = 0; i < prims.size(); ++i) {
    tot += prims[i].area;
    cdf[i] = tot;
  }

  const int64_t n = d->n_points;
  const float noise = d->color_noise;
  std::vector<uint64_t> key((size_t)n);
  std::vector<uint32_t> idx((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    double u = rng.ud() * tot;
    size_t k = (size_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
    if (k >= prims.size()) k = prims.size() - 1;
    const Prim& pr = prims[k];
    float* p = pnts + 3 * i;
    float* nn = nrms + 3 * i;
    for (int tries = 0;; ++tries) {
      if (!pr.sphere) {
        float a = rng.uf(), b = rng.uf();
        for (int c = 0; c < 3; ++c) {
          p[c] = pr.o[c] + a * pr.u[c] + b * pr.v[c];
          nn[c] = pr.n[c];
        }
      } else {
        float x, y, z, q;
        do {
          x = 2.0f * rng.uf() - 1.0f;
          y = 2.0f * rng.uf() - 1.0f;
          z = 2.0f * rng.uf() - 1.0f;
          q = x * x + y * y + z * z;
        } while (!(q > 1.0e-6f && q <= 1.0f));
        float l = sqrtf(q);
        nn[0] = x / l;
        nn[1] = y / l;
        nn[2] = z / l;
        for (int c = 0; c < 3; ++c) p[c] = pr.c[c] + pr.r * nn[c];
      }
      if (p[0] >= 0.0f && p[0] < S && p[1] >= 0.0f && p[1] < S && p[2] >= 0.0f && p[2] < S) break;
      if (tries > 64) return fail(QBC_E_STATE, "qbc_scene_generate: primitive %zu lies outside the cube", k);
    }
    float* cc = cols + 3 * i;
    for (int c = 0; c < 3; ++c) {
      float v = pr.col[c];
      if (noise > 0.0f) v = v + noise * (2.0f * rng.uf() - 1.0f);
      cc[c] = std::min(1.0f, std::max(0.0f, v));
    }
    // octree path key: octets of octree.c:100-109, root level most significant
    uint64_t kk = 0;
    float size = S;
    for (int level = 0; level < d->levels; ++level) {
      size /= 2.0f;
      kk = (kk << 3) | (uint64_t)octet_at(p, size);
    }
    key[(size_t)i] = kk;
    idx[(size_t)i] = (uint32_t)i;
  }

  radix_sort(key, idx, 3 * d->levels);

  std::vector<float> tmp((size_t)n * 3);
  float* arrs[3] = {pnts, nrms, cols};
  for (float* a : arrs) {
    for (int64_t i = 0; i < n; ++i) {
      const float* s = a + 3 * (int64_t)idx[(size_t)i];
      tmp[(size_t)(3 * i)] = s[0];
      tmp[(size_t)(3 * i + 1)] = s[1];
      tmp[(size_t)(3 * i + 2)] = s[2];
    }
    std::memcpy(a, tmp.data(), sizeof(float) * 3 * (size_t)n);
  }
  return QBC_OK;
}

// ---------------------------------------------------------------------------
// qmc flat model files (model_load_flat, src/qubatron/model.c:53-111; the
// writer is qmc.c:275-327): .pnt / .nrm / .col float3 per point, .rng int
// triples (first point index of a column, x index, y index)
// ---------------------------------------------------------------------------

namespace {

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

int open_sized(const char* path, File& file, int64_t* bytes) {
  file.f = std::fopen(path, "rb");
  if (!file.f) return fail(QBC_E_IO, "qmc flat file: cannot open %s", path);
  if (std::fseek(file.f, 0, SEEK_END) != 0) return fail(QBC_E_IO, "qmc flat file: cannot seek %s", path);
  const long end = std::ftell(file.f);
  if (end < 0 || std::fseek(file.f, 0, SEEK_SET) != 0) return fail(QBC_E_IO, "qmc flat file: cannot size %s", path);
  *bytes = end;
  return QBC_OK;
}

// Read up to `want` bytes into dst; the rest of `want` stays zero (a file
// shorter than the point file).
int read_into(File& file, const char* path, void* dst, int64_t want, int64_t have) {
  const int64_t n = std::min(want, have);
  if (n > 0 && std::fread(dst, 1, (size_t)n, file.f) != (size_t)n)
    return fail(QBC_E_IO, "qmc flat file: short read of %s", path);
  if (want > n) std::memset(static_cast<char*>(dst) + n, 0, (size_t)(want - n));
  return QBC_OK;
}

}  // namespace

extern "C" int qbc_flat_read(const char* pnt_path, const char* col_path, const char* nrm_path, const char* rng_path,
                             float* pnts, float* cols, float* nrms, int64_t point_cap, int64_t* points,
                             int32_t* ranges, int64_t range_cap, int64_t* range_ints) {
  qbc::clear_error();
  if (!pnt_path || !col_path || !nrm_path || !points) return fail(QBC_E_ARG, "qbc_flat_read: null path or count");
  File fp, fc, fn, fr;
  int64_t bp = 0, bc = 0, bn = 0, br = 0;
  int rc = open_sized(pnt_path, fp, &bp);
  if (!rc) rc = open_sized(col_path, fc, &bc);
  if (!rc) rc = open_sized(nrm_path, fn, &bn);
  if (!rc && rng_path) rc = open_sized(rng_path, fr, &br);
  if (rc) return rc;
  // the point count is the .pnt size in whole float3 (model.c:59-63)
  const int64_t n = bp / 12;
  const int64_t nr = rng_path ? br / 4 : 0;
  *points = n;
  if (range_ints) *range_ints = nr;
  if (pnts || cols || nrms) {
    if (!pnts || !cols || !nrms) return fail(QBC_E_ARG, "qbc_flat_read: give all three point arrays or none");
    if (point_cap < n) return fail(QBC_E_ARG, "qbc_flat_read: %lld points, capacity %lld", (long long)n, (long long)point_cap);
    if ((rc = read_into(fp, pnt_path, pnts, n * 12, bp))) return rc;
    if ((rc = read_into(fc, col_path, cols, n * 12, bc))) return rc;
    if ((rc = read_into(fn, nrm_path, nrms, n * 12, bn))) return rc;
  }
  if (ranges && rng_path) {
    if (range_cap < nr) return fail(QBC_E_ARG, "qbc_flat_read: %lld range ints, capacity %lld", (long long)nr, (long long)range_cap);
    if ((rc = read_into(fr, rng_path, ranges, nr * 4, br))) return rc;
  }
  return QBC_OK;
}
