// Particle path tracer on the GPU: the offline renderer of
// taichi-dev/taichi_elements (engine/renderer.py, engine/renderer_utils.py)
// as CUDA kernels, with no graphics API.
//
//  * Cell lists (renderer.py:482-517): every particle is listed in each grid
//    cell of size dx inside the bounding box that its sphere touches during
//    the shutter interval (a ternary search of the point-box distance along
//    the motion, renderer_utils.py:133-147).  Count pass, scan, fill pass.
//  * Rendering (renderer.py:396-480): one thread per pixel and sample; a
//    camera ray with pixel jitter and a shutter time; up to 4 bounces, each
//    hit the nearest of a particle sphere (DDA over the cells, :297-366), the
//    z = -5.5 plane (:375-380) and the floor y = floor_height reached by
//    sphere tracing (:180-191); diffuse bounce (cosine-weighted, out_dir), a
//    shadow ray to a jittered directional light, Russian roulette.
//    Samples accumulate into a float32 colour buffer.
//  * Tone mapping (renderer.py:519-531): vignette, exposure, square root.
// Random numbers come from a counter-based hash (splitmix64 of the seed, the
// pixel, the sample and a draw counter), so a seed renders the same image;
// they are not Taichi's ti.random stream, so images match the reference in
// distribution, not pixel for pixel.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_common.cuh"

namespace mpm {

constexpr float kInf = 1e10f;     // renderer_utils.py:4
constexpr float kEps = 1e-4f;     // renderer_utils.py:3
constexpr float kDistLimit = 100.0f;
constexpr int kMaxRayDepth = 4;
constexpr int kRenderThreads = 128;

struct RenderScene {
  // cell grid: cells [c0, c0 + nc) per axis, size dx; bbox in world units
  int c0[3], nc[3];
  float dx, inv_dx, radius;
  float bbox_min[3], bbox_max[3];
  float shutter_begin, shutter_time;
  int motion_blur;
  // camera
  float cam[3], look_at[3], up[3], fov;
  int res[2];
  float floor_height;
  int taichi_logo;
  float light_dir[3], light_noise, light_color[3];
  int render_voxel;  // the voxel view: cells holding particles drawn as cubes
  int pad_;
  uint64_t seed;
};

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ void set_comp(V3 &a, int i, float v) {
  if (i == 0) a.x = v;
  else if (i == 1) a.y = v;
  else a.z = v;
}
// Matrix.normalized(eps = 0): v / |v|
__device__ __forceinline__ V3 normalized(V3 a) { return (1.0f / sqrtf(dot(a, a))) * a; }

__device__ __forceinline__ uint64_t splitmix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s;
  __device__ __forceinline__ float next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)(z >> 40) * (1.0f / 16777216.0f);
  }
};

// ---------------------------------------------------------------- cells --

// squared distance of o to the box (renderer_utils.py:123-128)
__device__ __forceinline__ float point_aabb_distance2(V3 bmin, V3 bmax, V3 o) {
  const V3 p = v3(fmaxf(fminf(o.x, bmax.x), bmin.x), fmaxf(fminf(o.y, bmax.y), bmin.y),
                  fmaxf(fminf(o.z, bmax.z), bmin.z));
  const V3 d = p - o;
  return dot(d, d);
}

// renderer_utils.py:133-147: ternary search of the closest approach of the
// segment o1 -> o2 to the box
__device__ __forceinline__ bool sphere_aabb_intersect_motion(V3 bmin, V3 bmax, V3 o1, V3 o2, float r) {
  float lo = 0.0f, hi = 1.0f;
  for (int it = 0; it < 64 && lo + 1e-5f < hi; ++it) {
    const float m1 = 2.0f * lo / 3.0f + hi / 3.0f;
    const float m2 = lo / 3.0f + 2.0f * hi / 3.0f;
    const float d1 = point_aabb_distance2(bmin, bmax, (1.0f - m1) * o1 + m1 * o2);
    const float d2 = point_aabb_distance2(bmin, bmax, (1.0f - m2) * o1 + m2 * o2);
    if (d2 > d1) hi = m2;
    else lo = m1;
  }
  return point_aabb_distance2(bmin, bmax, (1.0f - lo) * o1 + lo * o2) < r * r;
}

__device__ __forceinline__ bool inside_particle_grid(const RenderScene &S, int i, int j, int k) {
  const float px = (float)i * S.dx, py = (float)j * S.dx, pz = (float)k * S.dx;  // renderer.py:289-294
  return S.bbox_min[0] <= px && px < S.bbox_max[0] && S.bbox_min[1] <= py && py < S.bbox_max[1] &&
         S.bbox_min[2] <= pz && pz < S.bbox_max[2];
}

__device__ __forceinline__ int64_t cell_index(const RenderScene &S, int i, int j, int k) {
  const int a = i - S.c0[0], b = j - S.c0[1], c = k - S.c0[2];
  if ((unsigned)a >= (unsigned)S.nc[0] || (unsigned)b >= (unsigned)S.nc[1] || (unsigned)c >= (unsigned)S.nc[2])
    return -1;
  return ((int64_t)a * S.nc[1] + b) * S.nc[2] + c;
}

// Visit the cells particle p is listed in (renderer.py:482-517).
template <typename Visit>
__device__ __forceinline__ void particle_cells(const RenderScene &S, V3 x, V3 v, Visit visit) {
  const int ipos[3] = {(int)floorf(x.x * S.inv_dx), (int)floorf(x.y * S.inv_dx), (int)floorf(x.z * S.inv_dx)};
  const float sb = S.motion_blur ? S.shutter_begin * S.shutter_time : 0.0f;
  const float se = S.motion_blur ? (S.shutter_begin + 1.0f) * S.shutter_time : 0.0f;
  const V3 ob = sb * v, oe = se * v;
  int lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float a = comp(ob, d), b = comp(oe, d);
    if (b < a) {
      const float t = b;
      b = a;
      a = t;
    }
    lo[d] = (int)floorf(a * S.inv_dx) - 1;
    hi[d] = (int)ceilf(b * S.inv_dx) + 2;
  }
  const V3 o1 = x + ob, o2 = x + oe;
  for (int i = lo[0]; i < hi[0]; ++i)
    for (int j = lo[1]; j < hi[1]; ++j)
      for (int k = lo[2]; k < hi[2]; ++k) {
        const int bi = ipos[0] + i, bj = ipos[1] + j, bk = ipos[2] + k;
        if (!inside_particle_grid(S, bi, bj, bk)) continue;
        const V3 bmin = v3((float)bi * S.dx, (float)bj * S.dx, (float)bk * S.dx);
        const V3 bmax = v3((float)(bi + 1) * S.dx, (float)(bj + 1) * S.dx, (float)(bk + 1) * S.dx);
        if (sphere_aabb_intersect_motion(bmin, bmax, o1, o2, S.radius)) {
          const int64_t c = cell_index(S, bi, bj, bk);
          if (c >= 0) visit(c);
        }
      }
}

__global__ __launch_bounds__(256) void k_cell_count(RenderScene S, const float *__restrict__ x,
                                                    const float *__restrict__ v, int64_t n,
                                                    int32_t *__restrict__ count) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const V3 xp = v3(x[3 * p], x[3 * p + 1], x[3 * p + 2]);
  const V3 vp = v ? v3(v[3 * p], v[3 * p + 1], v[3 * p + 2]) : v3(0.f, 0.f, 0.f);
  particle_cells(S, xp, vp, [&](int64_t c) { atomicAdd(&count[c], 1); });
}

__global__ __launch_bounds__(256) void k_cell_fill(RenderScene S, const float *__restrict__ x,
                                                   const float *__restrict__ v, int64_t n,
                                                   const int64_t *__restrict__ start, int32_t *__restrict__ fill,
                                                   int64_t list_len, int32_t *__restrict__ list) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const V3 xp = v3(x[3 * p], x[3 * p + 1], x[3 * p + 2]);
  const V3 vp = v ? v3(v[3 * p], v[3 * p + 1], v[3 * p + 2]) : v3(0.f, 0.f, 0.f);
  particle_cells(S, xp, vp, [&](int64_t c) {
    const int64_t at = start[c] + atomicAdd(&fill[c], 1);
    if (at < list_len) list[at] = (int32_t)p;
  });
}

// ------------------------------------------------------------- tracing --

struct Hit {
  float dist;
  V3 normal, color;
};

struct Cells {
  const uint32_t *occ;  // one bit per cell: the cell lists a particle (fits in L2)
  const int64_t *start;
  const int32_t *count;
  const int32_t *list;
  const float *x, *v;
  const uint8_t *rgb;
};

// renderer_utils.py:52-76
__device__ __forceinline__ bool ray_aabb_intersection(V3 bmin, V3 bmax, V3 o, V3 d, float &near_int,
                                                      float &far_int) {
  bool intersect = true;
  near_int = -kInf;
  far_int = kInf;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float di = comp(d, i), oi = comp(o, i), lo = comp(bmin, i), hi = comp(bmax, i);
    if (di == 0.0f) {
      if (oi < lo || oi > hi) intersect = false;
    } else {
      const float i1 = (lo - oi) / di, i2 = (hi - oi) / di;
      far_int = fminf(fmaxf(i1, i2), far_int);
      near_int = fmaxf(fminf(i1, i2), near_int);
    }
  }
  if (near_int > far_int) intersect = false;
  return intersect;
}

// renderer_utils.py:84-112: project to the closest approach first, then
// solve the quadratic there (kept as written, including a miss behind the
// origin returning the projection distance)
__device__ __forceinline__ float intersect_sphere(V3 pos, V3 d, V3 center, float radius) {
  V3 T = pos - center;
  float B = 2.0f * dot(T, d);
  const float old_dist = 0.5f * (-B);
  float dist = old_dist;
  const V3 np = pos + old_dist * d;
  T = np - center;
  B = 2.0f * dot(T, d);
  const float C = dot(T, T) - radius * radius;
  const float delta = B * B - 4.0f * C;
  if (delta > 0.0f) {
    const float ret1 = 0.5f * (-B - sqrtf(delta)) + old_dist;
    if (ret1 > 0.0f) dist = ret1;
  } else {
    dist = kInf;
  }
  return dist;
}

// renderer.py:297-366
__device__ Hit dda_particle(const RenderScene &S, const Cells &G, V3 eye, V3 d, float t) {
  Hit h{kInf, v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (fabsf(comp(d, i)) < 1e-6f) set_comp(d, i, 1e-6f);
  const V3 bmin = v3(S.bbox_min[0], S.bbox_min[1], S.bbox_min[2]);
  const V3 bmax = v3(S.bbox_max[0], S.bbox_max[1], S.bbox_max[2]);
  float near_int, far_int;
  const bool inter = ray_aabb_intersection(bmin, bmax, eye, d, near_int, far_int);
  near_int = fmaxf(0.0f, near_int);
  if (!inter) return h;
  const V3 pos = eye + (near_int + kEps) * d;
  const V3 rinv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  const int rs[3] = {d.x > 0.0f ? 1 : -1, d.y > 0.0f ? 1 : -1, d.z > 0.0f ? 1 : -1};
  const V3 o = S.inv_dx * pos;
  int ip[3] = {(int)floorf(o.x), (int)floorf(o.y), (int)floorf(o.z)};
  float dis[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) dis[i] = ((float)ip[i] - comp(o, i) + 0.5f + (float)rs[i] * 0.5f) * comp(rinv, i);
  // the walk leaves the bounding box after at most the sum of its extents
  const int max_steps = S.nc[0] + S.nc[1] + S.nc[2] + 8;
  for (int step = 0; step < max_steps; ++step) {
    if (!inside_particle_grid(S, ip[0], ip[1], ip[2])) {
      h.normal = v3(0.f, 0.f, 0.f);
      break;
    }
    const int64_t c = cell_index(S, ip[0], ip[1], ip[2]);
    if (c >= 0 && ((G.occ[c >> 5] >> (c & 31)) & 1u)) {
      const int64_t s0 = G.start[c];
      const int cnt = G.count[c];
      for (int q = 0; q < cnt; ++q) {
        const int p = G.list[s0 + q];
        V3 xp = v3(G.x[3 * p], G.x[3 * p + 1], G.x[3 * p + 2]);
        if (S.motion_blur && G.v) xp = xp + t * v3(G.v[3 * p], G.v[3 * p + 1], G.v[3 * p + 2]);
        const float dist = intersect_sphere(eye, d, xp, S.radius);
        if (dist < h.dist && dist > 0.0f) {
          h.dist = dist;
          h.normal = normalized((eye + dist * d) - xp);
          h.color = (1.0f / 255.0f) * v3((float)G.rgb[3 * p], (float)G.rgb[3 * p + 1], (float)G.rgb[3 * p + 2]);
        }
      }
    }
    if (h.dist < kInf) break;
    int m;
    if (dis[0] <= dis[1] && dis[0] <= dis[2]) m = 0;
    else if (dis[1] <= dis[0] && dis[1] <= dis[2]) m = 1;
    else m = 2;
    dis[m] += (float)rs[m] * comp(rinv, m);
    ip[m] += rs[m];
  }
  return h;
}

// renderer.py:146-160: cube edges drawn darker
__device__ __forceinline__ V3 voxel_color(const RenderScene &S, V3 pos) {
  V3 p = S.inv_dx * pos;
  p = v3(p.x - floorf(p.x), p.y - floorf(p.y), p.z - floorf(p.z));
  const float b = 0.1f;  // voxel_edges
  int count = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (comp(p, i) < b || comp(p, i) > 1.0f - b) ++count;
  const float f = count >= 2 ? 1.0f : 0.0f;
  return (1.3f - 1.2f * f) * v3(0.9f, 0.8f, 1.0f);
}

// renderer.py:217-281 (render_voxel = True): DDA to the first cell holding a
// particle; the normal is that of the last face crossed (zero when the first
// cell sampled is already occupied, as in the reference)
__device__ Hit dda_voxel(const RenderScene &S, const Cells &G, V3 eye, V3 d) {
  Hit h{kInf, v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
#pragma unroll
  for (int i = 0; i < 3; ++i)
    if (fabsf(comp(d, i)) < 1e-6f) set_comp(d, i, 1e-6f);
  const V3 rinv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  const int rs[3] = {d.x > 0.0f ? 1 : -1, d.y > 0.0f ? 1 : -1, d.z > 0.0f ? 1 : -1};
  const V3 bmin = v3(S.bbox_min[0], S.bbox_min[1], S.bbox_min[2]);
  const V3 bmax = v3(S.bbox_max[0], S.bbox_max[1], S.bbox_max[2]);
  float near_int, far_int;
  if (!ray_aabb_intersection(bmin, bmax, eye, d, near_int, far_int)) return h;
  near_int = fmaxf(0.0f, near_int);
  const V3 pos = eye + (near_int + 5.0f * kEps) * d;
  const V3 o = S.inv_dx * pos;
  int ip[3] = {(int)floorf(o.x), (int)floorf(o.y), (int)floorf(o.z)};
  float dis[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) dis[i] = ((float)ip[i] - comp(o, i) + 0.5f + (float)rs[i] * 0.5f) * comp(rinv, i);
  const int max_steps = S.nc[0] + S.nc[1] + S.nc[2] + 8;
  for (int step = 0; step < max_steps; ++step) {
    const int64_t c = cell_index(S, ip[0], ip[1], ip[2]);
    const bool occupied = c >= 0 && ((G.occ[c >> 5] >> (c & 31)) & 1u);
    const bool inside = inside_particle_grid(S, ip[0], ip[1], ip[2]);
    if (occupied) {
      float mini = -kInf;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        mini = fmaxf(mini, ((float)ip[i] - comp(o, i) + 0.5f - (float)rs[i] * 0.5f) * comp(rinv, i));
      h.dist = mini * S.dx + near_int;
      h.color = voxel_color(S, eye + h.dist * d);
      break;
    }
    int m;
    if (dis[0] <= dis[1] && dis[0] < dis[2]) m = 0;
    else if (dis[1] <= dis[0] && dis[1] <= dis[2]) m = 1;
    else m = 2;
    dis[m] += (float)rs[m] * comp(rinv, m);
    ip[m] += rs[m];
    h.normal = v3(m == 0 ? -(float)rs[0] : 0.f, m == 1 ? -(float)rs[1] : 0.f, m == 2 ? -(float)rs[2] : 0.f);
    if (!inside) break;  // the reference steps once more before it stops
  }
  return h;
}

// floor supporter (renderer.py:162-178 with supporter = 2)
__device__ __forceinline__ float sdf(const RenderScene &S, V3 o) { return o.y - S.floor_height; }

// renderer.py:180-191 (at most 200 steps)
__device__ __forceinline__ float ray_march(const RenderScene &S, V3 p, V3 d) {
  int j = 0;
  float dist = 0.0f;
  while (j < 200 && sdf(S, p + dist * d) > 1e-8f && dist < kDistLimit) {
    dist += sdf(S, p + dist * d);
    ++j;
  }
  if (dist > kDistLimit) dist = kInf;
  return dist;
}

// renderer.py:193-203
__device__ __forceinline__ V3 sdf_normal(const RenderScene &S, V3 p) {
  const float h = 1e-3f;
  V3 n = v3(0.f, 0.f, 0.f);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    V3 inc = p, dec = p;
    set_comp(inc, i, comp(p, i) + h);
    set_comp(dec, i, comp(p, i) - h);
    set_comp(n, i, (0.5f / h) * (sdf(S, inc) - sdf(S, dec)));
  }
  return normalized(n);
}

__device__ __forceinline__ bool in_disc(float px, float py, float cx, float cy, float r) {
  return (px - cx) * (px - cx) + (py - cy) * (py - cy) <= r * r;
}

// renderer_utils.py:164-195
__device__ __forceinline__ int inside_taichi(float px, float py) {
  int ret = -1;
  if (!in_disc(px, py, 0.50f, 0.50f, 0.52f) && ret == -1) ret = 0;
  if (!in_disc(px, py, 0.50f, 0.50f, 0.495f) && ret == -1) ret = 1;
  if (in_disc(px, py, 0.50f, 0.25f, 0.08f) && ret == -1) ret = 1;
  if (in_disc(px, py, 0.50f, 0.75f, 0.08f) && ret == -1) ret = 0;
  if (in_disc(px, py, 0.50f, 0.25f, 0.25f) && ret == -1) ret = 0;
  if (in_disc(px, py, 0.50f, 0.75f, 0.25f) && ret == -1) ret = 1;
  if (ret == -1) ret = px < 0.5f ? 1 : 0;
  return ret;
}

// renderer.py:205-214
__device__ __forceinline__ V3 sdf_color(const RenderScene &S, V3 p) {
  float scale = 1.0f;
  if (S.taichi_logo) scale = inside_taichi(p.x, p.z) ? 1.0f : 0.4f;
  return scale * v3(0.3f, 0.5f, 0.7f);
}

// renderer.py:368-386
__device__ Hit next_hit(const RenderScene &S, const Cells &G, V3 pos, V3 d, float t) {
  Hit h = S.render_voxel ? dda_voxel(S, G, pos, d) : dda_particle(S, G, pos, d, t);
  if (d.z != 0.0f) {
    const float rc = -(pos.z + 5.5f) / d.z;
    if (rc > 0.0f && rc < h.dist) {
      h.dist = rc;
      h.normal = v3(0.f, 0.f, 1.f);
      h.color = v3(0.6f, 0.7f, 0.7f);
    }
  }
  const float rm = ray_march(S, pos, d);
  if (rm < kDistLimit && rm < h.dist) {
    h.dist = rm;
    h.normal = sdf_normal(S, pos + rm * d);
    h.color = sdf_color(S, pos + rm * d);
  }
  return h;
}

// renderer_utils.py:8-19: cosine-weighted direction around n
__device__ __forceinline__ V3 out_dir(V3 n, Rng &rng) {
  V3 u = v3(1.f, 0.f, 0.f);
  if (fabsf(n.y) < 1.0f - 1e-3f) u = normalized(cross(n, v3(0.f, 1.f, 0.f)));
  const V3 v = cross(n, u);
  const float phi = 2.0f * 3.14159265358979f * rng.next();
  const float r = rng.next();
  const float ay = sqrtf(r), ax = sqrtf(1.0f - r);
  float sp, cp;
  sincosf(phi, &sp, &cp);
  return ax * (cp * u + sp * v) + ay * n;
}

// renderer.py:396-480: `spp` samples of every pixel added to color_buffer
// (res[0] x res[1] x 3, pixel (u, v) at (u * res[1] + v) * 3)
__global__ __launch_bounds__(kRenderThreads) void k_render(RenderScene S, Cells G, int sample0, int spp,
                                                           float *__restrict__ color_buffer) {
  const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= (int64_t)S.res[0] * S.res[1]) return;
  const int u = (int)(pix / S.res[1]), vv = (int)(pix % S.res[1]);
  const float aspect = (float)S.res[0] / (float)S.res[1];
  V3 acc = v3(0.f, 0.f, 0.f);
  for (int sidx = sample0; sidx < sample0 + spp; ++sidx) {
    Rng rng{splitmix(splitmix(S.seed) + (uint64_t)pix * 0x100000001B3ull + (uint64_t)sidx * 0x9E3779B97F4A7C15ull)};
    V3 pos = v3(S.cam[0], S.cam[1], S.cam[2]);
    V3 d = normalized(v3(S.look_at[0], S.look_at[1], S.look_at[2]) - pos);
    const float fu = 2.0f * S.fov * ((float)u + rng.next()) / (float)S.res[1] - S.fov * aspect - 1e-5f;
    const float fv = 2.0f * S.fov * ((float)vv + rng.next()) / (float)S.res[1] - S.fov - 1e-5f;
    const V3 du = normalized(cross(d, v3(S.up[0], S.up[1], S.up[2])));
    const V3 dv = normalized(cross(du, d));
    d = normalized(d + fu * du + fv * dv);
    const float t = (rng.next() + S.shutter_begin) * S.shutter_time;
    V3 contrib = v3(0.f, 0.f, 0.f), thr = v3(1.f, 1.f, 1.f);
    int depth = 0;
    while (depth < kMaxRayDepth) {
      const Hit h = next_hit(S, G, pos, d, t);
      const V3 hit_pos = pos + h.dist * d;
      ++depth;
      if (dot(h.normal, h.normal) != 0.0f) {
        d = out_dir(h.normal, rng);
        pos = hit_pos + 1e-4f * d;
        thr = mul(thr, h.color);
        const V3 noise = S.light_noise * v3(rng.next() - 0.5f, rng.next() - 0.5f, rng.next() - 0.5f);
        const V3 direct = normalized(v3(S.light_dir[0], S.light_dir[1], S.light_dir[2]) + noise);
        const float dt = dot(direct, h.normal);
        if (dt > 0.0f) {
          const Hit sh = next_hit(S, G, pos, direct, t);
          if (sh.dist > kDistLimit)
            contrib = contrib + dt * mul(thr, v3(S.light_color[0], S.light_color[1], S.light_color[2]));
        }
      } else {
        depth = kMaxRayDepth;  // sky
      }
      const float max_c = fmaxf(thr.x, fmaxf(thr.y, thr.z));
      if (rng.next() > max_c) {
        depth = kMaxRayDepth;
        thr = v3(0.f, 0.f, 0.f);
      } else {
        thr = (1.0f / max_c) * thr;
      }
    }
    acc = acc + contrib;
  }
  color_buffer[pix * 3 + 0] += acc.x;
  color_buffer[pix * 3 + 1] += acc.y;
  color_buffer[pix * 3 + 2] += acc.z;
}

// occupancy bits of the cell counts
__global__ void k_occupancy(const int32_t *__restrict__ count, int64_t ncells, uint32_t *__restrict__ occ) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool on = c < ncells && count[c] > 0;
  const unsigned bits = __ballot_sync(0xffffffffu, on);
  if ((threadIdx.x & 31) == 0 && c < ncells) occ[c >> 5] = bits;
}

// renderer.py:519-531
__global__ void k_tonemap(int rx, int ry, const float *__restrict__ color_buffer, float vignette_strength,
                          float vignette_radius, float vcx, float vcy, float exposure, int samples,
                          float *__restrict__ img) {
  const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= (int64_t)rx * ry) return;
  const int i = (int)(pix / ry), j = (int)(pix % ry);
  const float u = 1.0f * (float)i / (float)rx, v = 1.0f * (float)j / (float)ry;
  const float darken =
      1.0f - vignette_strength * fmaxf(sqrtf((u - vcx) * (u - vcx) + (v - vcy) * (v - vcy)) - vignette_radius, 0.0f);
#pragma unroll
  for (int c = 0; c < 3; ++c) img[pix * 3 + c] = sqrtf(color_buffer[pix * 3 + c] * darken * exposure / (float)samples);
}

// First hits of given rays (no randomness): distance, normal, colour.
__global__ void k_first_hits(RenderScene S, Cells G, const float *__restrict__ orig, const float *__restrict__ dir,
                             int64_t nrays, float t, float *__restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrays) return;
  const Hit h = next_hit(S, G, v3(orig[3 * r], orig[3 * r + 1], orig[3 * r + 2]),
                         v3(dir[3 * r], dir[3 * r + 1], dir[3 * r + 2]), t);
  out[r * 7 + 0] = h.dist;
  out[r * 7 + 1] = h.normal.x;
  out[r * 7 + 2] = h.normal.y;
  out[r * 7 + 3] = h.normal.z;
  out[r * 7 + 4] = h.color.x;
  out[r * 7 + 5] = h.color.y;
  out[r * 7 + 6] = h.color.z;
}

}  // namespace mpm

using namespace mpm;

extern "C" {

static bool scene_ok(const RenderScene *S) {
  return S && S->dx > 0.0f && S->nc[0] > 0 && S->nc[1] > 0 && S->nc[2] > 0 && S->res[0] > 0 && S->res[1] > 0 &&
         (int64_t)S->nc[0] * S->nc[1] * S->nc[2] < ((int64_t)1 << 34);
}

int mpm_render_cell_count(const void *scene, const float *x, const float *v, int64_t n, int32_t *count,
                          void *stream) {
  const RenderScene *S = (const RenderScene *)scene;
  if (!scene_ok(S) || !x || !count || n < 0) return MPM_E_INVALID;
  if (n == 0) return MPM_OK;
  k_cell_count<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*S, x, v, n, count);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_render_cell_fill(const void *scene, const float *x, const float *v, int64_t n, const int64_t *start,
                         int32_t *fill, int64_t list_len, int32_t *list, void *stream) {
  const RenderScene *S = (const RenderScene *)scene;
  if (!scene_ok(S) || !x || !start || !fill || !list || n < 0 || list_len < 0) return MPM_E_INVALID;
  if (n == 0) return MPM_OK;
  k_cell_fill<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*S, x, v, n, start, fill, list_len,
                                                                          list);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_render_occupancy(const int32_t *count, int64_t ncells, uint32_t *occ, void *stream) {
  if (!count || !occ || ncells < 0) return MPM_E_INVALID;
  if (ncells == 0) return MPM_OK;
  k_occupancy<<<(unsigned)((ncells + 255) / 256), 256, 0, (cudaStream_t)stream>>>(count, ncells, occ);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_render_samples(const void *scene, const uint32_t *occ, const int64_t *start, const int32_t *count,
                       const int32_t *list, const float *x, const float *v, const uint8_t *rgb, int32_t sample0,
                       int32_t spp, float *color_buffer, void *stream) {
  const RenderScene *S = (const RenderScene *)scene;
  if (!scene_ok(S) || !occ || !start || !count || !list || !x || !rgb || !color_buffer || spp < 0)
    return MPM_E_INVALID;
  if (spp == 0) return MPM_OK;
  const int64_t npix = (int64_t)S->res[0] * S->res[1];
  Cells G{occ, start, count, list, x, v, rgb};
  k_render<<<(unsigned)((npix + kRenderThreads - 1) / kRenderThreads), kRenderThreads, 0, (cudaStream_t)stream>>>(
      *S, G, sample0, spp, color_buffer);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_render_tonemap(int32_t rx, int32_t ry, const float *color_buffer, float vignette_strength,
                       float vignette_radius, float vcx, float vcy, float exposure, int32_t samples, float *img,
                       void *stream) {
  if (rx <= 0 || ry <= 0 || !color_buffer || !img || samples <= 0) return MPM_E_INVALID;
  const int64_t npix = (int64_t)rx * ry;
  k_tonemap<<<(unsigned)((npix + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      rx, ry, color_buffer, vignette_strength, vignette_radius, vcx, vcy, exposure, samples, img);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_render_first_hits(const void *scene, const uint32_t *occ, const int64_t *start, const int32_t *count,
                          const int32_t *list, const float *x, const float *v, const uint8_t *rgb, const float *orig,
                          const float *dir, int64_t nrays, float t, float *out, void *stream) {
  const RenderScene *S = (const RenderScene *)scene;
  if (!scene_ok(S) || !occ || !start || !count || !list || !x || !rgb || !orig || !dir || !out || nrays < 0)
    return MPM_E_INVALID;
  if (nrays == 0) return MPM_OK;
  Cells G{occ, start, count, list, x, v, rgb};
  k_first_hits<<<(unsigned)((nrays + 127) / 128), 128, 0, (cudaStream_t)stream>>>(*S, G, orig, dir, nrays, t, out);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_render_scene_bytes(void) { return (int)sizeof(RenderScene); }

}  // extern "C"
