// Mesh voxelizer and voxel seeding on the GPU: the add_mesh emitter of
// taichi-dev/taichi_elements (engine/voxelizer.py:46-126,
// engine/mpm_solver.py:1017-1079).
//
// Voxelization is a parity count along z: every triangle whose xy
// projection covers the centre of voxel column (p, q) adds +1 (normal.z > 0)
// or -1 to the voxels [padding, height) of that column, height being where
// the triangle's plane crosses the column (voxelizer.py:86-126).  Voxels
// inside a closed mesh end with a positive count.  The GPU form adds +-1 at
// the two ends of each column range in a difference array (atomics, one warp
// per triangle, lanes over the covered columns) and then prefix-sums each
// column along z; the integer result equals the reference's per-voxel adds.
// All float64 arithmetic uses explicit round-to-nearest operations in the
// reference's order (no contraction).
//
// Seeding (mpm_solver.py:1017-1047): each voxel with a positive count emits
// the particles l = 0 .. sample_density with rand + l < s,
// s = sample_density / super_sample^3, at (rand3 + (i, j, k)) * voxel dx +
// translation.  The random numbers come from a counter-based hash
// (splitmix64 of the seed, the voxel index and the draw), so a seed gives
// the same particles on every run; they are not Taichi's ti.random stream.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_common.cuh"

namespace mpm {

constexpr int kVoxThreads = 256;

// engine/voxelizer.py:60-64: vertices shifted by this vector times 1e-8
// (float64 precision) so that voxel centres never lie exactly on an edge
__constant__ double kJitter[3] = {-0.057616723909439505, -0.25608986292614977, 0.06716309129743714};

__device__ __forceinline__ double cross2d(double ax, double ay, double bx, double by) {
  return __dsub_rn(__dmul_rn(ax, by), __dmul_rn(ay, bx));
}

// inside_ccw (voxelizer.py:10-13) for p against triangle (a, b, c)
__device__ __forceinline__ bool inside_ccw(double px, double py, double ax, double ay, double bx, double by,
                                           double cx, double cy) {
  const double apx = __dsub_rn(ax, px), apy = __dsub_rn(ay, py);
  const double bpx = __dsub_rn(bx, px), bpy = __dsub_rn(by, py);
  const double cpx = __dsub_rn(cx, px), cpy = __dsub_rn(cy, py);
  return cross2d(apx, apy, bpx, bpy) >= 0.0 && cross2d(bpx, bpy, cpx, cpy) >= 0.0 &&
         cross2d(cpx, cpy, apx, apy) >= 0.0;
}

// int(floor(x)) for the bounding-rectangle columns, kept inside int range
__device__ __forceinline__ int ifloor(double x) { return (int)floor(fmax(fmin(x, 1.0e9), -1.0e9)); }

struct VoxGrid {
  int rx, ry, rz, padding;
  double dx, inv_dx;
};

// One warp per triangle, lanes over the columns of its bounding rectangle.
__global__ __launch_bounds__(kVoxThreads) void k_voxelize(const double *__restrict__ tri, int64_t ntri, VoxGrid g,
                                                         int32_t *__restrict__ vox) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntri; t += warps) {
    double v[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d) v[k][d] = __dadd_rn(tri[t * 9 + k * 3 + d], __dmul_rn(kJitter[d], 1e-8));
    double bmin[3], bmax[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      bmin[d] = fmin(fmin(v[0][d], v[1][d]), v[2][d]);
      bmax[d] = fmax(fmax(v[0][d], v[1][d]), v[2][d]);
    }
    const int p_min = max(g.padding, ifloor(__dmul_rn(bmin[0], g.inv_dx)));
    const int p_max = min(g.rx - g.padding, ifloor(__dmul_rn(bmax[0], g.inv_dx)) + 1);
    const int q_min = max(g.padding, ifloor(__dmul_rn(bmin[1], g.inv_dx)));
    const int q_max = min(g.ry - g.padding, ifloor(__dmul_rn(bmax[1], g.inv_dx)) + 1);
    // normal = normalized((b - a) x (c - a)), voxelizer.py:81
    double e1[3], e2[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      e1[d] = __dsub_rn(v[1][d], v[0][d]);
      e2[d] = __dsub_rn(v[2][d], v[0][d]);
    }
    double nrm[3] = {__dsub_rn(__dmul_rn(e1[1], e2[2]), __dmul_rn(e1[2], e2[1])),
                     __dsub_rn(__dmul_rn(e1[2], e2[0]), __dmul_rn(e1[0], e2[2])),
                     __dsub_rn(__dmul_rn(e1[0], e2[1]), __dmul_rn(e1[1], e2[0]))};
    const double len =
        __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nrm[0], nrm[0]), __dmul_rn(nrm[1], nrm[1])), __dmul_rn(nrm[2], nrm[2])));
    const double invlen = __ddiv_rn(1.0, len);
#pragma unroll
    for (int d = 0; d < 3; ++d) nrm[d] = __dmul_rn(nrm[d], invlen);
    if (!(fabs(nrm[2]) >= 1e-10)) continue;  // also skips a degenerate (NaN) normal
    if (p_max <= p_min || q_max <= q_min) continue;
    const int inc = nrm[2] > 0.0 ? 1 : -1;
    const int nq = q_max - q_min;
    const int64_t ncols = (int64_t)(p_max - p_min) * nq;
    for (int64_t c = lane; c < ncols; c += 32) {
      const int p = p_min + (int)(c / nq), q = q_min + (int)(c % nq);
      const double px = __dmul_rn((double)p + 0.5, g.dx), py = __dmul_rn((double)q + 0.5, g.dx);
      if (!(inside_ccw(px, py, v[0][0], v[0][1], v[1][0], v[1][1], v[2][0], v[2][1]) ||
            inside_ccw(px, py, v[0][0], v[0][1], v[2][0], v[2][1], v[1][0], v[1][1])))
        continue;
      // height = int(-normal . (base - a) / normal.z * inv_dx + 0.5), base = (px, py, 0)
      const double dot = __dadd_rn(__dadd_rn(__dmul_rn(nrm[0], __dsub_rn(px, v[0][0])),
                                             __dmul_rn(nrm[1], __dsub_rn(py, v[0][1]))),
                                   __dmul_rn(nrm[2], __dsub_rn(0.0, v[0][2])));
      const double hf = __dadd_rn(__dmul_rn(__ddiv_rn(-dot, nrm[2]), g.inv_dx), 0.5);
      int height = (int)fmax(fmin(hf, 2147483000.0), -2147483000.0);  // int() truncates toward zero
      height = min(height, g.ry - g.padding);  // voxelizer.py:120 clamps with res[1]
      height = min(height, g.rz);              // and the column ends at res[2]
      if (height <= g.padding) continue;
      const int64_t col = ((int64_t)p * g.ry + q) * g.rz;
      atomicAdd(&vox[col + g.padding], inc);
      if (height < g.rz) atomicAdd(&vox[col + height], -inc);
    }
  }
}

// difference array -> counts: running sum along z of each column; one warp
// per column, lanes over consecutive z (coalesced), a warp scan per 32
__global__ __launch_bounds__(kVoxThreads) void k_vox_scan(VoxGrid g, int32_t *__restrict__ vox) {
  const int lane = threadIdx.x & 31;
  const int64_t col = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (col >= (int64_t)g.rx * g.ry) return;
  int32_t *c = vox + col * g.rz;
  int32_t carry = 0;
  for (int k0 = 0; k0 < g.rz; k0 += 32) {
    const int k = k0 + lane;
    int32_t v = k < g.rz ? c[k] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    if (k < g.rz) c[k] = carry + v;
    carry += __shfl_sync(0xffffffffu, v, 31);
  }
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// uniform float in [0, 1) with 24 random bits
__device__ __forceinline__ float rand01(uint64_t seed, uint64_t voxel, int draw) {
  const uint64_t h = splitmix64(splitmix64(splitmix64(seed ^ 0x5851F42D4C957F2Dull) + voxel) + (uint64_t)draw);
  return (float)(h >> 40) * (1.0f / 16777216.0f);
}

struct SeedParams {
  int sample_density;
  float s;  // sample_density / super_sample^3
  int grid_size, padding;
  uint64_t seed;
  float vdx;  // voxel dx
  float tx, ty, tz;
};

// Draw l of a voxel emits when rand + l < s (float32).  rand lies in
// [0, 1 - 2^-24], and float32 addition is monotonic, so l >= s never emits
// and (1 - 2^-24) + l < s always does; only the draw in between is random.
__device__ __forceinline__ bool emits_draw(const SeedParams &sp, uint64_t vidx, int l) {
  const float fl = (float)l;
  if (fl >= sp.s) return false;
  if (__fadd_rn(0.99999994f, fl) < sp.s) return true;
  return __fadd_rn(rand01(sp.seed, vidx, 4 * l), fl) < sp.s;
}

// particles voxel (i, j, k) emits: l in [0, sample_density] with rand + l < s
__device__ __forceinline__ int voxel_emits(const VoxGrid &g, const SeedParams &sp, int i, int64_t vidx, int32_t count) {
  // mpm_solver.py:1026-1029 tests index i only, for each of the 3 axes
  const bool inside = -sp.grid_size / 2 + sp.padding <= i && i < sp.grid_size / 2 - sp.padding;
  if (!inside || count <= 0) return 0;
  int m = 0;
  for (int l = 0; l <= sp.sample_density && (float)l < sp.s; ++l) m += emits_draw(sp, vidx, l);
  return m;
}

// one warp per voxel column, lanes over consecutive z
__global__ __launch_bounds__(kVoxThreads) void k_seed_count(VoxGrid g, SeedParams sp, const int32_t *__restrict__ vox,
                                                           int32_t *__restrict__ col_count) {
  const int lane = threadIdx.x & 31;
  const int64_t col = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (col >= (int64_t)g.rx * g.ry) return;
  const int i = (int)(col / g.ry);
  int m = 0;
  for (int k = lane; k < g.rz; k += 32) m += voxel_emits(g, sp, i, col * g.rz + k, vox[col * g.rz + k]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
  if (lane == 0) col_count[col] = m;
}

__global__ __launch_bounds__(kVoxThreads) void k_seed_emit(VoxGrid g, SeedParams sp, const int32_t *__restrict__ vox,
                                                          const int64_t *__restrict__ col_offset, int64_t n_out,
                                                          float *__restrict__ x_out) {
  const int lane = threadIdx.x & 31;
  const int64_t col = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (col >= (int64_t)g.rx * g.ry) return;
  const int i = (int)(col / g.ry), j = (int)(col % g.ry);
  int64_t base = col_offset[col];
  for (int k0 = 0; k0 < g.rz; k0 += 32) {
    const int k = k0 + lane;
    const int64_t vidx = col * g.rz + k;
    const int m = k < g.rz ? voxel_emits(g, sp, i, vidx, vox[vidx]) : 0;
    int incl = m;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    int64_t o = base + incl - m;
    for (int l = 0; m > 0 && l <= sp.sample_density && (float)l < sp.s; ++l) {
      if (!emits_draw(sp, vidx, l)) continue;
      if (o >= n_out) break;  // the count pass and this pass agree; never write past the output
      const float r0 = rand01(sp.seed, vidx, 4 * l + 1), r1 = rand01(sp.seed, vidx, 4 * l + 2),
                  r2 = rand01(sp.seed, vidx, 4 * l + 3);
      // x = (rand3 + (i, j, k)) * (dx / super_sample) + translation, float32
      x_out[o * 3 + 0] = __fadd_rn(__fmul_rn(__fadd_rn(r0, (float)i), sp.vdx), sp.tx);
      x_out[o * 3 + 1] = __fadd_rn(__fmul_rn(__fadd_rn(r1, (float)j), sp.vdx), sp.ty);
      x_out[o * 3 + 2] = __fadd_rn(__fmul_rn(__fadd_rn(r2, (float)k), sp.vdx), sp.tz);
      ++o;
    }
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
}

}  // namespace mpm

using namespace mpm;

extern "C" {

static bool vox_ok(int32_t rx, int32_t ry, int32_t rz, int32_t padding, double dx) {
  return rx > 0 && ry > 0 && rz > 0 && padding >= 0 && dx > 0.0 && (int64_t)rx * ry * rz < (int64_t)1 << 34;
}

int mpm_voxelize(const double *triangles, int64_t ntri, int32_t rx, int32_t ry, int32_t rz, double dx,
                 int32_t padding, int32_t *voxels, void *stream) {
  if (!voxels || ntri < 0 || (ntri > 0 && !triangles) || !vox_ok(rx, ry, rz, padding, dx)) return MPM_E_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = (size_t)rx * ry * rz * sizeof(int32_t);
  if (cudaMemsetAsync(voxels, 0, bytes, s) != cudaSuccess) return MPM_E_CUDA;
  VoxGrid g{rx, ry, rz, padding, dx, 1.0 / dx};
  if (ntri > 0) {
    const int64_t blocks = (ntri * 32 + kVoxThreads - 1) / kVoxThreads;
    k_voxelize<<<(unsigned)(blocks < 65535 * 16 ? blocks : 65535 * 16), kVoxThreads, 0, s>>>(triangles, ntri, g,
                                                                                            voxels);
  }
  const int64_t cols = (int64_t)rx * ry;
  k_vox_scan<<<(unsigned)((cols * 32 + kVoxThreads - 1) / kVoxThreads), kVoxThreads, 0, s>>>(g, voxels);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_voxel_seed_count(const int32_t *voxels, int32_t rx, int32_t ry, int32_t rz, int32_t sample_density,
                         int32_t super_sample, int32_t grid_size, int32_t padding, uint64_t seed, int32_t *col_count,
                         void *stream) {
  if (!voxels || !col_count || sample_density < 0 || super_sample < 1 || !vox_ok(rx, ry, rz, padding, 1.0))
    return MPM_E_INVALID;
  VoxGrid g{rx, ry, rz, padding, 1.0, 1.0};
  const float ss3 = (float)super_sample * (float)super_sample * (float)super_sample;
  SeedParams sp{sample_density, (float)sample_density / ss3, grid_size, padding, seed, 0.f, 0.f, 0.f, 0.f};
  const int64_t cols = (int64_t)rx * ry;
  k_seed_count<<<(unsigned)((cols * 32 + kVoxThreads - 1) / kVoxThreads), kVoxThreads, 0, (cudaStream_t)stream>>>(
      g, sp, voxels, col_count);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_voxel_seed_emit(const int32_t *voxels, int32_t rx, int32_t ry, int32_t rz, int32_t sample_density,
                        int32_t super_sample, int32_t grid_size, int32_t padding, uint64_t seed, float voxel_dx,
                        float tx, float ty, float tz, const int64_t *col_offset, int64_t n_out, float *x_out,
                        void *stream) {
  if (!voxels || !col_offset || (n_out > 0 && !x_out) || n_out < 0 || sample_density < 0 || super_sample < 1 ||
      !vox_ok(rx, ry, rz, padding, 1.0))
    return MPM_E_INVALID;
  VoxGrid g{rx, ry, rz, padding, 1.0, 1.0};
  const float ss3 = (float)super_sample * (float)super_sample * (float)super_sample;
  SeedParams sp{sample_density, (float)sample_density / ss3, grid_size, padding, seed, voxel_dx, tx, ty, tz};
  const int64_t cols = (int64_t)rx * ry;
  k_seed_emit<<<(unsigned)((cols * 32 + kVoxThreads - 1) / kVoxThreads), kVoxThreads, 0, (cudaStream_t)stream>>>(
      g, sp, voxels, col_offset, n_out, x_out);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

}  // extern "C"
