// Particle output on the GPU: the quantised frame format of
// taichi-dev/taichi_elements engine/particle_io.py:12-76
// (ParticleIO.write_particles).  Per dimension d the positions and the
// velocities are mapped to [lo, hi] ranges (min / max over all particles,
// hi raised to lo + 1e-5 when narrower), then quantised to 24 (x) and 8 (v)
// bits and packed into one uint32 per component, (qx << 8) + qv; 24-bit
// colours are split into R, G, B bytes.  The float32 arithmetic follows the
// reference's numpy expression step by step with round-to-nearest
// operations and no contraction:
//   q = uint32(((x - lo) * (1 / (hi - lo))) * (2^bits - 1) + 0.499)
// with uint32 wrap-around in the shift and the add, as numpy's uint32 does.
// Output rows are in original particle order (scattered by the id row).
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_common.cuh"

namespace mpm {

constexpr int kIoThreads = 256;
constexpr int kVBits = 8;
constexpr int kXBits = 32 - kVBits;

// Order-preserving uint32 key of a float (total order of the non-NaN
// floats, -0 below +0), so that min / max reduce with integer atomics.
__device__ __forceinline__ uint32_t float_key(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__global__ void k_range_init(uint32_t *keys) {
  const int t = threadIdx.x;
  if (t < 12) keys[t] = (t & 1) ? 0u : 0xFFFFFFFFu;  // even slots min, odd slots max
}

// keys[(c*3 + d)*2 + {0: min, 1: max}], c = 0 positions, 1 velocities
__global__ __launch_bounds__(kIoThreads) void k_range_reduce(const float *__restrict__ st, int64_t cap, int64_t n,
                                                             uint32_t *keys) {
  uint32_t lo[6], hi[6];
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    lo[q] = 0xFFFFFFFFu;
    hi[q] = 0u;
  }
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const uint32_t k = float_key(st[((q < 3 ? kX : kV - 3) + q) * cap + j]);
      lo[q] = min(lo[q], k);
      hi[q] = max(hi[q], k);
    }
  }
#pragma unroll
  for (int q = 0; q < 6; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[q] = min(lo[q], __shfl_xor_sync(0xffffffffu, lo[q], o));
      hi[q] = max(hi[q], __shfl_xor_sync(0xffffffffu, hi[q], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      atomicMin(&keys[2 * q], lo[q]);
      atomicMax(&keys[2 * q + 1], hi[q]);
    }
  }
}

// ranges[c][d][0..1] (float32, the reference's (2, 3, 2) array) with the
// narrow-range rule hi = max(lo + 1e-5, hi) (engine/particle_io.py:48-50)
__global__ void k_range_finish(const uint32_t *keys, float *ranges) {
  const int q = threadIdx.x;
  if (q < 6) {
    const float lo = key_float(keys[2 * q]);
    const float hi = key_float(keys[2 * q + 1]);
    const float lo_eps = __fadd_rn(lo, 1e-5f);
    ranges[2 * q] = lo;
    ranges[2 * q + 1] = lo_eps > hi ? lo_eps : hi;
  }
}

__device__ __forceinline__ uint32_t quantise(float v, float lo, float inv, float scale) {
  const float u = __fadd_rn(__fmul_rn(__fmul_rn(__fsub_rn(v, lo), inv), scale), 0.499f);
  return __float2uint_rz(u);
}

__global__ __launch_bounds__(kIoThreads) void k_quantise(const float *__restrict__ st, int64_t cap, int64_t n,
                                                         const float *__restrict__ ranges,
                                                         uint32_t *__restrict__ out) {
  // per range: lo and 1 / (hi - lo), computed once per CTA (the reference
  // computes the reciprocal once per dimension, engine/particle_io.py:51-56)
  __shared__ float lo_s[6], inv_s[6];
  if (threadIdx.x < 6) {
    const float lo = ranges[2 * threadIdx.x], hi = ranges[2 * threadIdx.x + 1];
    lo_s[threadIdx.x] = lo;
    inv_s[threadIdx.x] = __fdiv_rn(1.0f, __fsub_rn(hi, lo));
  }
  __syncthreads();
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t id = __float_as_int(st[kId * cap + j]);
  if (id < 0 || id >= n) return;  // corrupted id row: leave the row untouched
  const float xs = (float)((1u << kXBits) - 1u), vs = (float)((1u << kVBits) - 1u);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const uint32_t qx = quantise(st[(kX + d) * cap + j], lo_s[d], inv_s[d], xs);
    const uint32_t qv = quantise(st[(kV + d) * cap + j], lo_s[3 + d], inv_s[3 + d], vs);
    out[id * 3 + d] = (qx << kVBits) + qv;  // uint32 wrap-around, as numpy
  }
}

__global__ __launch_bounds__(kIoThreads) void k_unpack_colors(const int32_t *__restrict__ color, int64_t n,
                                                              uint8_t *__restrict__ rgb) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = (uint32_t)color[i];
  rgb[i * 3 + 0] = (uint8_t)((c >> 16) & 255u);
  rgb[i * 3 + 1] = (uint8_t)((c >> 8) & 255u);
  rgb[i * 3 + 2] = (uint8_t)(c & 255u);
}

// ---------------------------------------------- packed particle storage --
//
// Conversion between the float32 row layout and the packed layout of
// quant=True (quant.cuh).  Both keep the slot order.

__global__ __launch_bounds__(kIoThreads) void k_quant_pack(const float *__restrict__ rows, int64_t rows_cap,
                                                           int64_t count, float *__restrict__ pk, int64_t cap,
                                                           int64_t begin, int32_t *status) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t j = begin + t;
  uint32_t bad = 0;
  if (t < count) {
    using R = PRows<true>;
    using L = PRows<false>;
    float x[3], v[3], F[3][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      x[d] = rows[(L::X + d) * rows_cap + t];
      v[d] = rows[(L::V + d) * rows_cap + t];
    }
#pragma unroll
    for (int a = 0; a < 9; ++a) F[a / 3][a % 3] = rows[(L::F + a) * rows_cap + t];
    st_x<true>(pk, cap, j, x, bad);
    st_v<true>(pk, cap, j, v, bad);
    st_F_mat<true>(pk, cap, j, F, __float_as_int(rows[L::Mat * rows_cap + t]));
    pk[R::Jp * cap + j] = rows[L::Jp * rows_cap + t];
    pk[R::Id * cap + j] = rows[L::Id * rows_cap + t];
    pk[R::Ep * cap + j] = rows[L::Ep * rows_cap + t];
#pragma unroll
    for (int a = 0; a < 9; ++a) pk[(R::C + a) * cap + j] = rows[(L::C + a) * rows_cap + t];
  }
  if (status && bad) atomicOr(status, (int32_t)bad);
}

__global__ __launch_bounds__(kIoThreads) void k_quant_unpack(const float *__restrict__ pk, int64_t cap,
                                                             int64_t begin, int64_t count, float *__restrict__ rows,
                                                             int64_t rows_cap) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int64_t j = begin + t;
  using R = PRows<true>;
  using L = PRows<false>;
  float x[3], v[3], F[3][3];
  ld_x<true>(pk, cap, j, x);
  ld_v<true>(pk, cap, j, v);
  ld_F<true>(pk, cap, j, F);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rows[(L::X + d) * rows_cap + t] = x[d];
    rows[(L::V + d) * rows_cap + t] = v[d];
  }
#pragma unroll
  for (int a = 0; a < 9; ++a) {
    rows[(L::F + a) * rows_cap + t] = F[a / 3][a % 3];
    rows[(L::C + a) * rows_cap + t] = pk[(R::C + a) * cap + j];
  }
  rows[L::Mat * rows_cap + t] = __int_as_float(ld_mat<true>(pk, cap, j));
  rows[L::Jp * rows_cap + t] = pk[R::Jp * cap + j];
  rows[L::Id * rows_cap + t] = pk[R::Id * cap + j];
  rows[L::Ep * rows_cap + t] = pk[R::Ep * cap + j];
}

}  // namespace mpm

using namespace mpm;

extern "C" {

static int io_grid(int64_t n) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  const int64_t need = (n + kIoThreads - 1) / kIoThreads;
  const int64_t g = (int64_t)sms * 8;
  return (int)(need < g ? (need > 0 ? need : 1) : g);
}

int mpm_particle_ranges(const float *pstate, int64_t cap, int64_t n, uint32_t *keys, float *ranges_out,
                        void *stream) {
  if (!pstate || !keys || !ranges_out || n < 1 || n > cap) return MPM_E_INVALID;
  const int g = io_grid(n);
  if (!g) return MPM_E_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  k_range_init<<<1, 32, 0, s>>>(keys);
  k_range_reduce<<<g, kIoThreads, 0, s>>>(pstate, cap, n, keys);
  k_range_finish<<<1, 32, 0, s>>>(keys, ranges_out);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_quantize_particles(const float *pstate, int64_t cap, int64_t n, const float *ranges, uint32_t *x_and_v,
                           void *stream) {
  if (!pstate || !ranges || !x_and_v || n < 0 || n > cap) return MPM_E_INVALID;
  if (n == 0) return MPM_OK;
  k_quantise<<<(unsigned)((n + kIoThreads - 1) / kIoThreads), kIoThreads, 0, (cudaStream_t)stream>>>(
      pstate, cap, n, ranges, x_and_v);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_unpack_colors(const int32_t *color, int64_t n, uint8_t *rgb, void *stream) {
  if (!color || !rgb || n < 0) return MPM_E_INVALID;
  if (n == 0) return MPM_OK;
  k_unpack_colors<<<(unsigned)((n + kIoThreads - 1) / kIoThreads), kIoThreads, 0, (cudaStream_t)stream>>>(color, n,
                                                                                                        rgb);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_quant_pack(const float *rows, int64_t rows_cap, int64_t count, float *packed, int64_t cap, int64_t begin,
                   int32_t *status, void *stream) {
  if (!rows || !packed || count < 0 || begin < 0 || count > rows_cap || begin + count > cap) return MPM_E_INVALID;
  if (count == 0) return MPM_OK;
  k_quant_pack<<<(unsigned)((count + kIoThreads - 1) / kIoThreads), kIoThreads, 0, (cudaStream_t)stream>>>(
      rows, rows_cap, count, packed, cap, begin, status);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_quant_unpack(const float *packed, int64_t cap, int64_t begin, int64_t count, float *rows, int64_t rows_cap,
                     void *stream) {
  if (!rows || !packed || count < 0 || begin < 0 || count > rows_cap || begin + count > cap) return MPM_E_INVALID;
  if (count == 0) return MPM_OK;
  k_quant_unpack<<<(unsigned)((count + kIoThreads - 1) / kIoThreads), kIoThreads, 0, (cudaStream_t)stream>>>(
      packed, cap, begin, count, rows, rows_cap);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

}  // extern "C"
