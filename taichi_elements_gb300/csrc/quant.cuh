// Particle state rows in HBM, for both storage modes of MPMSolver.
//
// float32 layout (quant=False): 28 rows of `cap` floats,
//   x 0-2, v 3-5, C 6-14, F 15-23, Jp 24, material word 25, id 26, E_p 27.
//
// Packed layout (quant=True, engine/mpm_solver.py:106-127 and :216-262): 21
// rows of `cap` 32-bit words with the reference's bit widths and ranges:
//   rows 0-1  position: three signed 21-bit fixed-point values of scale 2^-19
//             (range [-2, 2)), word pair = q0 | q1 << 21 | q2 << 42
//   rows 2-3  velocity: a 7-bit shared exponent and three signed 19-bit
//             mantissas (block floating point, the largest component keeps 18
//             significant bits), word pair = e | m0 << 7 | m1 << 26 | m2 << 45
//   rows 4-8  F: nine signed 16-bit fixed-point values of scale 4.1 / 2^15
//             (F_bound + 0.1), two per word in the reference's pairing
//             (F00,F01) (F02,F10) (F11,F12) (F20,F21) (F22,material)
//   row 9 Jp, row 10 id, row 11 E_p (float32 as above), rows 12-20 C.
// Values are rounded to the nearest representable value, ties away from
// zero.  Positions outside [-2, 2) raise the out-of-grid status and F
// entries outside the range saturate; non-finite values store 0 (and raise
// the non-finite status for x and v).
#pragma once

#include <stdint.h>

#include "mpm_gb300.h"

namespace mpm {

template <bool Q>
struct PRows {
  static constexpr int X = 0, V = 3, C = 6, F = 15, Jp = 24, Mat = 25, Id = 26, Ep = 27, N = 28;
};
template <>
struct PRows<true> {
  static constexpr int X = 0, V = 2, F = 4, Jp = 9, Id = 10, Ep = 11, C = 12, N = 21;
};

constexpr float kQxScale = 1.0f / 524288.0f;  // 2^-19
constexpr float kQxInv = 524288.0f;
constexpr int kQxMax = (1 << 20) - 1;
constexpr float kQfScale = (float)(4.1 / 32768.0);
constexpr float kQfInv = (float)(32768.0 / 4.1);
constexpr int kQvBias = 100;  // unit exponent u = e - 100, e in [0, 127]

__device__ __forceinline__ int32_t q_round(float s) {  // ties away from zero
  return __float2int_rz(__fadd_rn(s, copysignf(0.5f, s)));
}

// 16-bit code of one F entry: saturating, 0 for a non-finite value
__device__ __forceinline__ int32_t qf_code(float v) {
  return isfinite(v) ? max(-32768, min(32767, q_round(__fmul_rn(v, kQfInv)))) : 0;
}

__device__ __forceinline__ float q_fixed_F(float v) {  // quantize and decode one F entry
  return __fmul_rn((float)qf_code(v), kQfScale);
}

__device__ __forceinline__ float pow2f(int u) {  // 2^u for u in [-126, 127]
  return __int_as_float((u + 127) << 23);
}

// Block floating point encoding of a velocity: returns the exponent code and
// the three mantissas (each |m| <= 2^18 - 1).  Non-finite input encodes zero
// and sets bit 1 (non-finite) of *bad.
__device__ __forceinline__ void qv_encode(const float (&v)[3], int &e, int32_t (&m)[3], uint32_t &bad) {
  const float M = fmaxf(fabsf(v[0]), fmaxf(fabsf(v[1]), fabsf(v[2])));
  if (!(M <= 3.402823466e38f) || !isfinite(v[0]) || !isfinite(v[1]) || !isfinite(v[2])) {
    bad |= MPM_STATUS_NONFINITE;
    e = 0;
    m[0] = m[1] = m[2] = 0;
    return;
  }
  // M in [2^(k-1), 2^k) with k from the exponent field (subnormal and zero M
  // give the smallest unit)
  const int k = (int)((__float_as_uint(M) >> 23) & 0xFFu) - 126;
  int u = max(k - 18, -kQvBias);
  u = min(u, 127 - kQvBias);
  for (int pass = 0; pass < 2; ++pass) {
    const float s = pow2f(-u);
    int32_t big = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      m[d] = q_round(__fmul_rn(v[d], s));
      big = max(big, abs(m[d]));
    }
    if (big < (1 << 18) || u == 127 - kQvBias) break;
    ++u;  // rounding carried the largest mantissa to 2^18
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) m[d] = max(-((1 << 18) - 1), min((1 << 18) - 1, m[d]));
  e = u + kQvBias;
}

__device__ __forceinline__ void qv_decode(uint32_t lo, uint32_t hi, float (&v)[3]) {
  const uint64_t w = (uint64_t)lo | ((uint64_t)hi << 32);
  const float s = pow2f((int)(w & 127u) - kQvBias);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int32_t m = (int32_t)((uint32_t)(w >> (7 + 19 * d)) << 13) >> 13;  // sign-extend 19 bits
    v[d] = __fmul_rn((float)m, s);
  }
}

__device__ __forceinline__ void qx_decode(uint32_t lo, uint32_t hi, float (&x)[3]) {
  const uint64_t w = (uint64_t)lo | ((uint64_t)hi << 32);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int32_t q = (int32_t)((uint32_t)(w >> (21 * d)) << 11) >> 11;  // sign-extend 21 bits
    x[d] = __fmul_rn((float)q, kQxScale);
  }
}

// Quantizes x in place (the value the packed row holds) and returns the
// word pair; positions outside [-2, 2) are clamped and flagged.
__device__ __forceinline__ uint64_t qx_encode(float (&x)[3], uint32_t &bad) {
  uint64_t w = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int32_t q = q_round(__fmul_rn(x[d], kQxInv));
    if (!isfinite(x[d])) {
      bad |= MPM_STATUS_NONFINITE;
      q = 0;
    } else if (q < -kQxMax - 1 || q > kQxMax) {
      bad |= MPM_STATUS_OUT_OF_GRID;
      q = max(-kQxMax - 1, min(kQxMax, q));
    }
    x[d] = __fmul_rn((float)q, kQxScale);
    w |= (uint64_t)((uint32_t)q & 0x1FFFFFu) << (21 * d);
  }
  return w;
}

// ------------------------------------------------ row accessors (j = slot) --

template <bool Q>
__device__ __forceinline__ void ld_x(const float *__restrict__ s, int64_t cap, int64_t j, float (&x)[3]) {
  if (Q) {
    const uint32_t *u = reinterpret_cast<const uint32_t *>(s);
    qx_decode(u[j], u[cap + j], x);
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) x[d] = s[(PRows<Q>::X + d) * cap + j];
  }
}

// Stores x; in the packed layout x is first rounded to the stored value.
template <bool Q>
__device__ __forceinline__ void st_x(float *__restrict__ s, int64_t cap, int64_t j, float (&x)[3], uint32_t &bad) {
  if (Q) {
    const uint64_t w = qx_encode(x, bad);
    uint32_t *u = reinterpret_cast<uint32_t *>(s);
    u[j] = (uint32_t)w;
    u[cap + j] = (uint32_t)(w >> 32);
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) s[(PRows<Q>::X + d) * cap + j] = x[d];
  }
}

// Copies the stored position words of slot i of s to slot j of d unchanged.
template <bool Q>
__device__ __forceinline__ void cp_x(const float *__restrict__ s, int64_t i, float *__restrict__ d, int64_t j,
                                     int64_t cap) {
#pragma unroll
  for (int r = 0; r < (Q ? 2 : 3); ++r) d[r * cap + j] = s[r * cap + i];
}

template <bool Q>
__device__ __forceinline__ void ld_v(const float *__restrict__ s, int64_t cap, int64_t j, float (&v)[3]) {
  if (Q) {
    const uint32_t *u = reinterpret_cast<const uint32_t *>(s + PRows<Q>::V * cap);
    qv_decode(u[j], u[cap + j], v);
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = s[(PRows<Q>::V + d) * cap + j];
  }
}

// Stores v; in the packed layout v is first rounded to the stored value.
template <bool Q>
__device__ __forceinline__ void st_v(float *__restrict__ s, int64_t cap, int64_t j, float (&v)[3], uint32_t &bad) {
  if (Q) {
    int e;
    int32_t m[3];
    qv_encode(v, e, m, bad);
    const float sc = pow2f(e - kQvBias);
    uint64_t w = (uint64_t)e;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      v[d] = __fmul_rn((float)m[d], sc);
      w |= (uint64_t)((uint32_t)m[d] & 0x7FFFFu) << (7 + 19 * d);
    }
    uint32_t *u = reinterpret_cast<uint32_t *>(s + PRows<Q>::V * cap);
    u[j] = (uint32_t)w;
    u[cap + j] = (uint32_t)(w >> 32);
  } else {
#pragma unroll
    for (int d = 0; d < 3; ++d) s[(PRows<Q>::V + d) * cap + j] = v[d];
  }
}

template <bool Q>
__device__ __forceinline__ int ld_mat(const float *__restrict__ s, int64_t cap, int64_t j) {
  if (Q) return (int)(reinterpret_cast<const uint32_t *>(s)[(PRows<Q>::F + 4) * cap + j] >> 16);
  return __float_as_int(s[PRows<false>::Mat * cap + j]);
}

template <bool Q>
__device__ __forceinline__ void ld_F(const float *__restrict__ s, int64_t cap, int64_t j, float (&F)[3][3]) {
  if (Q) {
    const uint32_t *u = reinterpret_cast<const uint32_t *>(s + PRows<Q>::F * cap);
#pragma unroll
    for (int a = 0; a < 9; ++a) {
      const uint32_t wd = u[(a >> 1) * cap + j];
      const int16_t q = (int16_t)((a & 1) ? (wd >> 16) : (wd & 0xFFFFu));
      F[a / 3][a % 3] = __fmul_rn((float)q, kQfScale);
    }
  } else {
#pragma unroll
    for (int a = 0; a < 9; ++a) F[a / 3][a % 3] = s[(PRows<Q>::F + a) * cap + j];
  }
}

// Stores F (and, in the packed layout, the material word's low 16 bits,
// which share the last word).  The float32 layout stores the material row.
template <bool Q>
__device__ __forceinline__ void st_F_mat(float *__restrict__ s, int64_t cap, int64_t j, const float (&F)[3][3],
                                         int matword) {
  if (Q) {
    uint32_t h[10];
#pragma unroll
    for (int a = 0; a < 9; ++a)
      h[a] = (uint32_t)(uint16_t)qf_code(F[a / 3][a % 3]);
    h[9] = (uint32_t)matword & 0xFFFFu;
    uint32_t *u = reinterpret_cast<uint32_t *>(s + PRows<Q>::F * cap);
#pragma unroll
    for (int r = 0; r < 5; ++r) u[r * cap + j] = h[2 * r] | (h[2 * r + 1] << 16);
  } else {
#pragma unroll
    for (int a = 0; a < 9; ++a) s[(PRows<Q>::F + a) * cap + j] = F[a / 3][a % 3];
    s[PRows<false>::Mat * cap + j] = __int_as_float(matword);
  }
}

}  // namespace mpm
