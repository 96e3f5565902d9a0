// 3x3 singular value decomposition for the P2G stress (float32, registers only).
//
// Replaces Taichi's ti.svd (called at engine/mpm_solver.py:525 of
// taichi-dev/taichi_elements).  The structure follows the published method of
// McAdams, Selle, Tamstorf, Teran and Sifakis (2011), "Computing the Singular
// Value Decomposition of 3x3 matrices with minimal branching and elementary
// floating point operations": symmetric eigen-analysis of A^T A by cyclic
// Jacobi rotations, sorting of the columns of B = A V with sign-preserving
// swaps, then a Givens QR of B.  This implementation uses exact Jacobi angles
// (Rutishauser's formula) rather than the paper's approximate quarter angles.
//
// Convention (the one the reference's constitutive code relies on):
//   A = U diag(s) V^T with U, V proper rotations (det = +1),
//   s0 >= s1 >= |s2|, and s2 < 0 exactly when det(A) < 0.
#pragma once

namespace mpm {

// 1/sqrt(x) to about 1 ulp: the hardware estimate refined by one
// Newton-Raphson step for f(y) = 1/y^2 - x, y <- y (3 - x y^2) / 2.
// Rotation cosines/sines built from it keep U and V orthogonal to float
// precision, which the corotated stress 2 mu (F - U V^T) F^T needs.
__device__ __forceinline__ float rsqrt_nr(float x) {
  const float y = rsqrtf(x);
  return y * fmaf(-0.5f * x * y, y, 1.5f);
}

// 1/x to about 1 ulp: the hardware estimate refined by one Newton-Raphson
// step for f(r) = 1/r - x, r <- r (2 - x r).
__device__ __forceinline__ float rcp_nr(float x) {
  const float r = __fdividef(1.0f, x);
  return r * fmaf(-x, r, 2.0f);
}

// One Jacobi rotation in the (P, Q) plane, branch free.  With d = S_qq - S_pp
// and a = S_pq, Rutishauser's t = sign(theta) / (|theta| + sqrt(theta^2 + 1)),
// theta = d / (2a), is rewritten as t = 2 a sgn(d) / (|d| + sqrt(d^2 + 4a^2)),
// which needs no division by a and gives t = 0 (no rotation) when a = 0.
template <int P, int Q>
__device__ __forceinline__ void jacobi_pair(float (&S)[3][3], float (&V)[3][3]) {
  constexpr int R = 3 - P - Q;
  const float apq = S[P][Q];
  const float d = S[Q][Q] - S[P][P];
  const float r = fmaf(d, d, 4.0f * apq * apq);
  const float den = fabsf(d) + r * rsqrtf(fmaxf(r, 1e-37f));
  const float t = copysignf(2.0f, d) * apq * __fdividef(1.0f, fmaxf(den, 1e-37f));
  const float c = rsqrt_nr(fmaf(t, t, 1.0f));
  const float s = t * c;
  S[P][P] -= t * apq;
  S[Q][Q] += t * apq;
  S[P][Q] = 0.0f;
  S[Q][P] = 0.0f;
  const float srp = S[R][P], srq = S[R][Q];
  S[R][P] = S[P][R] = c * srp - s * srq;
  S[R][Q] = S[Q][R] = s * srp + c * srq;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float vp = V[i][P], vq = V[i][Q];
    V[i][P] = c * vp - s * vq;
    V[i][Q] = s * vp + c * vq;
  }
}

template <int I, int J>
__device__ __forceinline__ void givens_qr_step(float (&B)[3][3], float (&U)[3][3]) {
  // zero B[J][I] with a rotation of rows I and J; U accumulates G^T.
  const float a = B[I][I], b = B[J][I];
  const float r2 = fmaf(a, a, b * b);
  const bool nz = r2 > 0.0f;
  const float ir = rsqrt_nr(nz ? r2 : 1.0f);
  const float c = nz ? a * ir : 1.0f;
  const float s = nz ? b * ir : 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float bi = B[I][k], bj = B[J][k];
    B[I][k] = c * bi + s * bj;
    B[J][k] = c * bj - s * bi;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float ui = U[k][I], uj = U[k][J];
    U[k][I] = c * ui + s * uj;
    U[k][J] = c * uj - s * ui;
  }
}

template <int I, int J>
__device__ __forceinline__ void cond_swap(bool doit, float (&B)[3][3], float (&V)[3][3], float (&rho)[3]) {
  // swap columns I, J and negate the new column J (keeps det V = +1)
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float bi = B[k][I], bj = B[k][J];
    B[k][I] = doit ? bj : bi;
    B[k][J] = doit ? -bi : bj;
    const float vi = V[k][I], vj = V[k][J];
    V[k][I] = doit ? vj : vi;
    V[k][J] = doit ? -vi : vj;
  }
  const float ri = rho[I], rj = rho[J];
  rho[I] = doit ? rj : ri;
  rho[J] = doit ? ri : rj;
}

// Rotation factor R of the polar decomposition F = R S by Newton's
// iteration R <- (R + R^{-T}) / 2 (Higham, "Computing the polar
// decomposition - with applications", 1986), starting from R = F.  Valid for
// det F > 0, where R equals U V^T of the SVD convention above.  Newton's
// iteration converges quadratically: once a step moves R by at most 3e-4 the
// remaining error is below about 5e-8, so the loop stops there.  Returns false
// when that has not happened after MAX_ITERS steps (very large stretch), and
// for a nearly singular F (det F around 1e-17 relative to |F|^3, e.g. a
// particle flattened against a wall), where the iterates overflow before they
// converge; the caller then uses the SVD.  The iterates must stay finite:
// fmaxf drops a NaN operand, so a NaN iterate would read as converged.
template <int MAX_ITERS = 6>
__device__ __forceinline__ bool polar_rotation(const float (&F)[3][3], float (&R)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) R[i][j] = F[i][j];
  bool done = false;
  for (int it = 0; it < MAX_ITERS && !done; ++it) {
    float Cf[3][3];  // cofactor matrix: R^{-T} = Cf / det
    Cf[0][0] = R[1][1] * R[2][2] - R[1][2] * R[2][1];
    Cf[0][1] = R[1][2] * R[2][0] - R[1][0] * R[2][2];
    Cf[0][2] = R[1][0] * R[2][1] - R[1][1] * R[2][0];
    Cf[1][0] = R[0][2] * R[2][1] - R[0][1] * R[2][2];
    Cf[1][1] = R[0][0] * R[2][2] - R[0][2] * R[2][0];
    Cf[1][2] = R[0][1] * R[2][0] - R[0][0] * R[2][1];
    Cf[2][0] = R[0][1] * R[1][2] - R[0][2] * R[1][1];
    Cf[2][1] = R[0][2] * R[1][0] - R[0][0] * R[1][2];
    Cf[2][2] = R[0][0] * R[1][1] - R[0][1] * R[1][0];
    const float det = R[0][0] * Cf[0][0] + R[0][1] * Cf[0][1] + R[0][2] * Cf[0][2];
    const float h = 0.5f * rcp_nr(det);
    if (!(fabsf(h) <= 3.0e38f)) return false;  // det overflowed, vanished or is NaN
    float change = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float r = fmaf(0.5f, R[i][j], h * Cf[i][j]);
        change = fmaxf(change, fabsf(r - R[i][j]));
        R[i][j] = r;
      }
    done = change <= 3e-4f;
  }
  float sum = 0.0f;  // NaN or infinite if any entry is
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) sum += R[i][j];
  return done && fabsf(sum) <= 3.0e38f;
}

template <int SWEEPS = 4>
__device__ __forceinline__ void svd3(const float (&A)[3][3], float (&U)[3][3], float (&s)[3],
                                     float (&V)[3][3]) {
  float S[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      float acc = A[0][i] * A[0][j];
      acc = fmaf(A[1][i], A[1][j], acc);
      acc = fmaf(A[2][i], A[2][j], acc);
      S[i][j] = acc;
      S[j][i] = acc;
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      V[i][j] = (i == j) ? 1.0f : 0.0f;
      U[i][j] = (i == j) ? 1.0f : 0.0f;
    }
#pragma unroll
  for (int sweep = 0; sweep < SWEEPS; ++sweep) {
    jacobi_pair<0, 1>(S, V);
    jacobi_pair<0, 2>(S, V);
    jacobi_pair<1, 2>(S, V);
  }
  float B[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float acc = A[i][0] * V[0][j];
      acc = fmaf(A[i][1], V[1][j], acc);
      acc = fmaf(A[i][2], V[2][j], acc);
      B[i][j] = acc;
    }
  float rho[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) rho[j] = fmaf(B[0][j], B[0][j], fmaf(B[1][j], B[1][j], B[2][j] * B[2][j]));
  cond_swap<0, 1>(rho[0] < rho[1], B, V, rho);
  cond_swap<0, 2>(rho[0] < rho[2], B, V, rho);
  cond_swap<1, 2>(rho[1] < rho[2], B, V, rho);
  givens_qr_step<0, 1>(B, U);
  givens_qr_step<0, 2>(B, U);
  givens_qr_step<1, 2>(B, U);
  s[0] = B[0][0];
  s[1] = B[1][1];
  s[2] = B[2][2];
}

}  // namespace mpm
