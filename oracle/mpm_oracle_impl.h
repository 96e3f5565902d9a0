/*
 * CPU restatement of the MLS-MPM substep of taichi-dev/taichi_elements
 * (engine/mpm_solver.py), templated on the scalar type.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA engine
 * is checked against and the timed CPU baseline of the benchmark; nothing
 * in the product package links, loads or calls it.
 *
 * It is included twice by mpm_oracle.c, once with REAL=double / SFX=_d and
 * once with REAL=float / SFX=_f.  Every function names the reference lines
 * it restates.  Parity status: the reference publishes no golden vectors and
 * its Taichi runtime cannot be imported on this machine, so this restatement
 * is pinned only by known-answer physics tests and by an independent numpy
 * restatement (parity unpinned against the reference's own outputs).
 *
 * Third-party pieces restated (Taichi 1.1.0, not vendored in the reference):
 *   - ti.svd (call site engine/mpm_solver.py:525): restated as the published
 *     3x3 SVD structure of McAdams et al. 2011 ("Computing the Singular
 *     Value Decomposition of 3x3 matrices with minimal branching and
 *     elementary floating point operations"): Jacobi eigen-analysis of
 *     A^T A, column sort with sign-preserving swaps, Givens QR.  Convention:
 *     U, V are rotations (det +1), sigma_0 >= sigma_1 >= |sigma_2| and
 *     sigma_2 carries the sign of det(A).  Exact Jacobi angles are used.
 *   - Matrix.normalized(eps): v / (|v| + eps).
 */

#ifndef REAL
#error "REAL must be defined"
#endif

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

#if defined(ORACLE_IS_FLOAT)
#define RSQRT(x) (1.0f / sqrtf(x))
#define SQRT(x) sqrtf(x)
#define EXP(x) expf(x)
#define LOG(x) logf(x)
#define FABS(x) fabsf(x)
#define FLOOR(x) floorf(x)
#define FREXP(x, e) frexpf(x, e)
#define LDEXP(x, e) ldexpf(x, e)
#define SVD_SWEEPS 5
#else
#define RSQRT(x) (1.0 / sqrt(x))
#define SQRT(x) sqrt(x)
#define EXP(x) exp(x)
#define LOG(x) log(x)
#define FABS(x) fabs(x)
#define FLOOR(x) floor(x)
#define FREXP(x, e) frexp(x, e)
#define LDEXP(x, e) ldexp(x, e)
#define SVD_SWEEPS 40
#endif

typedef struct {
  REAL dx, inv_dx, p_vol, p_mass, mu0, la0, alpha, water_density;
  REAL gravity[3];
  REAL stress_scale_k; /* p_vol * 4 * inv_dx^2 */
  REAL sand_k;         /* (3 la0 + 2 mu0) / (2 mu0) */
  REAL nu;
  int plasticity; /* support_plasticity (engine/mpm_solver.py:62) */
  REAL v_clamp_k; /* dx * g2p2g_allowed_cfl, or 0 (no grid velocity clamp) */
  int quant;      /* quant=True: stored x, v, F rounded to the packed formats */
} FN(Consts);

static void FN(make_consts)(const double *pd, FN(Consts) * c) {
  /* pd layout is documented in mpm_oracle.c (ORACLE_PD_*). */
  c->dx = (REAL)pd[0];
  c->inv_dx = (REAL)pd[1];
  c->p_vol = (REAL)pd[2];
  c->p_mass = (REAL)pd[3];
  c->mu0 = (REAL)pd[4];
  c->la0 = (REAL)pd[5];
  c->alpha = (REAL)pd[6];
  c->water_density = (REAL)pd[7];
  c->gravity[0] = (REAL)pd[8];
  c->gravity[1] = (REAL)pd[9];
  c->gravity[2] = (REAL)pd[10];
  c->stress_scale_k = (REAL)pd[11];
  c->sand_k = (REAL)pd[12];
  c->nu = (REAL)pd[13];
  c->plasticity = pd[14] != 0.0;
  c->v_clamp_k = (REAL)pd[15];
  c->quant = pd[16] != 0.0;
}

/* ------------------------------------------- quantized storage values --- */

/* The values the packed fields of quant=True hold (engine/mpm_solver.py
 * :106-116): x as signed 21-bit fixed point of scale 2^-19 (range [-2, 2)),
 * F as signed 16-bit fixed point of scale 4.1 / 2^15 (F_bound + 0.1), v as
 * block floating point: one exponent for the vector, unit 2^u with
 * u = clamp(k - 18, -100, 27) where max |v_d| lies in [2^(k-1), 2^k), and
 * signed 19-bit mantissas (|m| <= 2^18 - 1; a rounding carry to 2^18 moves
 * to the next unit).  Rounding to nearest, ties away from zero; out-of-range
 * values saturate; non-finite values become 0. */
static REAL FN(q_round)(REAL s) {
  REAL t = s + (s < (REAL)0 ? (REAL)-0.5 : (REAL)0.5);
  if (t >= (REAL)2147483648.0) return (REAL)2147483647.0; /* saturates like the device's int32 conversion */
  if (t <= (REAL)-2147483648.0) return (REAL)-2147483648.0;
  return (REAL)(int64_t)t;
}

static REAL FN(q_x)(REAL x) {
  if (!isfinite(x)) return 0;
  REAL q = FN(q_round)(x * (REAL)524288.0);
  if (q < (REAL)-1048576.0) q = (REAL)-1048576.0;
  if (q > (REAL)1048575.0) q = (REAL)1048575.0;
  return q * (REAL)(1.0 / 524288.0);
}

static REAL FN(q_F)(REAL f) {
  if (!isfinite(f)) return 0;
  REAL q = FN(q_round)(f * (REAL)(32768.0 / 4.1));
  if (q < (REAL)-32768.0) q = (REAL)-32768.0;
  if (q > (REAL)32767.0) q = (REAL)32767.0;
  return q * (REAL)(4.1 / 32768.0);
}

static void FN(q_v)(REAL *v) {
  if (!isfinite(v[0]) || !isfinite(v[1]) || !isfinite(v[2])) {
    v[0] = v[1] = v[2] = 0;
    return;
  }
  REAL M = FABS(v[0]);
  if (FABS(v[1]) > M) M = FABS(v[1]);
  if (FABS(v[2]) > M) M = FABS(v[2]);
  int k = -126;
  if (M > (REAL)0) (void)FREXP(M, &k);
  int u = k - 18;
  if (u < -100) u = -100;
  if (u > 27) u = 27;
  REAL m[3];
  for (int pass = 0; pass < 2; ++pass) {
    REAL big = 0;
    for (int d = 0; d < 3; ++d) {
      m[d] = FN(q_round)(LDEXP(v[d], -u));
      if (FABS(m[d]) > big) big = FABS(m[d]);
    }
    if (big < (REAL)262144.0 || u == 27) break;
    ++u;
  }
  for (int d = 0; d < 3; ++d) {
    if (m[d] > (REAL)262143.0) m[d] = (REAL)262143.0;
    if (m[d] < (REAL)-262143.0) m[d] = (REAL)-262143.0;
    v[d] = LDEXP(m[d], u);
  }
}

/* ---------------------------------------------------------------- SVD --- */

static void FN(jacobi_pair)(REAL S[3][3], REAL V[3][3], int p, int q) {
  REAL apq = S[p][q];
  if (apq == (REAL)0) return;
  REAL theta = (S[q][q] - S[p][p]) / ((REAL)2 * apq);
  REAL t;
  REAL at = FABS(theta);
  if (at > (REAL)1e15) {
    t = (REAL)0.5 / theta;
  } else {
    t = (REAL)1 / (at + SQRT(theta * theta + (REAL)1));
    if (theta < (REAL)0) t = -t;
  }
  REAL c = RSQRT(t * t + (REAL)1);
  REAL s = t * c;
  S[p][p] -= t * apq;
  S[q][q] += t * apq;
  S[p][q] = S[q][p] = (REAL)0;
  int r = 3 - p - q;
  REAL srp = S[r][p], srq = S[r][q];
  S[r][p] = S[p][r] = c * srp - s * srq;
  S[r][q] = S[q][r] = s * srp + c * srq;
  for (int i = 0; i < 3; ++i) {
    REAL vp = V[i][p], vq = V[i][q];
    V[i][p] = c * vp - s * vq;
    V[i][q] = s * vp + c * vq;
  }
}

static void FN(givens_rows)(REAL B[3][3], REAL U[3][3], int i, int j) {
  /* zero B[j][i] using rows i and j; accumulate U = U * G^T */
  REAL a = B[i][i], b = B[j][i];
  REAL r2 = a * a + b * b;
  REAL c = (REAL)1, s = (REAL)0;
  if (r2 > (REAL)0) {
    REAL ir = RSQRT(r2);
    c = a * ir;
    s = b * ir;
  }
  for (int k = 0; k < 3; ++k) {
    REAL bi = B[i][k], bj = B[j][k];
    B[i][k] = c * bi + s * bj;
    B[j][k] = -s * bi + c * bj;
  }
  for (int k = 0; k < 3; ++k) {
    REAL ui = U[k][i], uj = U[k][j];
    U[k][i] = c * ui + s * uj;
    U[k][j] = -s * ui + c * uj;
  }
}

static void FN(swap_cols)(REAL B[3][3], REAL V[3][3], int i, int j) {
  /* swap columns i, j and negate the new column j: keeps det(V) = +1 */
  for (int k = 0; k < 3; ++k) {
    REAL t = B[k][i];
    B[k][i] = B[k][j];
    B[k][j] = -t;
    t = V[k][i];
    V[k][i] = V[k][j];
    V[k][j] = -t;
  }
}

void FN(oracle_svd3)(const REAL *A9, REAL *U9, REAL *s3, REAL *V9) {
  REAL A[3][3], S[3][3], V[3][3], B[3][3], U[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A[i][j] = A9[3 * i + j];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      REAL acc = 0;
      for (int k = 0; k < 3; ++k) acc += A[k][i] * A[k][j];
      S[i][j] = acc;
      V[i][j] = (REAL)(i == j);
      U[i][j] = (REAL)(i == j);
    }
  for (int sweep = 0; sweep < SVD_SWEEPS; ++sweep) {
    FN(jacobi_pair)(S, V, 0, 1);
    FN(jacobi_pair)(S, V, 0, 2);
    FN(jacobi_pair)(S, V, 1, 2);
#if !defined(ORACLE_IS_FLOAT)
    REAL off = S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][2] * S[1][2];
    REAL dia = S[0][0] * S[0][0] + S[1][1] * S[1][1] + S[2][2] * S[2][2];
    if (off <= (REAL)1e-40 * dia) break;
#endif
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      REAL acc = 0;
      for (int k = 0; k < 3; ++k) acc += A[i][k] * V[k][j];
      B[i][j] = acc;
    }
  REAL rho[3];
  for (int j = 0; j < 3; ++j)
    rho[j] = B[0][j] * B[0][j] + B[1][j] * B[1][j] + B[2][j] * B[2][j];
  if (rho[0] < rho[1]) {
    FN(swap_cols)(B, V, 0, 1);
    REAL t = rho[0]; rho[0] = rho[1]; rho[1] = t;
  }
  if (rho[0] < rho[2]) {
    FN(swap_cols)(B, V, 0, 2);
    REAL t = rho[0]; rho[0] = rho[2]; rho[2] = t;
  }
  if (rho[1] < rho[2]) {
    FN(swap_cols)(B, V, 1, 2);
    REAL t = rho[1]; rho[1] = rho[2]; rho[2] = t;
  }
  FN(givens_rows)(B, U, 0, 1);
  FN(givens_rows)(B, U, 0, 2);
  FN(givens_rows)(B, U, 1, 2);
  for (int i = 0; i < 3; ++i) {
    s3[i] = B[i][i];
    for (int j = 0; j < 3; ++j) {
      U9[3 * i + j] = U[i][j];
      V9[3 * i + j] = V[i][j];
    }
  }
}

/* ---------------------------------------------------- per-particle P2G --- */

static inline void FN(matmul3)(const REAL a[3][3], const REAL b[3][3], REAL o[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      o[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
}

/* Base cell of a particle: engine/mpm_solver.py:357,497.  x * inv_dx - 0.5
 * is two separately rounded operations (no contraction). */
static inline void FN(base_cell)(const REAL *xp, REAL inv_dx, int32_t base[3], REAL fx[3]) {
  for (int d = 0; d < 3; ++d) {
    volatile REAL s = xp[d] * inv_dx;
    volatile REAL t = s - (REAL)0.5;
    base[d] = (int32_t)FLOOR(t);
    volatile REAL bf = (REAL)base[d];
    fx[d] = s - bf;
  }
}

static inline void FN(weights)(const REAL fx[3], REAL w[3][3]) {
  /* engine/mpm_solver.py:505 : w[k][d] */
  for (int d = 0; d < 3; ++d) {
    REAL a = (REAL)1.5 - fx[d];
    REAL b = fx[d] - (REAL)1.0;
    REAL c = fx[d] - (REAL)0.5;
    w[0][d] = (REAL)0.5 * (a * a);
    w[1][d] = (REAL)0.75 - b * b;
    w[2][d] = (REAL)0.5 * (c * c);
  }
}

/* engine/mpm_solver.py:321-342 */
static void FN(sand_projection)(REAL sig[3], REAL *Jp, const FN(Consts) * k, REAL mu0, REAL la0) {
  REAL eps[3], out[3] = {1, 1, 1};
  for (int i = 0; i < 3; ++i) {
    REAL a = FABS(sig[i]);
    if (a < (REAL)1e-4) a = (REAL)1e-4;
    eps[i] = LOG(a);
  }
  REAL tr = eps[0] + eps[1] + eps[2] + *Jp;
  REAL eh[3];
  for (int i = 0; i < 3; ++i) eh[i] = eps[i] - tr / (REAL)3;
  REAL ehn = SQRT(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]) + (REAL)1e-20;
  if (tr >= (REAL)0) {
    *Jp = tr;
  } else {
    *Jp = 0;
    (void)mu0;
    (void)la0;
    REAL dg = ehn + k->sand_k * tr * k->alpha;
    REAL dgp = dg > (REAL)0 ? dg : (REAL)0;
    for (int i = 0; i < 3; ++i) out[i] = EXP(eps[i] - dgp / ehn * eh[i]);
  }
  for (int i = 0; i < 3; ++i) sig[i] = out[i];
}

/* One particle's P2G update (engine/mpm_solver.py:495-575): updates F and Jp
 * in place and returns the scatter inputs (mass, momentum m*v, affine). */
/* fused != 0: the constitutive update of the G2P2G substep (:410-476):
 * no water F reset (:508-511), h = exp(10 (1 - Jp)) for every material,
 * water keeps Jp, mass = p_mass for every material.
 * k->plasticity == 0 (support_plasticity=False): the reference has no Jp
 * field; water restarts from F = I (:508-511), h = 1 (:516-518, :419-421),
 * Jp is never updated (:533-534, :541-542) and sand has neither the return
 * map nor a stress (:553-566). */
static void FN(p2g_particle)(const FN(Consts) * k, REAL dt, int mat, REAL Ep,
                             REAL *F9, REAL *Jp, const REAL *C9, REAL *mass_out,
                             REAL affine[3][3], int fused) {
  REAL mu0 = k->mu0, la0 = k->la0;
  if (Ep > (REAL)0) { /* per-particle Young's modulus (extension) */
    mu0 = Ep / ((REAL)2 * ((REAL)1 + k->nu));
    la0 = Ep * k->nu / (((REAL)1 + k->nu) * ((REAL)1 - (REAL)2 * k->nu));
  }
  REAL F[3][3], C[3][3], G[3][3], Fn[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      F[i][j] = F9[3 * i + j];
      C[i][j] = C9[3 * i + j];
    }
  if (!fused && mat == 0) { /* :508-511 */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) F[i][j] = (REAL)(i == j);
    if (k->plasticity) F[0][0] = *Jp;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) G[i][j] = (REAL)(i == j) + dt * C[i][j];
  FN(matmul3)(G, F, Fn); /* :513 */
  if (fused && k->quant) { /* :413-417: clamp to F_bound, stored (rounded) F read back */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        REAL f = Fn[i][j] < (REAL)-4 ? (REAL)-4 : (Fn[i][j] > (REAL)4 ? (REAL)4 : Fn[i][j]);
        Fn[i][j] = FN(q_F)(f);
      }
  }
  REAL h = 1;
  if (k->plasticity && (fused || mat != 0)) h = EXP((REAL)10 * ((REAL)1 - *Jp)); /* :516-518, :427-429 */
  if (mat == 1) h = (REAL)0.3;                         /* :519-521 */
  REAL mu = mu0 * h, la = la0 * h;
  if (mat == 0) mu = 0;
  REAL U9[9], sg[3], V9[9];
  FN(oracle_svd3)(&Fn[0][0], U9, sg, V9); /* :525 */
  REAL U[3][3], V[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      U[i][j] = U9[3 * i + j];
      V[i][j] = V9[3 * i + j];
    }
  REAL J = 1;
  if (mat != 3) { /* :527-536 */
    for (int d = 0; d < 3; ++d) {
      REAL ns = sg[d];
      if (mat == 2) {
        if (ns < (REAL)(1 - 2.5e-2)) ns = (REAL)(1 - 2.5e-2);
        if (ns > (REAL)(1 + 4.5e-3)) ns = (REAL)(1 + 4.5e-3);
      }
      if (k->plasticity) *Jp *= sg[d] / ns;
      sg[d] = ns;
      J *= ns;
    }
  }
  REAL stress[3][3];
  if (mat == 0) { /* :537-542 */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) Fn[i][j] = (REAL)(i == j);
    Fn[0][0] = J;
    if (!fused && k->plasticity) *Jp = J;
  } else if (mat == 2) { /* :543-545 (fused :446-447) */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Fn[i][j] = U[i][0] * sg[0] * V[j][0] + U[i][1] * sg[1] * V[j][1] + U[i][2] * sg[2] * V[j][2];
        if (fused && k->quant) Fn[i][j] = FN(q_F)(Fn[i][j]);
      }
  }
  if (mat != 3) { /* :549-551 */
    REAL R[3][3], D[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) R[i][j] = U[i][0] * V[j][0] + U[i][1] * V[j][1] + U[i][2] * V[j][2];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) D[i][j] = Fn[i][j] - R[i][j];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        REAL acc = D[i][0] * Fn[j][0] + D[i][1] * Fn[j][1] + D[i][2] * Fn[j][2];
        stress[i][j] = (REAL)2 * mu * acc + (i == j ? la * J * (J - (REAL)1) : (REAL)0);
      }
  } else if (!k->plasticity) { /* sand without plasticity: zero stress, F kept */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) stress[i][j] = 0;
  } else { /* :552-566 */
    FN(sand_projection)(sg, Jp, k, mu0, la0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Fn[i][j] = U[i][0] * sg[0] * V[j][0] + U[i][1] * sg[1] * V[j][1] + U[i][2] * sg[2] * V[j][2];
        if (fused && k->quant) Fn[i][j] = FN(q_F)(Fn[i][j]); /* :458 */
      }
    REAL ls = 0, cen[3];
    for (int i = 0; i < 3; ++i) {
      REAL l = LOG(sg[i]);
      ls += l;
      cen[i] = (REAL)2 * mu0 * l * ((REAL)1 / sg[i]);
    }
    for (int i = 0; i < 3; ++i) cen[i] += la0 * ls * ((REAL)1 / sg[i]);
    REAL T[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        T[i][j] = U[i][0] * cen[0] * V[j][0] + U[i][1] * cen[1] * V[j][1] + U[i][2] * cen[2] * V[j][2];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) stress[i][j] = T[i][0] * Fn[j][0] + T[i][1] * Fn[j][1] + T[i][2] * Fn[j][2];
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) F9[3 * i + j] = k->quant ? FN(q_F)(Fn[i][j]) : Fn[i][j]; /* :567 */
  REAL sc = -dt * k->stress_scale_k;                     /* :569 */
  REAL mass = k->p_mass;
  if (!fused && mat == 0) mass *= k->water_density; /* :571-573 */
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) affine[i][j] = sc * stress[i][j] + mass * C[i][j]; /* :574 */
  *mass_out = mass;
}

/* ------------------------------------------------------------ grid ------ */

typedef struct {
  int32_t lo[3]; /* node index of the window origin (reference grid frame) */
  int32_t W[3];  /* window extent in nodes (multiples of 4) */
} FN(Window);

static inline int64_t FN(node_index)(const FN(Window) * w, int i, int j, int k) {
  return ((int64_t)(i - w->lo[0]) * w->W[1] + (j - w->lo[1])) * w->W[2] + (k - w->lo[2]);
}

/* engine/mpm_solver.py:577-584 ; grid arrays m (n) and mv (n*3), AoS mv. */
static int FN(scatter_particle)(const FN(Window) * w, const REAL *xp, const REAL *vp,
                                const FN(Consts) * k, REAL mass, REAL affine[3][3],
                                REAL *gm, REAL *gmv, int atomic) {
  int32_t base[3];
  REAL fx[3], wt[3][3];
  FN(base_cell)(xp, k->inv_dx, base, fx);
  for (int d = 0; d < 3; ++d)
    if (base[d] < w->lo[d] || base[d] + 3 > w->lo[d] + w->W[d]) return 1;
  FN(weights)(fx, wt);
  REAL mvp[3] = {mass * vp[0], mass * vp[1], mass * vp[2]};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      for (int c = 0; c < 3; ++c) {
        REAL dpos[3] = {((REAL)a - fx[0]) * k->dx, ((REAL)b - fx[1]) * k->dx, ((REAL)c - fx[2]) * k->dx};
        REAL weight = (REAL)1 * wt[a][0] * wt[b][1] * wt[c][2];
        int64_t n = FN(node_index)(w, base[0] + a, base[1] + b, base[2] + c);
        for (int d = 0; d < 3; ++d) {
          REAL ad = affine[d][0] * dpos[0] + affine[d][1] * dpos[1] + affine[d][2] * dpos[2];
          REAL val = weight * (mvp[d] + ad);
          if (atomic) {
#pragma omp atomic
            gmv[3 * n + d] += val;
          } else {
            gmv[3 * n + d] += val;
          }
        }
        REAL mm = weight * mass;
        if (atomic) {
#pragma omp atomic
          gm[n] += mm;
        } else {
          gm[n] += mm;
        }
      }
  return 0;
}

/* Grid update for one node: engine/mpm_solver.py:586-598 (normalisation,
 * gravity and the fused mode's velocity clamp), then the grid_postprocess list in order (:794-795): bounding box
 * (:600-616, kind 2), sphere (:618-642, kind 1) and surface (:647-687,
 * kind 0) colliders.  coll: 12 doubles per record, see mpm_oracle.c. */
static void FN(grid_node)(int gi, int gj, int gk, REAL m, REAL *v, REAL dt, const FN(Consts) * k,
                          const int32_t *res, int padding, int unbounded, int grid_size,
                          int ncoll, const double *coll) {
  if (m > (REAL)0) {
    REAL inv = (REAL)1 / m;
    for (int d = 0; d < 3; ++d) v[d] = inv * v[d];
    for (int d = 0; d < 3; ++d) v[d] += dt * k->gravity[d];
  }
  if (k->v_clamp_k > (REAL)0) { /* fused G2P2G mode, :589 and :594-598 */
    REAL va = k->v_clamp_k / dt;
    for (int d = 0; d < 3; ++d) v[d] = v[d] < -va ? -va : (v[d] > va ? va : v[d]);
  }
  int I[3] = {gi, gj, gk};
  (void)unbounded;
  for (int c = 0; c < ncoll; ++c) {
    const double *cd = coll + 12 * c;
    int kind = (int)cd[0], surface = (int)cd[1];
    if (kind == 2) { /* bounding box :600-616; surface field = unbounded flag */
      for (int d = 0; d < 3; ++d) {
        int lo = surface ? -grid_size / 2 + padding : padding;
        int hi = surface ? grid_size / 2 - padding : res[d] - padding;
        if (I[d] < lo && v[d] < 0) v[d] = 0;
        if (I[d] >= hi && v[d] > 0) v[d] = 0;
      }
      continue;
    }
    REAL p[3] = {(REAL)cd[2], (REAL)cd[3], (REAL)cd[4]};
    REAL nrm[3] = {(REAL)cd[5], (REAL)cd[6], (REAL)cd[7]};
    REAL radius = (REAL)cd[8], friction = (REAL)cd[9];
    REAL off[3];
    for (int d = 0; d < 3; ++d) off[d] = (REAL)I[d] * k->dx - p[d];
    if (kind == 0) { /* surface (plane) collider :661-685 */
      REAL dn = off[0] * nrm[0] + off[1] * nrm[1] + off[2] * nrm[2];
      if (dn < 0) {
        if (surface == 0) {
          v[0] = v[1] = v[2] = 0;
        } else {
          REAL nc = nrm[0] * v[0] + nrm[1] * v[1] + nrm[2] * v[2];
          REAL s = surface == 1 ? nc : (nc < 0 ? nc : 0);
          for (int d = 0; d < 3; ++d) v[d] = v[d] - nrm[d] * s;
          REAL vn = SQRT(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
          if (nc < 0 && vn > (REAL)1e-30) {
            REAL mag = vn + nc * friction;
            if (mag < 0) mag = 0;
            REAL inv = (REAL)1 / vn;
            for (int d = 0; d < 3; ++d) v[d] = v[d] * inv * mag;
          }
        }
      }
    } else { /* sphere collider :621-640 */
      REAL r2 = off[0] * off[0] + off[1] * off[1] + off[2] * off[2];
      if (r2 < radius * radius) {
        if (surface == 0) {
          v[0] = v[1] = v[2] = 0;
        } else {
          REAL inv = (REAL)1 / (SQRT(r2) + (REAL)1e-5);
          REAL n3[3] = {off[0] * inv, off[1] * inv, off[2] * inv};
          REAL nc = n3[0] * v[0] + n3[1] * v[1] + n3[2] * v[2];
          REAL s = surface == 1 ? nc : (nc < 0 ? nc : 0);
          for (int d = 0; d < 3; ++d) v[d] = v[d] - n3[d] * s;
        }
      }
    }
  }
}

/* G2P for one particle: engine/mpm_solver.py:701-724 */
static int FN(g2p_particle)(const FN(Window) * w, const FN(Consts) * k, REAL dt, int mat,
                            REAL *xp, REAL *vp, REAL *C9, const REAL *gv, int quant) {
  int32_t base[3];
  REAL fx[3], wt[3][3];
  FN(base_cell)(xp, k->inv_dx, base, fx);
  for (int d = 0; d < 3; ++d)
    if (base[d] < w->lo[d] || base[d] + 3 > w->lo[d] + w->W[d]) return 1;
  FN(weights)(fx, wt);
  REAL nv[3] = {0, 0, 0}, nC[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  REAL s4 = (REAL)4 * k->inv_dx;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      for (int c = 0; c < 3; ++c) {
        REAL dpos[3] = {(REAL)a - fx[0], (REAL)b - fx[1], (REAL)c - fx[2]};
        int64_t n = FN(node_index)(w, base[0] + a, base[1] + b, base[2] + c);
        const REAL *g = gv + 3 * n;
        REAL weight = (REAL)1 * wt[a][0] * wt[b][1] * wt[c][2];
        for (int d = 0; d < 3; ++d) nv[d] += weight * g[d];
        REAL sw = s4 * weight;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) nC[i][j] += sw * (g[i] * dpos[j]);
      }
  if (mat != 4) {
    for (int d = 0; d < 3; ++d) vp[d] = nv[d];
    if (quant) FN(q_v)(vp); /* the advection reads the stored v */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) C9[3 * i + j] = nC[i][j];
    for (int d = 0; d < 3; ++d) xp[d] += dt * vp[d];
    if (quant)
      for (int d = 0; d < 3; ++d) xp[d] = FN(q_x)(xp[d]);
  }
  return 0;
}

/* ------------------------------------------------------- public API ----- */

/* The stored values of quant=True for n particles, in place: x (n*3),
 * v (n*3, one shared exponent per particle) and F (n*9). */
void FN(oracle_quant_values)(int64_t n, REAL *x, REAL *v, REAL *F) {
  for (int64_t p = 0; p < n; ++p) {
    for (int d = 0; d < 3; ++d) x[3 * p + d] = FN(q_x)(x[3 * p + d]);
    FN(q_v)(v + 3 * p);
    for (int a = 0; a < 9; ++a) F[9 * p + a] = FN(q_F)(F[9 * p + a]);
  }
}

/* P2G over all particles into a zeroed dense window grid. Returns the number
 * of particles whose stencil left the window (0 on success). */
int FN(oracle_p2g)(const double *pd, int64_t n, const REAL *x, const REAL *v, const REAL *C,
                   REAL *F, REAL *Jp, const int32_t *mat, const REAL *E_p, REAL dt,
                   const int32_t *lo, const int32_t *W, REAL *gm, REAL *gmv, int nthreads) {
  FN(Consts) k;
  FN(make_consts)(pd, &k);
  FN(Window) w;
  for (int d = 0; d < 3; ++d) {
    w.lo[d] = lo[d];
    w.W[d] = W[d];
  }
  int bad = 0;
  int atomic = nthreads > 1;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(+ : bad) if (atomic)
  for (int64_t p = 0; p < n; ++p) {
    REAL affine[3][3], mass;
    FN(p2g_particle)(&k, dt, mat[p], E_p ? E_p[p] : (REAL)0, F + 9 * p, Jp + p, C + 9 * p, &mass, affine, 0);
    bad += FN(scatter_particle)(&w, x + 3 * p, v + 3 * p, &k, mass, affine, gm, gmv, atomic);
  }
  return bad;
}

/* Grid update over every node of the window: gmv (momentum) becomes velocity
 * in place. Nodes with m == 0 keep their (zero) momentum as velocity. */
void FN(oracle_grid_update)(const double *pd, const int32_t *res, int padding, int unbounded,
                            int grid_size, int ncoll, const double *coll, REAL dt,
                            const int32_t *lo, const int32_t *W, const REAL *gm, REAL *gmv,
                            const uint8_t *node_mask, int nthreads) {
  FN(Consts) k;
  FN(make_consts)(pd, &k);
  int64_t tot = (int64_t)W[0] * W[1] * W[2];
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t n = 0; n < tot; ++n) {
    if (node_mask && !node_mask[n]) continue;
    int i = (int)(n / ((int64_t)W[1] * W[2])) + lo[0];
    int j = (int)((n / W[2]) % W[1]) + lo[1];
    int kk = (int)(n % W[2]) + lo[2];
    FN(grid_node)(i, j, kk, gm[n], gmv + 3 * n, dt, &k, res, padding, unbounded, grid_size, ncoll, coll);
  }
}

int FN(oracle_g2p)(const double *pd, int64_t n, REAL *x, REAL *v, REAL *C, const int32_t *mat,
                   REAL dt, const int32_t *lo, const int32_t *W, const REAL *gv, int nthreads) {
  FN(Consts) k;
  FN(make_consts)(pd, &k);
  FN(Window) w;
  for (int d = 0; d < 3; ++d) {
    w.lo[d] = lo[d];
    w.W[d] = W[d];
  }
  int bad = 0;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(+ : bad)
  for (int64_t p = 0; p < n; ++p)
    bad += FN(g2p_particle)(&w, &k, dt, mat[p], x + 3 * p, v + 3 * p, C + 9 * p, gv, k.quant);
  return bad;
}

/* One G2P2G substep (engine/mpm_solver.py:363-485, step :773-787) on dense
 * window grids: for every particle, G2P from gv_in (node velocities of the
 * previous substep, AoS) at x -- particles p >= first_new keep v with C = 0
 * (:401-404) -- advection unless stationary (:406-408), the fused
 * constitutive update, and P2G at the new x into gm / gmv (zeroed by the
 * caller); then the grid update of every window node (normalisation, gravity,
 * post-process list), leaving the new node velocities in gmv.  Returns the
 * number of particles whose stencil left the window. */
int FN(oracle_g2p2g)(const double *pd, const int32_t *res, int padding, int unbounded, int grid_size, int ncoll,
                     const double *coll, int64_t n, int64_t first_new, REAL *x, REAL *v, REAL *F, REAL *Jp,
                     const int32_t *mat, const REAL *E_p, REAL dt, const int32_t *lo, const int32_t *W,
                     const REAL *gv_in, REAL *gm, REAL *gmv) {
  FN(Consts) k;
  FN(make_consts)(pd, &k);
  FN(Window) w;
  for (int d = 0; d < 3; ++d) {
    w.lo[d] = lo[d];
    w.W[d] = W[d];
  }
  int bad = 0;
  for (int64_t p = 0; p < n; ++p) {
    REAL nv[3] = {v[3 * p], v[3 * p + 1], v[3 * p + 2]};
    REAL C9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (p < first_new) {
      REAL xs[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
      /* the gather of g2p_particle, applied to scratch copies (mat 0 so that
       * it writes v and C; x is advected below) */
      REAL xg[3] = {xs[0], xs[1], xs[2]};
      if (FN(g2p_particle)(&w, &k, (REAL)0, 0, xg, nv, C9, gv_in, 0)) {
        bad += 1;
        continue;
      }
    }
    if (mat[p] != 4) {
      if (k.quant) FN(q_v)(nv); /* :405-408 read the stored v */
      for (int d = 0; d < 3; ++d) {
        v[3 * p + d] = nv[d];
        x[3 * p + d] += dt * v[3 * p + d];
        if (k.quant) x[3 * p + d] = FN(q_x)(x[3 * p + d]);
      }
    }
    REAL affine[3][3], mass;
    FN(p2g_particle)(&k, dt, mat[p], E_p ? E_p[p] : (REAL)0, F + 9 * p, Jp + p, C9, &mass, affine, 1);
    bad += FN(scatter_particle)(&w, x + 3 * p, v + 3 * p, &k, mass, affine, gm, gmv, 0);
  }
  for (int i = 0; i < W[0]; ++i)
    for (int j = 0; j < W[1]; ++j)
      for (int kk = 0; kk < W[2]; ++kk) {
        int64_t nn = ((int64_t)i * W[1] + j) * W[2] + kk;
        FN(grid_node)(lo[0] + i, lo[1] + j, lo[2] + kk, gm[nn], gmv + 3 * nn, dt, &k, res, padding, unbounded,
                      grid_size, ncoll, coll);
      }
  return bad;
}

/* Full substeps with a block-sparse grid (engine/mpm_solver.py:789-797):
 * particles are bucketed by the 4^3 leaf block of their base cell
 * (build_pid, :344-361), P2G runs in parallel over buckets, only blocks
 * touched by a stencil are updated and cleared.  This is the timed CPU
 * baseline; it is numerically the same as p2g/grid_update/g2p above up to
 * float atomic ordering.  Scratch: gm/gmv dense window arrays (zeroed on
 * entry), blkflag (nblocks bytes, zeroed), keys/order/counts scratch. */
int FN(oracle_substeps)(const double *pd, const int32_t *res, int padding, int unbounded,
                        int grid_size, int ncoll, const double *coll, int64_t n, REAL *x,
                        REAL *v, REAL *C, REAL *F, REAL *Jp, const int32_t *mat,
                        const REAL *E_p, REAL dt, int nsub, const int32_t *lo, const int32_t *W,
                        REAL *gm, REAL *gmv, uint8_t *blkflag, int32_t *pkey, int64_t *order,
                        int64_t *bcount, int nthreads, REAL *max_v_out) {
  FN(Consts) k;
  FN(make_consts)(pd, &k);
  FN(Window) w;
  for (int d = 0; d < 3; ++d) {
    w.lo[d] = lo[d];
    w.W[d] = W[d];
  }
  int NB[3] = {W[0] / 4, W[1] / 4, W[2] / 4};
  int64_t nblk = (int64_t)NB[0] * NB[1] * NB[2];
  int bad = 0;
  for (int s = 0; s < nsub; ++s) {
    /* build_pid: bucket by leaf block of the base cell */
    for (int64_t b = 0; b <= nblk; ++b) bcount[b] = 0;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(+ : bad)
    for (int64_t p = 0; p < n; ++p) {
      int32_t base[3];
      REAL fx[3];
      FN(base_cell)(x + 3 * p, k.inv_dx, base, fx);
      int ok = 1;
      for (int d = 0; d < 3; ++d)
        if (base[d] < w.lo[d] || base[d] + 3 > w.lo[d] + w.W[d]) ok = 0;
      if (!ok) {
        pkey[p] = -1;
        bad += 1;
        continue;
      }
      int32_t b0 = (base[0] - w.lo[0]) >> 2, b1 = (base[1] - w.lo[1]) >> 2, b2 = (base[2] - w.lo[2]) >> 2;
      pkey[p] = (int32_t)(((int64_t)b0 * NB[1] + b1) * NB[2] + b2);
    }
    if (bad) return bad;
    for (int64_t p = 0; p < n; ++p) bcount[pkey[p] + 1]++;
    for (int64_t b = 0; b < nblk; ++b) bcount[b + 1] += bcount[b];
    for (int64_t p = 0; p < n; ++p) order[bcount[pkey[p]]++] = p;
    /* bcount[b] is now the end of bucket b; the start is bcount[b-1] */
    /* mark touched blocks (the base block and its +1 neighbours) */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (int64_t b = 0; b < nblk; ++b) {
      int64_t st = b == 0 ? 0 : bcount[b - 1];
      if (bcount[b] == st) continue;
      int b0 = (int)(b / ((int64_t)NB[1] * NB[2])), b1 = (int)((b / NB[2]) % NB[1]), b2 = (int)(b % NB[2]);
      for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c)
          for (int e = 0; e < 2; ++e) {
            int c0 = b0 + a, c1 = b1 + c, c2 = b2 + e;
            if (c0 < NB[0] && c1 < NB[1] && c2 < NB[2]) blkflag[((int64_t)c0 * NB[1] + c1) * NB[2] + c2] = 1;
          }
    }
    /* p2g over buckets */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
    for (int64_t b = 0; b < nblk; ++b) {
      int64_t st = b == 0 ? 0 : bcount[b - 1];
      for (int64_t q = st; q < bcount[b]; ++q) {
        int64_t p = order[q];
        REAL affine[3][3], mass;
        FN(p2g_particle)(&k, dt, mat[p], E_p ? E_p[p] : (REAL)0, F + 9 * p, Jp + p, C + 9 * p, &mass, affine, 0);
        FN(scatter_particle)(&w, x + 3 * p, v + 3 * p, &k, mass, affine, gm, gmv, nthreads > 1);
      }
    }
    /* grid update over touched blocks */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (int64_t b = 0; b < nblk; ++b) {
      if (!blkflag[b]) continue;
      int b0 = (int)(b / ((int64_t)NB[1] * NB[2])), b1 = (int)((b / NB[2]) % NB[1]), b2 = (int)(b % NB[2]);
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 4; ++c)
          for (int e = 0; e < 4; ++e) {
            int i = w.lo[0] + 4 * b0 + a, j = w.lo[1] + 4 * b1 + c, kk = w.lo[2] + 4 * b2 + e;
            int64_t nn = FN(node_index)(&w, i, j, kk);
            FN(grid_node)(i, j, kk, gm[nn], gmv + 3 * nn, dt, &k, res, padding, unbounded, grid_size, ncoll, coll);
          }
    }
    /* g2p */
    REAL mv = 0;
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(max : mv)
    for (int64_t p = 0; p < n; ++p) {
      FN(g2p_particle)(&w, &k, dt, mat[p], x + 3 * p, v + 3 * p, C + 9 * p, gmv, k.quant);
      for (int d = 0; d < 3; ++d) {
        REAL a = FABS(v[3 * p + d]);
        if (a > mv) mv = a;
      }
    }
    if (max_v_out) max_v_out[s] = mv;
    /* clear touched blocks (deactivate_all, :789) */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (int64_t b = 0; b < nblk; ++b) {
      if (!blkflag[b]) continue;
      blkflag[b] = 0;
      int b0 = (int)(b / ((int64_t)NB[1] * NB[2])), b1 = (int)((b / NB[2]) % NB[1]), b2 = (int)(b % NB[2]);
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 4; ++c)
          for (int e = 0; e < 4; ++e) {
            int64_t nn = FN(node_index)(&w, w.lo[0] + 4 * b0 + a, w.lo[1] + 4 * b1 + c, w.lo[2] + 4 * b2 + e);
            gm[nn] = 0;
            gmv[3 * nn] = gmv[3 * nn + 1] = gmv[3 * nn + 2] = 0;
          }
    }
  }
  return bad;
}

#undef RSQRT
#undef SQRT
#undef EXP
#undef LOG
#undef FABS
#undef FLOOR
#undef FREXP
#undef LDEXP
#undef SVD_SWEEPS
#undef FN
