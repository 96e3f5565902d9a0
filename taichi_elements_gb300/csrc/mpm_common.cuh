// Shared device helpers of the MLS-MPM engine: workspace layout, grid window
// addressing, exact binning arithmetic, quadratic B-spline weights and the
// per-particle constitutive update (P2G front half).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_gb300.h"
#include "quant.cuh"
#include "svd3.cuh"

namespace mpm {

constexpr int kBlockCells = 64;  // 4^3 leaf block (engine/mpm_solver.py:159)
constexpr int kTileW = 6;        // block + 2-node halo along each axis
constexpr int kTileN = kTileW * kTileW * kTileW;
constexpr int kFlagTile = 512;   // window blocks per flag-compaction CTA
constexpr int kStatTile = 256;   // particle blocks per stats CTA

// Row indices of the particle state buffer (see include/mpm_gb300.h).
enum Row : int {
  kX = 0, kV = 3, kC = 6, kF = 15, kJp = 24, kMat = 25, kId = 26, kEp = 27
};

// Device pointers into the caller-owned workspace.
struct Ws {
  int32_t *counters;  // [32]: 0 #pblocks, 1 #gblocks, 2 #items, 3 status, 4 #binned, 5-8 work queues,
                      // 16-21 particle bounding box after G2P (order-preserving float keys: min x,y,z, max x,y,z)
  int32_t *blk_flag;  // [nblk]
  int32_t *blk_slot;  // [nblk] window block -> compact particle-block index
  int32_t *pblocks;   // [nblk] compact particle-active blocks (ascending)
  int32_t *gblocks;   // [nblk] compact grid-active blocks (ascending)
  int32_t *flag_tiles;  // [2 * nflagtiles]
  int32_t *pb_count, *pb_start, *pb_lvl, *pb_item;  // [nblk] each
  int32_t *pb_nlev;   // [nblk] levels (largest cell count) of each particle block
  int32_t *pb_tiles;  // [3 * nstattiles]
  unsigned long long *lvl_mask;  // [cap]
  int32_t *lvl_L;                // [cap]
  int2 *items;                   // [cap/32 + nblk + 1]
  int32_t *cellkey, *pid;  // [cap]
  int32_t *inv;            // [cap] sorted slot of the particle at input slot i (pid's inverse)
  int32_t *slot_rank;  // [cap] rank inside its cell of the particle at sorted slot j
  int32_t *stay_rank;  // [cap] next rank of a particle that stays in its cell, else -1
  int32_t *cell_cnt;              // [nblk * 64]
  int32_t *arr_cnt, *arr_rank;    // [nblk * 64] particles without a kept rank: count, next rank
  unsigned long long *leave;      // [nblk * 64] ranks (< 64) of the particles that left the cell
  float4 *grid_mom;               // [nblk * 64] (m, mv)
  float4 *grid_vel;               // [nblk * 64] (v, m)
  int64_t nblk;
  int32_t nflagtiles, nstattiles;
  int64_t items_cap;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Computes the workspace layout; when `base` is null only the size is
// returned.  Pointers are 256-byte aligned.
inline size_t ws_layout(const MpmParams &p, int64_t cap, char *base, Ws *w) {
  const int64_t nblk = (int64_t)p.win_nb[0] * p.win_nb[1] * p.win_nb[2];
  const int32_t nft = (int32_t)((nblk + kFlagTile - 1) / kFlagTile);
  const int32_t nst = (int32_t)((nblk + kStatTile - 1) / kStatTile);
  const int64_t items_cap = cap / 32 + nblk + 1;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes, 256);
    return base ? base + o : nullptr;
  };
  Ws t;
  t.counters = (int32_t *)take(32 * 4);
  t.blk_flag = (int32_t *)take(nblk * 4);
  t.blk_slot = (int32_t *)take(nblk * 4);
  t.pblocks = (int32_t *)take(nblk * 4);
  t.gblocks = (int32_t *)take(nblk * 4);
  t.flag_tiles = (int32_t *)take((size_t)2 * nft * 4);
  t.pb_count = (int32_t *)take(nblk * 4);
  t.pb_start = (int32_t *)take(nblk * 4);
  t.pb_lvl = (int32_t *)take(nblk * 4);
  t.pb_item = (int32_t *)take(nblk * 4);
  t.pb_nlev = (int32_t *)take(nblk * 4);
  t.pb_tiles = (int32_t *)take((size_t)3 * nst * 4);
  t.lvl_mask = (unsigned long long *)take((size_t)cap * 8);
  t.lvl_L = (int32_t *)take((size_t)cap * 4);
  t.items = (int2 *)take((size_t)items_cap * 8);
  t.cellkey = (int32_t *)take((size_t)cap * 4);
  t.pid = (int32_t *)take((size_t)cap * 4);
  t.inv = (int32_t *)take((size_t)cap * 4);
  t.slot_rank = (int32_t *)take((size_t)cap * 4);
  t.stay_rank = (int32_t *)take((size_t)cap * 4);
  t.cell_cnt = (int32_t *)take((size_t)nblk * kBlockCells * 4);
  t.arr_cnt = (int32_t *)take((size_t)nblk * kBlockCells * 4);
  t.arr_rank = (int32_t *)take((size_t)nblk * kBlockCells * 4);
  t.leave = (unsigned long long *)take((size_t)nblk * kBlockCells * 8);
  t.grid_mom = (float4 *)take((size_t)nblk * kBlockCells * 16);
  t.grid_vel = (float4 *)take((size_t)nblk * kBlockCells * 16);
  t.nblk = nblk;
  t.nflagtiles = nft;
  t.nstattiles = nst;
  t.items_cap = items_cap;
  if (w) *w = t;
  return off;
}

// ---------------------------------------------------------------- binning --

// Base cell of a particle, engine/mpm_solver.py:357 and :497:
// floor(x * inv_dx - 0.5) with two separately rounded float32 operations.
// Returns the window-relative base (clamped so the 3^3 stencil stays in the
// window) and fx = x * inv_dx - base (global frame).  Flags are OR-ed into
// *bad (bit 0 out of window, bit 1 non-finite).
struct Base {
  int b[3];     // window-relative base node
  float fx[3];  // fractional offset in cells (reference's fx)
};

__device__ __forceinline__ Base particle_base(const MpmParams &P, float x0, float x1, float x2,
                                              uint32_t &bad) {
  Base r;
  const float xs[3] = {x0, x1, x2};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float s = __fmul_rn(xs[d], P.inv_dx);
    const float t = __fsub_rn(s, 0.5f);
    int g;
    if (isfinite(t)) {
      g = __float2int_rd(t);
    } else {
      bad |= MPM_STATUS_NONFINITE;
      g = P.win_lo[d];
    }
    int rel = g - P.win_lo[d];
    const int hi = P.win_nb[d] * 4 - 3;
    if (rel < 0 || rel > hi) {
      bad |= MPM_STATUS_OUT_OF_GRID;
      rel = rel < 0 ? 0 : hi;
      g = rel + P.win_lo[d];
    }
    r.b[d] = rel;
    r.fx[d] = __fsub_rn(s, (float)g);
  }
  return r;
}

// Bounding-box slots of counters[] and the order-preserving int32 key of a
// float (monotonic: a < b iff key(a) < key(b) for finite values).
constexpr int kBoxMin = 16, kBoxMax = 19;
__device__ __forceinline__ int float_key_i32(float f) {
  const int b = __float_as_int(f);
  return b >= 0 ? b : b ^ 0x7FFFFFFF;
}

__device__ __forceinline__ void set_status(const Ws &w, uint32_t bits) {
  if (bits) atomicOr((unsigned int *)&w.counters[3], bits);
}

__device__ __forceinline__ void block_coords(const MpmParams &P, int64_t b, int &bx, int &by, int &bz) {
  bz = (int)(b % P.win_nb[2]);
  by = (int)((b / P.win_nb[2]) % P.win_nb[1]);
  bx = (int)(b / ((int64_t)P.win_nb[1] * P.win_nb[2]));
}

__device__ __forceinline__ int block_linear(const MpmParams &P, int bx, int by, int bz) {
  return (bx * P.win_nb[1] + by) * P.win_nb[2] + bz;
}

// Cell index inside a 4^3 block, ordered y, x, z.  Eight consecutive cells
// (one quarter-warp of 128-bit shared-memory accesses in rank-major order)
// then cover x in {2k, 2k+1} and z in 0..3, whose 6^3-tile nodes fall in
// eight different 16-byte bank groups (x stride 36 = 4 mod 8).
__device__ __forceinline__ int local_cell(int lx, int ly, int lz) { return (ly * 4 + lx) * 4 + lz; }

// Key of the particle's cell: window block * 64 + cell within the block.
__device__ __forceinline__ int cell_key(const MpmParams &P, const Base &b) {
  const int blin = block_linear(P, b.b[0] >> 2, b.b[1] >> 2, b.b[2] >> 2);
  return blin * kBlockCells + local_cell(b.b[0] & 3, b.b[1] & 3, b.b[2] & 3);
}

// Grid node address (float4 index) of a window-relative node.
__device__ __forceinline__ int64_t node_addr(const MpmParams &P, int gx, int gy, int gz) {
  const int blin = block_linear(P, gx >> 2, gy >> 2, gz >> 2);
  return (int64_t)blin * kBlockCells + (((gx & 3) * 4 + (gy & 3)) * 4 + (gz & 3));
}

// Quadratic B-spline weights, engine/mpm_solver.py:505: w[k][d].
__device__ __forceinline__ void bspline_weights(const float (&fx)[3], float (&w)[3][3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float a = 1.5f - fx[d];
    const float b = fx[d] - 1.0f;
    const float c = fx[d] - 0.5f;
    w[0][d] = 0.5f * (a * a);
    w[1][d] = 0.75f - b * b;
    w[2][d] = 0.5f * (c * c);
  }
}

// -------------------------------------------------------- constitutive ---

struct P2GOut {
  float mass;
  float affine[3][3];
};

// Per-particle P2G update, engine/mpm_solver.py:506-574 with sand_projection
// :321-342.  F and Jp are updated in place.  FUSED selects the variant of the
// fused G2P2G substep (:419-476): no water F reset before the update
// (:508-511), hardening h = exp(10 (1 - Jp)) for every material, water keeps
// its Jp (:537-542 sets only F) and the mass is p_mass for every material.
// P.plasticity == 0 is support_plasticity=False: the reference then has no Jp
// field, so water restarts from F = I (:508-511), h = 1 (:516-518), Jp is
// never updated (:533-534, :541-542) and sand carries no stress and keeps
// (I + dt C) F (:553-566 are skipped).
// FUSED with Q (quant=True) follows the fused kernel's reads of the packed
// field: (I + dt C) F is clamped to +-F_bound = 4 (:415-416) and rounded to
// the 16-bit fixed-point grid before the SVD, and the F rebuilt for snow and
// sand is rounded before the stress reads it (:446-447, :458-469).  The
// unfused P2G keeps its local F for the stress and rounds only on store.
template <bool FUSED = false, bool Q = false>
__device__ __forceinline__ P2GOut constitutive(const MpmParams &P, float dt, int mat, float Ep,
                                               float (&F)[3][3], float &Jp, const float (&C)[3][3]) {
  float mu0 = P.mu0, la0 = P.la0;
  if (Ep > 0.0f) {
    mu0 = Ep / (2.0f * (1.0f + P.nu));
    la0 = Ep * P.nu / ((1.0f + P.nu) * (1.0f - 2.0f * P.nu));
  }
  if (!FUSED && mat == 0) {  // :508-511
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] = (i == j) ? 1.0f : 0.0f;
    F[0][0] = P.plasticity ? Jp : 1.0f;
  }
  float Fn[3][3];  // (I + dt C) F, :513
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float acc = F[i][j];
      acc = fmaf(dt * C[i][0], F[0][j], acc);
      acc = fmaf(dt * C[i][1], F[1][j], acc);
      acc = fmaf(dt * C[i][2], F[2][j], acc);
      Fn[i][j] = acc;
    }
  if (FUSED && Q) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Fn[i][j] = q_fixed_F(fminf(fmaxf(Fn[i][j], -4.0f), 4.0f));
  }
  float h = 1.0f;
  if (P.plasticity && (FUSED || mat != 0)) h = expf(10.0f * (1.0f - Jp));  // :516-518 (:427-429)
  if (mat == 1) h = 0.3f;                       // :519-521
  float mu = mu0 * h;
  const float la = la0 * h;
  if (mat == 0) mu = 0.0f;

  float stress[3][3];
  if (mat == 0) {
    // Water needs only J = s0*s1*s2 = det(Fn) (:527-542): mu = 0 and the
    // rotation factors cancel, so the SVD is skipped.
    const float J = Fn[0][0] * (Fn[1][1] * Fn[2][2] - Fn[1][2] * Fn[2][1]) -
                    Fn[0][1] * (Fn[1][0] * Fn[2][2] - Fn[1][2] * Fn[2][0]) +
                    Fn[0][2] * (Fn[1][0] * Fn[2][1] - Fn[1][1] * Fn[2][0]);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        Fn[i][j] = (i == j) ? 1.0f : 0.0f;
        stress[i][j] = (i == j) ? la * J * (J - 1.0f) : 0.0f;
      }
    Fn[0][0] = J;
    if (!FUSED && P.plasticity) Jp = J;
  } else if (mat == 3 && !P.plasticity) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) stress[i][j] = 0.0f;
  } else {
    if (mat == 1 || mat == 4 || mat == 2) {
      // Elastic and stationary particles never clamp sigma (:527-536), and a
      // snow particle whose singular values all lie inside the clamp range
      // [1 - 2.5e-2, 1 + 4.5e-3] is not clamped either (Jp *= s/s = 1, F is
      // reconstructed unchanged).  Then J = s0*s1*s2 = det(Fn) and the
      // corotated stress needs only the rotation R = U V^T, which for
      // det Fn > 0 is the polar factor.  The singular values are the
      // eigenvalues of the symmetric stretch S = R^T Fn; the snow test checks
      // that every Gershgorin disc of S lies inside the clamp range.
      // Inverted, extremely stretched or clamped particles take the SVD below,
      // which keeps the reference's rotation-only convention for det Fn < 0.
      const float J = Fn[0][0] * (Fn[1][1] * Fn[2][2] - Fn[1][2] * Fn[2][1]) -
                      Fn[0][1] * (Fn[1][0] * Fn[2][2] - Fn[1][2] * Fn[2][0]) +
                      Fn[0][2] * (Fn[1][0] * Fn[2][1] - Fn[1][1] * Fn[2][0]);
      float R[3][3];
      bool ok = J > 0.0f && polar_rotation<6>(Fn, R);
      if (ok && mat == 2) {
        float S[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) S[i][j] = R[0][i] * Fn[0][j] + R[1][i] * Fn[1][j] + R[2][i] * Fn[2][j];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          float rad = 0.0f;
#pragma unroll
          for (int j = 0; j < 3; ++j)
            if (j != i) rad += 0.5f * (fabsf(S[i][j]) + fabsf(S[j][i]));
          // margin of 4e-7 covers the float32 error of S
          ok = ok && (S[i][i] - rad - 4e-7f >= 1.0f - 2.5e-2f) && (S[i][i] + rad + 4e-7f <= 1.0f + 4.5e-3f);
        }
      }
      if (ok) {
        const float lj = la * J * (J - 1.0f);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const float acc = (Fn[i][0] - R[i][0]) * Fn[j][0] + (Fn[i][1] - R[i][1]) * Fn[j][1] +
                              (Fn[i][2] - R[i][2]) * Fn[j][2];
            stress[i][j] = 2.0f * mu * acc + ((i == j) ? lj : 0.0f);
          }
        goto done;
      }
    }
    float U[3][3], sg[3], V[3][3];
    svd3<4>(Fn, U, sg, V);
    if (mat != 3) {
      float J = 1.0f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float ns = sg[d];
        if (mat == 2) ns = fminf(fmaxf(ns, 1.0f - 2.5e-2f), 1.0f + 4.5e-3f);  // :530-532
        if (P.plasticity) Jp *= sg[d] / ns;                                       // :534
        sg[d] = ns;
        J *= ns;
      }
      if (mat == 2) {  // :543-545
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            Fn[i][j] = U[i][0] * sg[0] * V[j][0] + U[i][1] * sg[1] * V[j][1] + U[i][2] * sg[2] * V[j][2];
            if (FUSED && Q) Fn[i][j] = q_fixed_F(Fn[i][j]);
          }
      }
      // :549-551  stress = 2 mu (F - U V^T) F^T + la J (J-1) I
      float D[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          D[i][j] = Fn[i][j] - (U[i][0] * V[j][0] + U[i][1] * V[j][1] + U[i][2] * V[j][2]);
      const float lj = la * J * (J - 1.0f);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float acc = D[i][0] * Fn[j][0] + D[i][1] * Fn[j][1] + D[i][2] * Fn[j][2];
          stress[i][j] = 2.0f * mu * acc + ((i == j) ? lj : 0.0f);
        }
    } else {
      // sand_projection, :321-342
      float eps[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) eps[i] = logf(fmaxf(fabsf(sg[i]), 1e-4f));
      const float tr = eps[0] + eps[1] + eps[2] + Jp;
      float eh[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) eh[i] = eps[i] - tr / 3.0f;
      const float ehn = sqrtf(eh[0] * eh[0] + eh[1] * eh[1] + eh[2] * eh[2]) + 1e-20f;
      if (tr >= 0.0f) {
        Jp = tr;
        sg[0] = sg[1] = sg[2] = 1.0f;
      } else {
        Jp = 0.0f;
        const float dg = ehn + P.sand_k * tr * P.alpha;
        const float dgp = fmaxf(dg, 0.0f);
#pragma unroll
        for (int i = 0; i < 3; ++i) sg[i] = expf(eps[i] - dgp / ehn * eh[i]);
      }
      // :555-566
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          Fn[i][j] = U[i][0] * sg[0] * V[j][0] + U[i][1] * sg[1] * V[j][1] + U[i][2] * sg[2] * V[j][2];
          if (FUSED && Q) Fn[i][j] = q_fixed_F(Fn[i][j]);
        }
      float ls = 0.0f, cen[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float l = logf(sg[i]);
        ls += l;
        cen[i] = 2.0f * mu0 * l * (1.0f / sg[i]);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) cen[i] += la0 * ls * (1.0f / sg[i]);
      float T[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          T[i][j] = U[i][0] * cen[0] * V[j][0] + U[i][1] * cen[1] * V[j][1] + U[i][2] * cen[2] * V[j][2];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          stress[i][j] = T[i][0] * Fn[j][0] + T[i][1] * Fn[j][1] + T[i][2] * Fn[j][2];
    }
  }
done:
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) F[i][j] = Fn[i][j];
  P2GOut o;
  const float sc = -dt * P.stress_k;  // :569
  o.mass = P.p_mass;
  if (!FUSED && mat == 0) o.mass *= P.water_density;  // :571-573
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) o.affine[i][j] = fmaf(sc, stress[i][j], o.mass * C[i][j]);  // :574
  return o;
}

// One grid post-process record applied to a node velocity (the reference's
// grid_postprocess list, engine/mpm_solver.py:794-795): bounding box
// (:600-616), surface collider (:647-687) or sphere collider (:618-642).  I is
// the node's index in the reference grid frame.
__device__ __forceinline__ void postprocess_op(const MpmParams &P, const MpmCollider &cl, const int (&I)[3],
                                               float (&v)[3]) {
  if (cl.kind == 2) {  // bounding box, :600-616
    const bool unb = cl.surface != 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int lo = unb ? -P.grid_size / 2 + P.padding : P.padding;
      const int hi = unb ? P.grid_size / 2 - P.padding : P.res[d] - P.padding;
      if (I[d] < lo && v[d] < 0.0f) v[d] = 0.0f;
      if (I[d] >= hi && v[d] > 0.0f) v[d] = 0.0f;
    }
    return;
  }
  float off[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) off[d] = (float)I[d] * P.dx - cl.point[d];
  if (cl.kind == 0) {
    const float dn = off[0] * cl.normal[0] + off[1] * cl.normal[1] + off[2] * cl.normal[2];
    if (dn < 0.0f) {
      if (cl.surface == 0) {
        v[0] = v[1] = v[2] = 0.0f;
      } else {
        const float nc = cl.normal[0] * v[0] + cl.normal[1] * v[1] + cl.normal[2] * v[2];
        const float s = cl.surface == 1 ? nc : fminf(nc, 0.0f);
#pragma unroll
        for (int d = 0; d < 3; ++d) v[d] = v[d] - cl.normal[d] * s;
        const float vn = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (nc < 0.0f && vn > 1e-30f) {
          const float mag = fmaxf(0.0f, vn + nc * cl.friction);
          const float inv = 1.0f / vn;
#pragma unroll
          for (int d = 0; d < 3; ++d) v[d] = v[d] * inv * mag;
        }
      }
    }
  } else {
    const float r2 = off[0] * off[0] + off[1] * off[1] + off[2] * off[2];
    if (r2 < cl.radius * cl.radius) {
      if (cl.surface == 0) {
        v[0] = v[1] = v[2] = 0.0f;
      } else {
        const float inv = 1.0f / (sqrtf(r2) + 1e-5f);
        const float n3[3] = {off[0] * inv, off[1] * inv, off[2] * inv};
        const float nc = n3[0] * v[0] + n3[1] * v[1] + n3[2] * v[2];
        const float s = cl.surface == 1 ? nc : fminf(nc, 0.0f);
#pragma unroll
        for (int d = 0; d < 3; ++d) v[d] = v[d] - n3[d] * s;
      }
    }
  }
}

// Grid node update, engine/mpm_solver.py:586-598 (momentum to velocity,
// gravity and, in the fused G2P2G mode, the per-component velocity clamp to
// dx * cfl / dt) followed by the post-process list in order.
__device__ __forceinline__ float3 grid_node_update(const MpmParams &P, const int (&I)[3], float m,
                                                   float3 mv, float dt) {
  float v[3] = {mv.x, mv.y, mv.z};
  if (m > 0.0f) {
    const float inv = 1.0f / m;
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = inv * v[d] + dt * P.gravity[d];
  }
  if (P.v_clamp_k > 0.0f) {  // :594-598
    const float va = P.v_clamp_k / dt;
#pragma unroll
    for (int d = 0; d < 3; ++d) v[d] = fminf(fmaxf(v[d], -va), va);
  }
  for (int c = 0; c < P.n_colliders; ++c) postprocess_op(P, P.colliders[c], I, v);
  return make_float3(v[0], v[1], v[2]);
}

}  // namespace mpm
