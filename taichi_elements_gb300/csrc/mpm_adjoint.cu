// Hand-written adjoint of one MLS-MPM substep (water and elastic materials)
// for gradients of a loss on a final state through whole rollouts.  The
// reference (taichi-dev/taichi_elements) has no autodiff; the forward pass it
// differentiates is the substep of engine/mpm_solver.py:487-724 as restated
// by mpm_kernels.cu.
//
// Per substep t, in reverse order, given the workspace of the forward
// substep t (its binning and sorted order, the grid momentum snapshot `keep`
// taken before the grid update, and the grid velocity) and the particle state
// `cur` before the substep:
//   k_g2p_adj   reverse of G2P (:694-724): particle gradients of x', v', C'
//               give grid-velocity gradients (scattered through per-warp
//               shared-memory tiles, like P2G) and the weight / position part
//               of dL/dx.
//   k_grid_adj  reverse of the grid update: post-process records replayed and
//               transposed (box and collider projections, surface friction),
//               then v = mv/m + dt g.
//   k_p2g_adj   reverse of P2G (:487-584): grid gradients gathered at the
//               particle, the constitutive update recomputed and reversed
//               (stress, det, polar rotation R of F = R S through
//               (tr(S) I - S)^-1 acting on axial(R^T dR), or through the
//               SVD with clamped 1/(s_i + s_j) terms where S is not positive
//               definite, (I + dt C) F), giving dL/d(x, v, C, F,
//               Jp) of substep t and accumulating dL/dE per particle.
// Gradient buffers are indexed by original particle id, so the sorted orders
// of the forward and of the recomputation need not agree.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_common.cuh"

namespace mpm {

// rows of a gradient buffer (float32, row stride = cap): dL/d(x, v, C, F,
// Jp, per-particle E) of one particle state
enum GRow : int { gX = 0, gV = 3, gC = 6, gF = 15, gJp = 24, gE = 25 };

constexpr int kAdjThreads = 128;
constexpr int kAdjWarps = kAdjThreads / 32;

__device__ __forceinline__ void bspline_dweights(const float (&fx)[3], float (&dw)[3][3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    dw[0][d] = fx[d] - 1.5f;           // d/dfx 0.5 (1.5 - fx)^2
    dw[1][d] = -2.0f * (fx[d] - 1.0f);  // d/dfx 0.75 - (fx - 1)^2
    dw[2][d] = fx[d] - 0.5f;            // d/dfx 0.5 (fx - 0.5)^2
  }
}

__device__ __forceinline__ void cofactor(const float (&A)[3][3], float (&Cf)[3][3]) {
  Cf[0][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
  Cf[0][1] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  Cf[0][2] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  Cf[1][0] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
  Cf[1][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
  Cf[1][2] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
  Cf[2][0] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  Cf[2][1] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
  Cf[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
}

// Transpose of one post-process record at velocity v (the record's input).
__device__ __forceinline__ void postprocess_op_adj(const MpmParams &P, const MpmCollider &cl, const int (&I)[3],
                                                   const float (&v)[3], float (&G)[3]) {
  if (cl.kind == 2) {
    const bool unb = cl.surface != 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int lo = unb ? -P.grid_size / 2 + P.padding : P.padding;
      const int hi = unb ? P.grid_size / 2 - P.padding : P.res[d] - P.padding;
      if ((I[d] < lo && v[d] < 0.0f) || (I[d] >= hi && v[d] > 0.0f)) G[d] = 0.0f;
    }
    return;
  }
  float off[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) off[d] = (float)I[d] * P.dx - cl.point[d];
  if (cl.kind == 0) {
    const float *n = cl.normal;
    const float dn = off[0] * n[0] + off[1] * n[1] + off[2] * n[2];
    if (dn >= 0.0f) return;
    if (cl.surface == 0) {
      G[0] = G[1] = G[2] = 0.0f;
      return;
    }
    const float nc = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
    const bool proj = cl.surface == 1 || nc < 0.0f;
    const float s = proj ? nc : 0.0f;
    float u[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) u[d] = v[d] - n[d] * s;
    const float su = sqrtf(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    float Gu[3] = {G[0], G[1], G[2]};
    float gnc = 0.0f;
    if (nc < 0.0f && su > 1e-30f) {  // friction: out = u / |u| * max(0, |u| + nc f)
      const float k = fmaxf(0.0f, su + nc * cl.friction);
      const float inv = 1.0f / su;
      const float uh[3] = {u[0] * inv, u[1] * inv, u[2] * inv};
      const float uhG = uh[0] * G[0] + uh[1] * G[1] + uh[2] * G[2];
#pragma unroll
      for (int d = 0; d < 3; ++d) Gu[d] = k * inv * (G[d] - uh[d] * uhG) + (k > 0.0f ? uhG * uh[d] : 0.0f);
      gnc = k > 0.0f ? cl.friction * uhG : 0.0f;
    }
    const float nGu = n[0] * Gu[0] + n[1] * Gu[1] + n[2] * Gu[2];
    const float coef = (proj ? -nGu : 0.0f) + gnc;
#pragma unroll
    for (int d = 0; d < 3; ++d) G[d] = Gu[d] + n[d] * coef;
  } else {
    const float r2 = off[0] * off[0] + off[1] * off[1] + off[2] * off[2];
    if (r2 >= cl.radius * cl.radius) return;
    if (cl.surface == 0) {
      G[0] = G[1] = G[2] = 0.0f;
      return;
    }
    const float inv = 1.0f / (sqrtf(r2) + 1e-5f);
    const float n3[3] = {off[0] * inv, off[1] * inv, off[2] * inv};
    const float nc = n3[0] * v[0] + n3[1] * v[1] + n3[2] * v[2];
    if (cl.surface == 1 || nc < 0.0f) {
      const float nG = n3[0] * G[0] + n3[1] * G[1] + n3[2] * G[2];
#pragma unroll
      for (int d = 0; d < 3; ++d) G[d] -= n3[d] * nG;
    }
  }
}

// ------------------------------------------------------------ snapshot ----

__global__ __launch_bounds__(256) void k_grid_snapshot(const MpmParams P, const Ws w, float4 *__restrict__ keep) {
  const int ng = w.counters[1];
  const int64_t total = (int64_t)ng * kBlockCells;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t addr = (int64_t)w.gblocks[t >> 6] * kBlockCells + (t & 63);
    keep[addr] = w.grid_mom[addr];
  }
}

// ------------------------------------------------------------- G2P adj ----

// One pass of the G2P-adjoint stencil of a warp's particles over the 27
// nodes: every lane adds w (Gvt + s4 GC (off - fx)) into its warp tile (the
// store is predicated on `mine`, the lanes of this pass hold distinct
// cells); with GATHER (first pass) it also accumulates dL/dfx from the grid
// velocities `vt` through the weights and through (off - fx).
template <bool GATHER>
__device__ __forceinline__ void g2p_adj_nodes(float4 *tile, const float4 *vt, int base_node, bool mine,
                                              const float (&wt)[3][3], const float (&dw)[3][3], const float (&fx)[3],
                                              const float (&Gvt)[3], const float (&GC)[3][3], float s4,
                                              float (&gfx)[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int node = base_node + (a * kTileW + bb) * kTileW + c;
        const float d[3] = {(float)a - fx[0], (float)bb - fx[1], (float)c - fx[2]};
        const float wgt = wt[a][0] * wt[bb][1] * wt[c][2];
        float q[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) q[r] = Gvt[r] + s4 * (GC[r][0] * d[0] + GC[r][1] * d[1] + GC[r][2] * d[2]);
        // unconditional read and arithmetic, predicated store only
        float4 *nd = tile + node;
        float4 g = *nd;
        g.x += wgt * q[0];
        g.y += wgt * q[1];
        g.z += wgt * q[2];
        if (mine) *nd = g;
        __syncwarp();
        if constexpr (GATHER) {
          const float4 v4 = vt[node];
          const float gw = v4.x * q[0] + v4.y * q[1] + v4.z * q[2];
          gfx[0] += gw * dw[a][0] * wt[bb][1] * wt[c][2];
          gfx[1] += gw * wt[a][0] * dw[bb][1] * wt[c][2];
          gfx[2] += gw * wt[a][0] * wt[bb][1] * dw[c][2];
#pragma unroll
          for (int cc = 0; cc < 3; ++cc)
            gfx[cc] -= s4 * wgt * (GC[0][cc] * v4.x + GC[1][cc] * v4.y + GC[2][cc] * v4.z);
        }
      }
}

// Gradient indexing: with BY_ID, gradient columns are original particle ids;
// otherwise `gin` is in the order of the sorted substep output (column j)
// and `gout` in the order of the substep input `cur` (column pid[j]).  The
// position part of dL/dx from G2P goes to `gmid` (3 rows, column j) and is
// added into `gout` by k_p2g_adj.
template <bool BY_ID>
__global__ __launch_bounds__(kAdjThreads, 4) void k_g2p_adj(const MpmParams P, const Ws w, const float *__restrict__ cur,
                                                         int64_t cap, float dt, const float *__restrict__ gin,
                                                         float *__restrict__ gmid, float4 *__restrict__ ggrid) {
  __shared__ float4 vt[kTileN];
  __shared__ float4 tiles[kAdjWarps][kTileN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4 *tile = tiles[warp];
  const int nitems = (int)min((int64_t)w.counters[2], w.items_cap);
  const float s4 = 4.0f * P.inv_dx;
  uint32_t bad = 0;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int2 item = w.items[it];
    const int k = item.x, start = item.y;
    const int end = (int)min((int64_t)min(start + P.chunk, w.pb_start[k] + w.pb_count[k]), cap);
    int bx, by, bz;
    block_coords(P, w.pblocks[k], bx, by, bz);
    for (int t = threadIdx.x; t < kTileN; t += blockDim.x) {
      const int tx = t / 36, ty = (t / 6) % 6, tz = t % 6;
      const int gx = bx * 4 + tx, gy = by * 4 + ty, gz = bz * 4 + tz;
      float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gx < P.win_nb[0] * 4 && gy < P.win_nb[1] * 4 && gz < P.win_nb[2] * 4)
        g = w.grid_vel[node_addr(P, gx, gy, gz)];
      vt[t] = g;
    }
    for (int t = lane; t < kTileN; t += 32) tile[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    for (int j0 = start + warp * 32; j0 < end; j0 += kAdjThreads) {
      const int j = j0 + lane;
      bool active = j < end;
      int cell = -1 - lane;
      int lx = 0, ly = 0, lz = 0;
      float wt[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      float dw[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      float fx[3] = {0.f, 0.f, 0.f}, Gvt[3] = {0.f, 0.f, 0.f}, Gx[3] = {0.f, 0.f, 0.f}, GC[3][3];
#pragma unroll
      for (int a = 0; a < 9; ++a) GC[a / 3][a % 3] = 0.0f;
      const int64_t i = active ? (int64_t)w.pid[j] : 0;
      if (active && (i < 0 || i >= cap)) {
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        active = false;
      }
      const int64_t gi = !active ? 0 : BY_ID ? (int64_t)__float_as_int(cur[kId * cap + i]) : (int64_t)j;
      if (active && (gi < 0 || gi >= cap)) {  // corrupted id row
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        active = false;
      }
      if (active) {
        const int mat = __float_as_int(cur[kMat * cap + i]) & 0xFF;
#pragma unroll
        for (int d = 0; d < 3; ++d) Gx[d] = gin[(gX + d) * cap + gi];
        if (mat == 4) {  // stationary: x' = x, v' = v, C' = C
#pragma unroll
          for (int d = 0; d < 3; ++d) gmid[d * cap + j] = Gx[d];
          active = false;
        } else {
          const Base b = particle_base(P, cur[kX * cap + i], cur[(kX + 1) * cap + i], cur[(kX + 2) * cap + i], bad);
          lx = b.b[0] - bx * 4;
          ly = b.b[1] - by * 4;
          lz = b.b[2] - bz * 4;
          if ((unsigned)lx > 3u || (unsigned)ly > 3u || (unsigned)lz > 3u) {
            bad |= MPM_STATUS_TABLE_OVERFLOW;
            active = false;
            lx = ly = lz = 0;
          } else {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              fx[d] = b.fx[d];
              Gvt[d] = gin[(gV + d) * cap + gi] + dt * Gx[d];  // x' = x + dt v'
            }
#pragma unroll
            for (int a = 0; a < 9; ++a) GC[a / 3][a % 3] = gin[(gC + a) * cap + gi];
            bspline_weights(b.fx, wt);
            bspline_dweights(b.fx, dw);
            cell = local_cell(lx, ly, lz);
          }
        }
      }
      // grid-velocity gradients g(v_i) += w (Gvt + s4 GC (off - fx)), one
      // pass per set of lanes with distinct cells; the first pass also
      // gathers dL/dfx
      const unsigned peers = __match_any_sync(0xffffffffu, cell);
      const int round_of_lane = __popc(peers & ((1u << lane) - 1u));
      const int base_node = (lx * kTileW + ly) * kTileW + lz;
      float gfx[3] = {0.f, 0.f, 0.f};
      g2p_adj_nodes<true>(tile, vt, base_node, active && round_of_lane == 0, wt, dw, fx, Gvt, GC, s4, gfx);
      if (active) {
#pragma unroll
        for (int d = 0; d < 3; ++d) gmid[d * cap + j] = Gx[d] + P.inv_dx * gfx[d];
      }
      for (int round = 1; __any_sync(0xffffffffu, active && round_of_lane >= round); ++round)
        g2p_adj_nodes<false>(tile, vt, base_node, active && round_of_lane == round, wt, dw, fx, Gvt, GC, s4, gfx);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kTileN; t += blockDim.x) {
      float4 g = tiles[0][t];
#pragma unroll
      for (int q = 1; q < kAdjWarps; ++q) {
        g.x += tiles[q][t].x;
        g.y += tiles[q][t].y;
        g.z += tiles[q][t].z;
      }
      if (g.x != 0.0f || g.y != 0.0f || g.z != 0.0f) {
        const int tx = t / 36, ty = (t / 6) % 6, tz = t % 6;
        const int gx = bx * 4 + tx, gy = by * 4 + ty, gz = bz * 4 + tz;
        if (gx < P.win_nb[0] * 4 && gy < P.win_nb[1] * 4 && gz < P.win_nb[2] * 4)
          atomicAdd(&ggrid[node_addr(P, gx, gy, gz)], make_float4(g.x, g.y, g.z, 0.0f));
      }
    }
    __syncthreads();
  }
  set_status(w, bad);
}

// ------------------------------------------------------------ grid adj ----

__global__ __launch_bounds__(256) void k_grid_adj(const MpmParams P, const Ws w, const float4 *__restrict__ keep,
                                                  float4 *__restrict__ ggrid, float dt) {
  const int ng = w.counters[1];
  const int64_t total = (int64_t)ng * kBlockCells;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int blin = w.gblocks[t >> 6];
    const int l = (int)(t & 63);
    const int64_t addr = (int64_t)blin * kBlockCells + l;
    const float4 gv4 = ggrid[addr];
    const float4 mm = keep[addr];
    int bx, by, bz;
    block_coords(P, blin, bx, by, bz);
    const int I[3] = {P.win_lo[0] + bx * 4 + (l >> 4), P.win_lo[1] + by * 4 + ((l >> 2) & 3),
                      P.win_lo[2] + bz * 4 + (l & 3)};
    const float m = mm.x;
    const float inv = m > 0.0f ? 1.0f / m : 0.0f;
    float v0[3] = {mm.y, mm.z, mm.w};
    if (m > 0.0f) {
#pragma unroll
      for (int d = 0; d < 3; ++d) v0[d] = inv * v0[d] + dt * P.gravity[d];
    }
    float G[3] = {gv4.x, gv4.y, gv4.z};
    // reverse the post-process list; each record's input is recomputed by
    // replaying the records before it
    for (int c = P.n_colliders - 1; c >= 0; --c) {
      float vin[3] = {v0[0], v0[1], v0[2]};
      for (int q = 0; q < c; ++q) postprocess_op(P, P.colliders[q], I, vin);
      postprocess_op_adj(P, P.colliders[c], I, vin, G);
    }
    float4 out;
    if (m > 0.0f) {  // v0 = mv / m + dt g
      out.y = G[0] * inv;
      out.z = G[1] * inv;
      out.w = G[2] * inv;
      out.x = -(G[0] * mm.y + G[1] * mm.z + G[2] * mm.w) * inv * inv;
    } else {
      out = make_float4(0.0f, G[0], G[1], G[2]);
    }
    ggrid[addr] = out;
  }
}

// ------------------------------------------------------------- P2G adj ----

template <bool BY_ID>
__global__ __launch_bounds__(kAdjThreads, 4) void k_p2g_adj(const MpmParams P, const Ws w, const float *__restrict__ cur,
                                                         int64_t cap, float dt, const float *__restrict__ gin,
                                                         const float *__restrict__ gmid, float *__restrict__ gout,
                                                         const float4 *__restrict__ ggrid) {
  __shared__ float4 gt[kTileN];
  const int nitems = (int)min((int64_t)w.counters[2], w.items_cap);
  uint32_t bad = 0;
  const float sc = -dt * P.stress_k;
  const float dmu0 = 1.0f / (2.0f * (1.0f + P.nu));
  const float dla0 = P.nu / ((1.0f + P.nu) * (1.0f - 2.0f * P.nu));
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int2 item = w.items[it];
    const int k = item.x, start = item.y;
    const int end = (int)min((int64_t)min(start + P.chunk, w.pb_start[k] + w.pb_count[k]), cap);
    int bx, by, bz;
    block_coords(P, w.pblocks[k], bx, by, bz);
    for (int t = threadIdx.x; t < kTileN; t += blockDim.x) {
      const int tx = t / 36, ty = (t / 6) % 6, tz = t % 6;
      const int gx = bx * 4 + tx, gy = by * 4 + ty, gz = bz * 4 + tz;
      float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
      if (gx < P.win_nb[0] * 4 && gy < P.win_nb[1] * 4 && gz < P.win_nb[2] * 4)
        g = ggrid[node_addr(P, gx, gy, gz)];
      gt[t] = g;
    }
    __syncthreads();
    for (int j = start + threadIdx.x; j < end; j += blockDim.x) {
      const int64_t i = w.pid[j];
      if (i < 0 || i >= cap) {
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        continue;
      }
      const float *src = cur + i;
      const int64_t id = __float_as_int(src[kId * cap]);
      const int mat = __float_as_int(src[kMat * cap]) & 0xFF;
      if (mat != 0 && mat != 1) {  // the adjoint covers water and elastic only
        bad |= MPM_STATUS_UNSUPPORTED;
        continue;
      }
      if (BY_ID && (id < 0 || id >= cap)) {
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        continue;
      }
      const int64_t gi = BY_ID ? id : (int64_t)j;  // column of gin
      const int64_t go = BY_ID ? id : i;           // column of gout
      float x[3], v[3], C[3][3], F[3][3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        x[d] = src[(kX + d) * cap];
        v[d] = src[(kV + d) * cap];
      }
#pragma unroll
      for (int a = 0; a < 9; ++a) {
        C[a / 3][a % 3] = src[(kC + a) * cap];
        F[a / 3][a % 3] = src[(kF + a) * cap];
      }
      const float Jp = src[kJp * cap];
      const float Ep = P.has_Ep ? src[kEp * cap] : 0.0f;
      const Base b = particle_base(P, x[0], x[1], x[2], bad);
      const int lx = b.b[0] - bx * 4, ly = b.b[1] - by * 4, lz = b.b[2] - bz * 4;
      if ((unsigned)lx > 3u || (unsigned)ly > 3u || (unsigned)lz > 3u) {
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        continue;
      }
      float wt[3][3], dw[3][3];
      bspline_weights(b.fx, wt);
      bspline_dweights(b.fx, dw);
      float mu0 = P.mu0, la0 = P.la0;
      const bool perE = Ep > 0.0f;
      if (perE) {
        mu0 = Ep * dmu0;
        la0 = Ep * dla0;
      }
      // ---- forward recomputation (engine/mpm_solver.py:506-574) ----
      float Fin[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) Fin[r][c] = mat == 0 ? (r == c ? (r == 0 ? Jp : 1.0f) : 0.0f) : F[r][c];
      float Fn[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          Fn[r][c] = Fin[r][c] + dt * (C[r][0] * Fin[0][c] + C[r][1] * Fin[1][c] + C[r][2] * Fin[2][c]);
      float Cf[3][3];
      cofactor(Fn, Cf);
      const float J = Fn[0][0] * Cf[0][0] + Fn[0][1] * Cf[0][1] + Fn[0][2] * Cf[0][2];
      const float h = mat == 1 ? 0.3f : 1.0f;
      const float mu = mat == 0 ? 0.0f : mu0 * h, la = la0 * h;
      // Rotation R = U V^T of Fn: the Newton polar factor when det Fn > 0 (as
      // in the forward), else from the SVD (inverted / extreme stretch).
      float U[3][3], sg[3], V[3][3], R[3][3];
      const bool polar_ok = mat == 1 && J > 0.0f && polar_rotation<6>(Fn, R);
      if (mat == 1 && !polar_ok) {
        svd3<4>(Fn, U, sg, V);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) R[r][c] = U[r][0] * V[c][0] + U[r][1] * V[c][1] + U[r][2] * V[c][2];
      }
      float stress[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float acc = 0.0f;
          if (mat == 1)
            acc = 2.0f * mu * ((Fn[r][0] - R[r][0]) * Fn[c][0] + (Fn[r][1] - R[r][1]) * Fn[c][1] +
                               (Fn[r][2] - R[r][2]) * Fn[c][2]);
          stress[r][c] = acc + (r == c ? la * J * (J - 1.0f) : 0.0f);
        }
      const float mass = mat == 0 ? P.p_mass * P.water_density : P.p_mass;
      float A[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) A[r][c] = sc * stress[r][c] + mass * C[r][c];
      // ---- reverse of the scatter (engine/mpm_solver.py:576-584) ----
      float gv[3] = {0.f, 0.f, 0.f}, gA[3][3], gfx[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int a = 0; a < 9; ++a) gA[a / 3][a % 3] = 0.0f;
      const int base_node = (lx * kTileW + ly) * kTileW + lz;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float4 g4 = gt[base_node + (a * kTileW + bb) * kTileW + c];
            const float Gmv[3] = {g4.y, g4.z, g4.w};
            const float d[3] = {((float)a - b.fx[0]) * P.dx, ((float)bb - b.fx[1]) * P.dx, ((float)c - b.fx[2]) * P.dx};
            const float wgt = wt[a][0] * wt[bb][1] * wt[c][2];
            float gw = g4.x * mass;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
              const float Ad = A[r][0] * d[0] + A[r][1] * d[1] + A[r][2] * d[2];
              gw += Gmv[r] * (mass * v[r] + Ad);
              gv[r] += wgt * mass * Gmv[r];
#pragma unroll
              for (int q = 0; q < 3; ++q) gA[r][q] += wgt * Gmv[r] * d[q];
            }
            gfx[0] += gw * dw[a][0] * wt[bb][1] * wt[c][2];
            gfx[1] += gw * wt[a][0] * dw[bb][1] * wt[c][2];
            gfx[2] += gw * wt[a][0] * wt[bb][1] * dw[c][2];
#pragma unroll
            for (int q = 0; q < 3; ++q)
              gfx[q] -= P.dx * wgt * (A[0][q] * Gmv[0] + A[1][q] * Gmv[1] + A[2][q] * Gmv[2]);
          }
      // ---- reverse of affine = sc stress + m C ----
      float gC_[3][3], gS[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          gC_[r][c] = mass * gA[r][c];
          gS[r][c] = sc * gA[r][c];
        }
      const float trgS = gS[0][0] + gS[1][1] + gS[2][2];
      // ---- reverse of the constitutive model ----
      float GFo[3][3];
#pragma unroll
      for (int a = 0; a < 9; ++a) GFo[a / 3][a % 3] = gin[(gF + a) * cap + gi];
      const float GJpo = gin[gJp * cap + gi];
      float gFn[3][3];
      float gJ = la * (2.0f * J - 1.0f) * trgS;
      float gEv = 0.0f;
      float gJp_out = 0.0f;
      if (mat == 0) {  // water: F' = diag(J,1,1), Jp' = J
        gJ += GFo[0][0] + GJpo;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) gFn[r][c] = gJ * Cf[r][c];
        if (perE) gEv = dla0 * h * J * (J - 1.0f) * trgS;
      } else {  // elastic: F' = Fn, Jp' = Jp
        float D[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) D[r][c] = Fn[r][c] - R[r][c];
        float gR[3][3];
        float gmu = 0.0f;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            // S1 = 2 mu D Fn^T: gD = 2 mu gS Fn, gFn += 2 mu gS^T D
            const float gD = 2.0f * mu * (gS[r][0] * Fn[0][c] + gS[r][1] * Fn[1][c] + gS[r][2] * Fn[2][c]);
            const float gF2 = 2.0f * mu * (gS[0][r] * D[0][c] + gS[1][r] * D[1][c] + gS[2][r] * D[2][c]);
            gFn[r][c] = GFo[r][c] + gD + gF2 + gJ * Cf[r][c];
            gR[r][c] = -gD;
            gmu += gS[r][c] * 2.0f * (D[r][0] * Fn[c][0] + D[r][1] * Fn[c][1] + D[r][2] * Fn[c][2]);
          }
        if (polar_ok) {
          // Polar backward without an SVD: with S = R^T Fn and dR = R [w]x,
          // S[w]x + [w]x S = [(tr S I - S) w]x gives
          // dL/dFn += R [z]x, z = (tr S I - S)^{-1} axial(R^T gR),
          // axial(X) = (X21 - X12, X02 - X20, X10 - X01); the eigenvalues of
          // tr S I - S are the sums s_i + s_j, kept away from zero.
          float S[3][3], M[3][3];
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              S[r][c] = R[0][r] * Fn[0][c] + R[1][r] * Fn[1][c] + R[2][r] * Fn[2][c];
              M[r][c] = R[0][r] * gR[0][c] + R[1][r] * gR[1][c] + R[2][r] * gR[2][c];
            }
          const float trS = S[0][0] + S[1][1] + S[2][2];
          float A[3][3];
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) A[r][c] = (r == c ? trS : 0.0f) - 0.5f * (S[r][c] + S[c][r]);
          const float mv[3] = {M[2][1] - M[1][2], M[0][2] - M[2][0], M[1][0] - M[0][1]};
          float Ac[3][3];
          cofactor(A, Ac);
          float detA = A[0][0] * Ac[0][0] + A[0][1] * Ac[0][1] + A[0][2] * Ac[0][2];
          if (fabsf(detA) < 1e-12f) detA = detA < 0.0f ? -1e-12f : 1e-12f;
          const float inv_det = 1.0f / detA;
          float z[3];
#pragma unroll
          for (int r = 0; r < 3; ++r) z[r] = inv_det * (Ac[0][r] * mv[0] + Ac[1][r] * mv[1] + Ac[2][r] * mv[2]);
          const float Zx[3][3] = {{0.0f, -z[2], z[1]}, {z[2], 0.0f, -z[0]}, {-z[1], z[0], 0.0f}};
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) gFn[r][c] += R[r][0] * Zx[0][c] + R[r][1] * Zx[1][c] + R[r][2] * Zx[2][c];
        } else {
        // polar rotation R = U V^T: dF = U [K o (M - M^T)] V^T with
        // M = U^T gR V and K_ij = 1 / (s_i + s_j), clamped away from zero
        float M[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float acc = 0.0f;
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
              for (int q = 0; q < 3; ++q) acc += U[p][r] * gR[p][q] * V[q][c];
            M[r][c] = acc;
          }
        float Kx[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float den = sg[r] + sg[c];
            if (fabsf(den) < 1e-6f) den = den < 0.0f ? -1e-6f : 1e-6f;
            Kx[r][c] = r == c ? 0.0f : (M[r][c] - M[c][r]) / den;
          }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float acc = 0.0f;
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
              for (int q = 0; q < 3; ++q) acc += U[r][p] * Kx[p][q] * V[c][q];
            gFn[r][c] += acc;
          }
        }
        if (perE) gEv = h * (dmu0 * gmu + dla0 * J * (J - 1.0f) * trgS);
        gJp_out = GJpo;
      }
      // ---- reverse of Fn = (I + dt C) Fin ----
      float gFin[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          gC_[r][c] += dt * (gFn[r][0] * Fin[c][0] + gFn[r][1] * Fin[c][1] + gFn[r][2] * Fin[c][2]);
          float acc = gFn[r][c];
#pragma unroll
          for (int p = 0; p < 3; ++p) acc += dt * C[p][r] * gFn[p][c];
          gFin[r][c] = acc;
        }
      if (mat == 0) gJp_out = gFin[0][0];
      // ---- outputs: gradient of the state before the substep ----
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        gout[(gX + d) * cap + go] = gmid[d * cap + j] + P.inv_dx * gfx[d];
        gout[(gV + d) * cap + go] = gv[d];
      }
#pragma unroll
      for (int a = 0; a < 9; ++a) {
        gout[(gC + a) * cap + go] = gC_[a / 3][a % 3];
        gout[(gF + a) * cap + go] = mat == 1 ? gFin[a / 3][a % 3] : 0.0f;
      }
      gout[gJp * cap + go] = gJp_out;
      gout[gE * cap + go] = gin[gE * cap + gi] + (perE ? gEv : 0.0f);  // E passes through the substep
    }
    __syncthreads();
  }
  set_status(w, bad);
}

// Gradient rows between original-id columns and the column order of a
// particle state (its id row maps column j to an id).
__global__ void k_grad_reorder(const float *__restrict__ st, int64_t cap, int64_t n, int rows,
                               const float *__restrict__ src, float *__restrict__ dst, bool to_state_order) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t id = __float_as_int(st[kId * cap + j]);
  if (id < 0 || id >= n) return;  // corrupted id row: leave the column untouched
  const int64_t from = to_state_order ? id : j, to = to_state_order ? j : id;
  for (int r = 0; r < rows; ++r) dst[r * cap + to] = src[r * cap + from];
}

}  // namespace mpm

using namespace mpm;

extern "C" {

static int adj_dev_sms() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return sms;
}

static bool adj_params_ok(const MpmParams *p) {
  if (!p || p->version != MPM_ABI_VERSION || p->quant || p->chunk < 32 || (p->chunk & 31) != 0) return false;
  for (int d = 0; d < 3; ++d)
    if (p->win_nb[d] <= 0 || (p->win_lo[d] & 3) != 0) return false;
  return p->n_colliders >= 0 && p->n_colliders <= MPM_MAX_COLLIDERS;
}

int mpm_grid_snapshot(const MpmParams *p, void *ws, int64_t cap, float *keep, void *stream) {
  if (!adj_params_ok(p) || !ws || !keep) return MPM_E_INVALID;
  const int sms = adj_dev_sms();
  if (!sms) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  k_grid_snapshot<<<sms * 8, 256, 0, (cudaStream_t)stream>>>(*p, w, (float4 *)keep);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_g2p_adj(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float dt, const float *gin,
                float *gmid, float *ggrid, int32_t by_id, void *stream) {
  if (!adj_params_ok(p) || !ws || !cur || !gin || !gmid || !ggrid || n < 0 || n > cap) return MPM_E_INVALID;
  const int sms = adj_dev_sms();
  if (!sms) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  if (by_id)
    k_g2p_adj<true><<<sms * 4, kAdjThreads, 0, (cudaStream_t)stream>>>(*p, w, cur, cap, dt, gin, gmid, (float4 *)ggrid);
  else
    k_g2p_adj<false><<<sms * 4, kAdjThreads, 0, (cudaStream_t)stream>>>(*p, w, cur, cap, dt, gin, gmid, (float4 *)ggrid);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_grid_adj(const MpmParams *p, void *ws, int64_t cap, const float *keep, float *ggrid, float dt,
                 void *stream) {
  if (!adj_params_ok(p) || !ws || !keep || !ggrid) return MPM_E_INVALID;
  const int sms = adj_dev_sms();
  if (!sms) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  k_grid_adj<<<sms * 8, 256, 0, (cudaStream_t)stream>>>(*p, w, (const float4 *)keep, (float4 *)ggrid, dt);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_p2g_adj(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float dt, const float *gin,
                const float *gmid, float *gout, const float *ggrid, int32_t by_id, void *stream) {
  if (!adj_params_ok(p) || !ws || !cur || !gin || !gmid || !gout || !ggrid || gin == gout || n < 0 || n > cap)
    return MPM_E_INVALID;
  const int sms = adj_dev_sms();
  if (!sms) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  if (by_id)
    k_p2g_adj<true><<<sms * 4, kAdjThreads, 0, (cudaStream_t)stream>>>(*p, w, cur, cap, dt, gin, gmid, gout,
                                                                      (const float4 *)ggrid);
  else
    k_p2g_adj<false><<<sms * 4, kAdjThreads, 0, (cudaStream_t)stream>>>(*p, w, cur, cap, dt, gin, gmid, gout,
                                                                       (const float4 *)ggrid);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

int mpm_grad_reorder(const float *state, int64_t cap, int64_t n, int32_t rows, const float *src, float *dst,
                     int32_t to_state_order, void *stream) {
  if (!state || !src || !dst || src == dst || n < 0 || n > cap || rows < 1 || rows > 64) return MPM_E_INVALID;
  if (n == 0) return MPM_OK;
  k_grad_reorder<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(state, cap, n, rows, src, dst,
                                                                                to_state_order != 0);
  return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA;
}

}  // extern "C"
