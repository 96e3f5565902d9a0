// GB300 (sm_103a) kernels of the MLS-MPM substep and their C ABI.
//
// Pipeline of one substep (engine/mpm_solver.py:789-799 of
// taichi-dev/taichi_elements), all on one stream, no host synchronisation:
//
//   k_flags_count/k_flags_write   active 4^3 blocks -> ordered compact lists
//                                 (particle blocks, and grid blocks = particle
//                                 blocks dilated by {0,1}^3)
//   k_pb_stats/k_pb_scan          per particle block: count, start, level
//                                 table base and work-item base (two-pass scan)
//   k_pb_levels                   rank-major level tables, work items, clears
//                                 the block flags
//   k_scatter                     sorted order pid[pos] = i
//   k_cell_clear                  clears the cell counters
//   k_p2g                         per work item: stress, APIC scatter into a
//                                 shared-memory 6^3 tile, one float4 atomic
//                                 flush per touched node
//   k_grid                        momentum->velocity, gravity, box, colliders
//   k_g2p                         per work item: 6^3 velocity tile in shared
//                                 memory, gather, advect, bin for the next
//                                 substep
//
// Sorted order inside a block is rank-major: all cells' first particles (in
// cell order), then all cells' second particles, ...  Consecutive lanes thus
// work on different cells, so their shared-memory atomics and gathers hit
// different nodes.  A particle that stays in its cell keeps its rank (less
// the cell's leavers ranked below it), so the sorted order changes only
// where particles cross cells and P2G's reads of the previous order through
// pid stay nearly contiguous.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>
#include <mutex>

#include "mpm_common.cuh"
#include "tma.cuh"

namespace mpm {

// fused G2P2G: CTAs of 128 threads, per-warp tiles; CTAs per SM the
// register budget is sized for
constexpr int kFusedThreads = 128;
constexpr int kFusedWarps = kFusedThreads / 32;
#ifndef MPM_FUSED_MIN_CTAS
#define MPM_FUSED_MIN_CTAS 4
#endif
constexpr int kG2PThreads = 128;


__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// ------------------------------------------------------------ binning ----

// kNeighbourMask[need]: bits of all neighbour offsets d (dx*4+dy*2+dz) whose
// set bits are a subset of `need`.
__constant__ int kNeighbourMask[8] = {0x01, 0x03, 0x05, 0x0F, 0x11, 0x33, 0x55, 0xFF};

// Scene constants.  A single scene uses the kernel's own parameters; in
// batched mode a particle's scene index sits in bits 8.. of its material word
// and a grid block's scene follows from its slot in the shared window.
template <bool BATCH>
__device__ __forceinline__ const MpmParams &scene_of_particle(const MpmParams &P, const MpmParams *tab, int matword) {
  if constexpr (BATCH) {
    const int s = min(max(matword >> 8, 0), P.n_scenes - 1);
    return tab[s];
  } else {
    return P;
  }
}

template <bool BATCH>
__device__ __forceinline__ int scene_index_of_block(const MpmParams &P, int bx, int by, int bz) {
  if constexpr (BATCH) {
    const int s = bx / P.slot_nb[0] + P.slots[0] * (by / P.slot_nb[1] + P.slots[1] * (bz / P.slot_nb[2]));
    return min(max(s, 0), P.n_scenes - 1);
  } else {
    return 0;
  }
}

template <bool BATCH>
__device__ __forceinline__ const MpmParams &scene_of_block(const MpmParams &P, const MpmParams *tab, int bx, int by,
                                                           int bz) {
  if constexpr (BATCH) {
    return tab[scene_index_of_block<true>(P, bx, by, bz)];
  } else {
    return P;
  }
}

// Bins the particle at slot i for the next substep and returns its cell key.
// A particle still in cell old_key with a rank r_old < 64 there keeps that
// rank, less the cell's leavers ranked below it (k_scatter subtracts them);
// the others get their rank from the arrival order in k_scatter.
template <bool BATCH>
__device__ __forceinline__ int bin_one(const MpmParams &P, const MpmParams *tab, const Ws &w, int64_t i, float x0,
                                       float x1, float x2, int matword, uint32_t &bad, int old_key = -1,
                                       int r_old = -1) {
  const Base b = particle_base(scene_of_particle<BATCH>(P, tab, matword), x0, x1, x2, bad);
  const int key = cell_key(P, b);
  const int sr = (key == old_key && (unsigned)r_old < 64u) ? r_old : -1;
  atomicAdd(&w.cell_cnt[key], 1);  // results unused: fire-and-forget reductions
  if (sr < 0) atomicAdd(&w.arr_cnt[key], 1);
  w.stay_rank[i] = sr;
  const int blin = key >> 6;
  // Blocks this particle's 3^3 stencil reaches: its own block plus, per axis,
  // the next block when the base sits in the last two cells of the block.
  // Bit (dx*4 + dy*2 + dz) of the flag marks block b + (dx,dy,dz); the
  // grid-active set is then exactly the set of blocks holding stencil nodes
  // (the blocks the reference's sparse grid activates in P2G, :582-584).
  const int need = ((b.b[0] & 3) >= 2 ? 4 : 0) | ((b.b[1] & 3) >= 2 ? 2 : 0) | ((b.b[2] & 3) >= 2 ? 1 : 0);
  const int mask = kNeighbourMask[need];
  // lanes of a warp mostly share a block: one fire-and-forget OR per block
  const unsigned act = __activemask();
  const unsigned same = __match_any_sync(act, blin);
  const int all = (int)__reduce_or_sync(same, (unsigned)mask);
  if ((threadIdx.x & 31) == __ffs(same) - 1) atomicOr(&w.blk_flag[blin], all);
  w.cellkey[i] = key;
  return key;
}

template <bool BATCH, bool Q>
__global__ void k_bin_count(const MpmParams P, const MpmParams *tab, const Ws w, const float *__restrict__ ps,
                            int64_t cap, int64_t begin, int64_t end) {
  const int64_t i = begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t bad = 0;
  if (i < end) {
    const int matword = BATCH ? ld_mat<Q>(ps, cap, i) : 0;
    float x[3];
    ld_x<Q>(ps, cap, i, x);
    bin_one<BATCH>(P, tab, w, i, x[0], x[1], x[2], matword, bad);
  }
  set_status(w, bad);
}


// grid-active = some particle block b - d whose stencils reach b (bit d)
__device__ __forceinline__ bool grid_flag(const MpmParams &P, const Ws &w, int64_t b) {
  int bx, by, bz;
  block_coords(P, b, bx, by, bz);
  const int64_t sy = P.win_nb[2], sx = (int64_t)P.win_nb[1] * P.win_nb[2];
  bool f = false;
#pragma unroll
  for (int dx = 0; dx < 2; ++dx)
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dz = 0; dz < 2; ++dz)
        if (bx >= dx && by >= dy && bz >= dz)
          f |= ((w.blk_flag[b - dx * sx - dy * sy - dz] >> (dx * 4 + dy * 2 + dz)) & 1) != 0;
  return f;
}

template <typename T>
__device__ __forceinline__ T block_sum_256(T v, T *sh) {
  // inclusive-sum of a 256-thread CTA; returns the total; sh needs 8 slots
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T t = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) t += sh[k];
  __syncthreads();
  return t;
}

// exclusive scan across a 256-thread CTA; returns the exclusive prefix and
// writes the CTA total to *total.  sh needs 8 slots.
__device__ __forceinline__ int block_excl_scan_256(int v, int *sh, int *total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += n;
  }
  if (lane == 31) sh[wid] = inc;
  __syncthreads();
  int before = 0, tot = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int s = sh[k];
    before += (k < wid) ? s : 0;
    tot += s;
  }
  __syncthreads();
  *total = tot;
  return before + inc - v;
}

__global__ __launch_bounds__(256) void k_flags_count(const MpmParams P, const Ws w) {
  __shared__ int sh[8];
  int cp = 0, cg = 0;
  for (int q = 0; q < kFlagTile / 256; ++q) {
    const int64_t b = (int64_t)blockIdx.x * kFlagTile + q * 256 + threadIdx.x;
    if (b < w.nblk) {
      cp += w.blk_flag[b] != 0;
      cg += grid_flag(P, w, b);
    }
  }
  const int tp = block_sum_256(cp, sh);
  const int tg = block_sum_256(cg, sh);
  if (threadIdx.x == 0) {
    w.flag_tiles[2 * blockIdx.x] = tp;
    w.flag_tiles[2 * blockIdx.x + 1] = tg;
  }
}

__global__ __launch_bounds__(256) void k_flags_write(const MpmParams P, const Ws w) {
  __shared__ int sh[8];
  // offsets of this tile = sum over preceding tiles
  int op = 0, og = 0;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += 256) {
    op += w.flag_tiles[2 * t];
    og += w.flag_tiles[2 * t + 1];
  }
  op = block_sum_256(op, sh);
  og = block_sum_256(og, sh);
  for (int q = 0; q < kFlagTile / 256; ++q) {
    const int64_t b = (int64_t)blockIdx.x * kFlagTile + q * 256 + threadIdx.x;
    int fp = 0, fg = 0;
    if (b < w.nblk) {
      fp = w.blk_flag[b] != 0;
      fg = grid_flag(P, w, b);
    }
    int totp, totg;
    const int ep = block_excl_scan_256(fp, sh, &totp);
    const int eg = block_excl_scan_256(fg, sh, &totg);
    if (fp) {
      w.pblocks[op + ep] = (int)b;
      w.blk_slot[b] = op + ep;
    }
    if (fg) w.gblocks[og + eg] = (int)b;
    op += totp;
    og += totg;
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    w.counters[0] = op;
    w.counters[1] = og;
    w.counters[2] = 0;
    w.counters[4] = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {  // the next G2P's bounding box starts empty
      w.counters[kBoxMin + d] = float_key_i32(INFINITY);
      w.counters[kBoxMax + d] = float_key_i32(-INFINITY);
    }
  }
}

__global__ __launch_bounds__(256) void k_pb_stats(const MpmParams P, const Ws w) {
  __shared__ int sh[8];
  const int npb = w.counters[0];
  if ((int64_t)blockIdx.x * kStatTile >= npb) return;
  const int k = blockIdx.x * kStatTile + threadIdx.x;
  int n = 0, mx = 0, ni = 0;
  if (k < npb) {
    const int4 *c4 = reinterpret_cast<const int4 *>(w.cell_cnt + (int64_t)w.pblocks[k] * kBlockCells);
#pragma unroll 4
    for (int q = 0; q < 16; ++q) {
      const int4 c = c4[q];
      n += c.x + c.y + c.z + c.w;
      mx = max(mx, max(max(c.x, c.y), max(c.z, c.w)));
    }
    ni = (n + P.chunk - 1) / P.chunk;
  }
  int tn, tm, ti;
  const int en = block_excl_scan_256(n, sh, &tn);
  const int em = block_excl_scan_256(mx, sh, &tm);
  const int ei = block_excl_scan_256(ni, sh, &ti);
  if (k < npb) {
    w.pb_count[k] = n;
    w.pb_start[k] = en;
    w.pb_lvl[k] = em;
    w.pb_item[k] = ei;
  }
  if (threadIdx.x == 0) {
    w.pb_tiles[3 * blockIdx.x] = tn;
    w.pb_tiles[3 * blockIdx.x + 1] = tm;
    w.pb_tiles[3 * blockIdx.x + 2] = ti;
  }
}

__global__ __launch_bounds__(256) void k_pb_scan(const MpmParams P, const Ws w) {
  __shared__ int sh[8];
  const int npb = w.counters[0];
  if ((int64_t)blockIdx.x * kStatTile >= npb) return;
  int on = 0, om = 0, oi = 0;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += 256) {
    on += w.pb_tiles[3 * t];
    om += w.pb_tiles[3 * t + 1];
    oi += w.pb_tiles[3 * t + 2];
  }
  on = block_sum_256(on, sh);
  om = block_sum_256(om, sh);
  oi = block_sum_256(oi, sh);
  const int k = blockIdx.x * kStatTile + threadIdx.x;
  if (k < npb) {
    const int s = w.pb_start[k] + on;
    const int it = w.pb_item[k] + oi;
    w.pb_start[k] = s;
    w.pb_lvl[k] += om;
    w.pb_item[k] = it;
    if (k == npb - 1) {
      const int c = w.pb_count[k];
      w.counters[2] = it + (c + P.chunk - 1) / P.chunk;
      w.counters[4] = s + c;
    }
  }
}

// One warp per particle block: rank-major level table, work items, and the
// clearing of the block flag (the cell counters are cleared by k_cell_clear
// once k_scatter has ranked the particles).
__global__ __launch_bounds__(256) void k_pb_levels(const MpmParams P, const Ws w, int64_t cap) {
  const int npb = w.counters[0];
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < npb; k += nwarps) {
    const int blin = w.pblocks[k];
    int32_t *cc = w.cell_cnt + (int64_t)blin * kBlockCells;
    const int c0 = cc[lane], c1 = cc[lane + 32];
    int mx = max(c0, c1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int lvl = w.pb_lvl[k];
    if ((int64_t)lvl + mx > cap) {  // counts exceed the capacity: binning is stale
      if (lane == 0) set_status(w, MPM_STATUS_TABLE_OVERFLOW);
      mx = 0;
    }
    if (lane == 0) w.pb_nlev[k] = mx;
    int L = 0;
    for (int r = 0; r < mx; ++r) {
      const unsigned m0 = __ballot_sync(0xffffffffu, c0 > r);
      const unsigned m1 = __ballot_sync(0xffffffffu, c1 > r);
      if (lane == 0) {
        w.lvl_mask[lvl + r] = (unsigned long long)m0 | ((unsigned long long)m1 << 32);
        w.lvl_L[lvl + r] = L;
      }
      L += __popc(m0) + __popc(m1);
    }
    const int n = w.pb_count[k], st = w.pb_start[k], ib = w.pb_item[k];
    const int ni = (n + P.chunk - 1) / P.chunk;
    for (int j = lane; j < ni; j += 32) {
      if (ib + j < w.items_cap)
        w.items[ib + j] = make_int2(k, st + j * P.chunk);
      else
        set_status(w, MPM_STATUS_TABLE_OVERFLOW);
    }
    if (lane == 0) w.blk_flag[blin] = 0;
  }
}

__global__ void k_scatter(const MpmParams P, const Ws w, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  w.inv[i] = -1;  // until the particle's sorted slot is known
  const int key = w.cellkey[i];
  // Rank inside the cell: particles that stayed in their cell keep their
  // order (ranks 0 .. N - A - 1, set in G2P); the A others take the ranks
  // above in arrival order.
  const int sr = w.stay_rank[i];
  const int N = w.cell_cnt[key];
  const int r = sr >= 0 ? sr - __popcll(w.leave[key] & ((1ull << sr) - 1ull))
                        : (N - w.arr_cnt[key]) + atomicAdd(&w.arr_rank[key], 1);
  const int blin = key >> 6, c = key & 63;
  const int k = w.blk_slot[blin];
  if (k < 0 || k >= w.counters[0] || r < 0 || r >= N) {  // stale binning: report, never index out of range
    set_status(w, MPM_STATUS_TABLE_OVERFLOW);
    return;
  }
  const int lv = w.pb_lvl[k] + r;
  if (lv >= n) {
    set_status(w, MPM_STATUS_TABLE_OVERFLOW);
    return;
  }
  const unsigned long long below = c == 0 ? 0ull : (w.lvl_mask[lv] & ((1ull << c) - 1ull));
  const int pos = w.pb_start[k] + w.lvl_L[lv] + __popcll(below);
  if (pos < 0 || pos >= n) {
    set_status(w, MPM_STATUS_TABLE_OVERFLOW);
    return;
  }
  w.pid[pos] = (int)i;
  w.inv[i] = pos;
  w.slot_rank[pos] = r;
}

// Clears the per-cell counters and leave masks of the particle blocks once
// k_scatter has used them, ready for the next binning.  The next G2P marks
// leavers only in cells of these blocks (their cells before advection), and
// k_scatter reads a mask only at a stayer's cell, which was a cell of the
// previous particle blocks too: masks left in blocks that emptied are never
// read before their block is cleared again.
__global__ __launch_bounds__(256) void k_cell_clear(const MpmParams P, const Ws w) {
  const int npb = w.counters[0];
  const int64_t total = (int64_t)npb * kBlockCells;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = (int64_t)w.pblocks[t >> 6] * kBlockCells + (t & 63);
    w.cell_cnt[a] = 0;
    w.arr_cnt[a] = 0;
    w.arr_rank[a] = 0;
    w.leave[a] = 0ull;
  }
}

// ---------------------------------------------------------------- P2G ----
//
// P2G visits the particles in the order of the state buffer `cur` (the
// sorted order of the previous substep), 32 consecutive slots per warp step,
// so each state row of a step is one contiguous 128-byte segment.  Each warp
// runs its own two-stage pipeline: once the current step's rows are in
// registers, one lane issues the bulk copies (TMA) of the next step's rows
// and of their sorted slots (`inv`) into the warp's staging buffer, which
// land while the warp works on the current step.  Per particle: constitutive update (engine/mpm_solver.py
// :506-574), the updated state written to its sorted slot `inv[i]` of `nxt`,
// and the APIC scatter (:576-584) into the warp's 8^3 float4 tile of grid
// nodes with plain shared-memory read-modify-writes.  The tile is anchored at
// the step's smallest base cell: the particles of a step are the 32 cells of
// one level of one block of the previous binning, so their base cells lie in
// a 6-wide range and several steps share one anchor.  When a step does not fit
// the tile is flushed to the grid (one float4 reduction per touched node) and
// re-anchored; the rare particle outside a fresh anchor scatters with global
// atomics.  Lanes of a step hold distinct cells (rank-major order), so the 27
// node updates of a pass never collide; particles that moved into a shared
// cell are found with __match_any_sync and scatter in later passes.  Steps
// are taken from a guided queue in runs of consecutive steps.

constexpr int kP2GWarps = 4;
// P2G CTAs per SM the register budget is sized for (168 registers at 3; 4 would
// fit the shared memory but spill)
#ifndef MPM_P2G_MIN_CTAS
#define MPM_P2G_MIN_CTAS 3
#endif
constexpr int kP2GThreads = kP2GWarps * 32;
constexpr int kP2GQueue = 5, kP2GDone = 6;     // counters[]: run queue, warps done
constexpr int kP2GTileW = 8;                   // tile nodes per axis
// tile index = tx * 76 + ty * 9 + tz: the x stride is 4 mod 8, so the 8 lanes
// of a quarter-warp (cells z = 0..3 at x = 2k, 2k+1) hit 8 bank groups
constexpr int kP2GTileSX = 76, kP2GTileSY = 9;
constexpr int kP2GTileN = 7 * kP2GTileSX + 7 * kP2GTileSY + 8;  // 603
constexpr int kP2GRowsMax = MPM_NROWS + 1;     // state rows + inv

// Per-warp shared memory.  A tiled tensor copy needs a 128-byte-aligned
// shared destination: the struct (buffers first) is 128-byte aligned and its
// size a multiple of 128, and the dynamic shared base is 128-byte aligned.
struct __align__(128) P2GWarpSmem {
  float buf[kP2GRowsMax][32];
  float4 tile[kP2GTileN + 1];
  unsigned long long bar;
};
static_assert(sizeof(P2GWarpSmem) % 128 == 0, "per-warp staging buffers must stay 128-byte aligned");
constexpr size_t kP2GSmem = sizeof(P2GWarpSmem) * kP2GWarps;

template <bool Q, bool HAS_EP>
struct P2GRows {  // rows staged per step (the state rows P2G reads)
  static constexpr int N = Q ? MPM_QROWS : (HAS_EP ? MPM_NROWS : MPM_NROWS - 1);
};

__device__ __forceinline__ int p2g_tile_index(int tx, int ty, int tz) {
  return tx * kP2GTileSX + ty * kP2GTileSY + tz;
}

// Flushes the warp's tile anchored at node o (window-relative) to the grid
// and clears it.  MARK: also flag the 4^3 blocks that received momentum
// (bit 0 of blk_flag), which then make the grid-active list of a substep
// without binning.
template <bool MARK = false>
__device__ __forceinline__ void p2g_tile_flush(const MpmParams &P, const Ws &w, float4 *tile, const int (&o)[3],
                                               int lane) {
  uint32_t touched = 0u;  // bit (bx * 3 + by) * 3 + bz over the <= 3^3 blocks the window overlaps
  for (int t = lane; t < kP2GTileW * kP2GTileW * kP2GTileW; t += 32) {
    const int tx = t >> 6, ty = (t >> 3) & 7, tz = t & 7;
    float4 &nd = tile[p2g_tile_index(tx, ty, tz)];
    const float4 g = nd;
    if (g.x != 0.0f) {
      const int gx = o[0] + tx, gy = o[1] + ty, gz = o[2] + tz;
      if (gx < P.win_nb[0] * 4 && gy < P.win_nb[1] * 4 && gz < P.win_nb[2] * 4) {
        atomicAdd(&w.grid_mom[node_addr(P, gx, gy, gz)], g);
        if (MARK)
          touched |= 1u << ((((gx >> 2) - (o[0] >> 2)) * 3 + ((gy >> 2) - (o[1] >> 2))) * 3 + ((gz >> 2) - (o[2] >> 2)));
      }
      nd = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  if (MARK) {
    touched = __reduce_or_sync(0xffffffffu, touched);
    if (lane < 27 && ((touched >> lane) & 1u)) {
      const int bx = (o[0] >> 2) + lane / 9, by = (o[1] >> 2) + (lane / 3) % 3, bz = (o[2] >> 2) + lane % 3;
      atomicOr(&w.blk_flag[block_linear(P, bx, by, bz)], 1);
    }
  }
  __syncwarp();
}

// The APIC scatter (engine/mpm_solver.py:576-584) of one warp step into the
// warp's tile: node value = w * (m v + A (off - fx) dx) = w * ((m, q) +
// a Ax + b Ay + c Az), q = m v - A fx dx, Ax..Az the columns of A dx.  The
// tile is anchored at the step's base cells (see k_p2g); a particle outside a
// fresh anchor scatters with global atomics.  MARK: flag the blocks that
// receive momentum (see p2g_tile_flush).
// ROLL keeps the stencil's x loop rolled: fewer registers (the batched P2G
// then fits 4 CTAs per SM, 16 warps, and runs 10% faster on the batch's small
// scenes) for a longer instruction stream.
template <bool MARK, bool ROLL = false>
__device__ __forceinline__ void p2g_scatter_step(const MpmParams &P, const Ws &w, float4 *tile, int (&o)[3],
                                                 bool &anchored, bool act, const Base &bs, const float (&wt)[3][3],
                                                 float mass, const float (&q)[3], const float (&adx)[3][3],
                                                 int lane) {
  // anchor the tile: all base cells within [o, o + 5]
  int lo[3], hi[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = __reduce_min_sync(0xffffffffu, act ? bs.b[d] : INT32_MAX);
    hi[d] = __reduce_max_sync(0xffffffffu, act ? bs.b[d] : INT32_MIN);
  }
  if (__any_sync(0xffffffffu, act)) {
    const bool fits = anchored && lo[0] >= o[0] && lo[1] >= o[1] && lo[2] >= o[2] &&
                      hi[0] <= o[0] + kP2GTileW - 3 && hi[1] <= o[1] + kP2GTileW - 3 &&
                      hi[2] <= o[2] + kP2GTileW - 3;
    if (!fits) {
      if (anchored) p2g_tile_flush<MARK>(P, w, tile, o, lane);
      // one cell of slack below: the steps of one block of the previous
      // binning have base cells in [B - 1, B + 4] (B the block's first
      // cell), and the first step's smallest is usually B
#pragma unroll
      for (int d = 0; d < 3; ++d) o[d] = hi[d] - lo[d] <= kP2GTileW - 4 ? max(lo[d] - 1, 0) : lo[d];
      anchored = true;
    }
  }
  const int tx0 = bs.b[0] - o[0], ty0 = bs.b[1] - o[1], tz0 = bs.b[2] - o[2];
  const bool inwin = act && (unsigned)tx0 <= kP2GTileW - 3 && (unsigned)ty0 <= kP2GTileW - 3 &&
                     (unsigned)tz0 <= kP2GTileW - 3;
  if (act && !inwin) {  // rare: straight to the grid
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int bb = 0; bb < 3; ++bb)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const int gx = bs.b[0] + a, gy = bs.b[1] + bb, gz = bs.b[2] + c;
          if (gx >= P.win_nb[0] * 4 || gy >= P.win_nb[1] * 4 || gz >= P.win_nb[2] * 4) continue;
          const float wgt = wt[a][0] * wt[bb][1] * wt[c][2];
          float4 g;
          g.x = wgt * mass;
          g.y = wgt * (q[0] + adx[0][0] * (float)a + adx[0][1] * (float)bb + adx[0][2] * (float)c);
          g.z = wgt * (q[1] + adx[1][0] * (float)a + adx[1][1] * (float)bb + adx[1][2] * (float)c);
          g.w = wgt * (q[2] + adx[2][0] * (float)a + adx[2][1] * (float)bb + adx[2][2] * (float)c);
          atomicAdd(&w.grid_mom[node_addr(P, gx, gy, gz)], g);
          if (MARK && wgt != 0.0f) atomicOr(&w.blk_flag[block_linear(P, gx >> 2, gy >> 2, gz >> 2)], 1);
        }
  }
  // tile scatter: one pass per set of lanes with distinct base cells
  const int cell = inwin ? p2g_tile_index(tx0, ty0, tz0) : -1 - lane;
  const unsigned peers = __match_any_sync(0xffffffffu, cell);
  const int round_of_lane = __popc(peers & ((1u << lane) - 1u));
  const int base_node = inwin ? cell : 0;
  for (int round = 0;; ++round) {
    const bool mine = inwin && round_of_lane == round;
#pragma unroll(ROLL ? 1 : 3)
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int bb = 0; bb < 3; ++bb) {
        const float wxa = a == 0 ? wt[0][0] : (a == 1 ? wt[1][0] : wt[2][0]);  // no indexing by a rolled a
        const float fa = (float)a;
        const float wab = wxa * wt[bb][1];
        const float2 p0 = make_float2(mass, fmaf(adx[0][1], (float)bb, fmaf(adx[0][0], fa, q[0])));
        const float2 p1 = make_float2(fmaf(adx[1][1], (float)bb, fmaf(adx[1][0], fa, q[1])),
                                      fmaf(adx[2][1], (float)bb, fmaf(adx[2][0], fa, q[2])));
        const float2 dz0 = make_float2(0.0f, adx[0][2]), dz1 = make_float2(adx[1][2], adx[2][2]);
        float2 t0 = p0, t1 = p1;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          // unconditional read and arithmetic, predicated store only
          const float wgt = wab * wt[c][2];
          const float2 w2 = make_float2(wgt, wgt);
          float4 *nd = tile + base_node + a * kP2GTileSX + bb * kP2GTileSY + c;
          float4 g = *nd;
          const float2 g01 = __ffma2_rn(w2, t0, make_float2(g.x, g.y));
          const float2 g23 = __ffma2_rn(w2, t1, make_float2(g.z, g.w));
          if (mine) *nd = make_float4(g01.x, g01.y, g23.x, g23.y);
          __syncwarp();
          if (c < 2) {
            t0 = __fadd2_rn(t0, dz0);
            t1 = __fadd2_rn(t1, dz1);
          }
        }
      }
    if (!__any_sync(0xffffffffu, inwin && round_of_lane > round)) break;
  }
}

// The next step of this warp (warp-uniform; -1 when the queue is empty)
// from the step queue in counters[q].  Lane 0 keeps the cursor (q_next,
// q_end) of its current run.  Runs are guided: a grab takes about a
// (2 * warps)-th of the steps left, at most kStepRun, so the last grabs are
// single steps and warps finish together.
constexpr int kStepRun = 16;
__device__ __forceinline__ int step_queue_next(const Ws &w, int q, int lane, int nsteps, int nwarps, int &q_next,
                                               int &q_end) {
  int g = -1;
  if (lane == 0) {
    if (q_next >= q_end) {
      const int seen = *(volatile const int *)&w.counters[q];
      const int len = max(1, min(kStepRun, (nsteps - seen) / (2 * nwarps)));
      const int r = atomicAdd(&w.counters[q], len);
      q_next = min(r, nsteps);
      q_end = min(r + len, nsteps);
    }
    if (q_next < q_end) g = q_next++;
  }
  return __shfl_sync(0xffffffffu, g, 0);
}

// The last warp of the launch to finish resets the queue counters[q] (and
// the done counter counters[d]), so the kernel can run again.
__device__ __forceinline__ void step_queue_done(const Ws &w, int q, int d, int lane, int nwarps) {
  if (lane == 0) {
    __threadfence();
    if (atomicAdd(&w.counters[d], 1) == nwarps - 1) {
      w.counters[q] = 0;
      w.counters[d] = 0;
    }
  }
}

// Stages step g: one tensor-map box of NR rows x 32 slots and the 32 sorted
// slots, completing on the warp's mbarrier.
template <int NR>
__device__ __forceinline__ void p2g_issue(P2GWarpSmem &sm, const CUtensorMap &rows_map, const Ws &w, int g,
                                          int lane) {
  if (lane == 0) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&sm.bar, (NR + 1) * 128);
    tma_load_2d(sm.buf[0], &rows_map, g * 32, 0, &sm.bar);
    bulk_g2s(sm.buf[NR], w.inv + (int64_t)g * 32, 128, &sm.bar);
  }
}

// ROLL: the scatter's x loop rolled, 4 CTAs per SM (MpmParams.occupancy; the
// batched form always)
template <bool HAS_EP, bool BATCH, bool Q, bool ROLL = BATCH>
__global__ __launch_bounds__(kP2GThreads, ROLL ? 4 : MPM_P2G_MIN_CTAS) void k_p2g(const MpmParams P,
                                                                                 const MpmParams *tab, const Ws w,
                                                        const __grid_constant__ CUtensorMap rows_map,
                                                        const float *__restrict__ cur, float *__restrict__ nxt,
                                                        int64_t cap, int64_t n, float dt) {
  using R = PRows<Q>;
  constexpr int NR = P2GRows<Q, HAS_EP>::N;
  extern __shared__ __align__(128) unsigned char p2g_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  P2GWarpSmem &sm = reinterpret_cast<P2GWarpSmem *>(p2g_smem)[warp];
  const int nsteps = (int)((n + 31) / 32);
  const int nwarps = (int)gridDim.x * kP2GWarps;
  uint32_t bad = 0;

  for (int t = lane; t < kP2GTileN + 1; t += 32) sm.tile[t] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (lane == 0) {
    mbar_init(&sm.bar, 1);
    fence_mbar_init();
  }
  __syncwarp();

  // One staging buffer: a step's rows go to registers first, then the next
  // step's copy is issued into the buffer and lands while this step computes.
  int q_next = 0, q_end = 0;  // lane 0's cursor in the run queue
  uint32_t parity = 0u;
  int g0 = step_queue_next(w, kP2GQueue, lane, nsteps, nwarps, q_next, q_end);
  if (g0 >= 0) p2g_issue<NR>(sm, rows_map, w, g0, lane);
  bool anchored = false;
  int o[3] = {0, 0, 0};

  while (g0 >= 0) {
    if (!mbar_wait(&sm.bar, parity)) {  // the staged rows never arrived: report and leave
      bad |= MPM_STATUS_TIMEOUT;
      anchored = false;
      break;
    }
    parity ^= 1u;
    const float *sb = &sm.buf[0][0];
    const int64_t i = (int64_t)g0 * 32 + lane;
    bool act = i < n;
    // this lane's particle, from the staged rows
    float x[3], v[3], C[3][3], F[3][3];
    ld_x<Q>(sb, 32, lane, x);
    ld_v<Q>(sb, 32, lane, v);
    ld_F<Q>(sb, 32, lane, F);
#pragma unroll
    for (int a = 0; a < 9; ++a) C[a / 3][a % 3] = sb[(R::C + a) * 32 + lane];
    float Jp = sb[R::Jp * 32 + lane];
    const int matword = ld_mat<Q>(sb, 32, lane);
    const float idf = sb[R::Id * 32 + lane];
    const float Ep = HAS_EP ? sb[R::Ep * 32 + lane] : 0.0f;
    float xw[2] = {sb[lane], sb[32 + lane]};  // position words (rows 0, 1 and, unpacked, 2)
    const float x2w = Q ? 0.0f : sb[2 * 32 + lane];
    float vw[3];  // velocity words, copied unchanged for stationary particles
#pragma unroll
    for (int r = 0; r < 3; ++r) vw[r] = (Q && r == 2) ? 0.0f : sb[(R::V + r) * 32 + lane];
    const int64_t j = __float_as_int(sb[NR * 32 + lane]);
    __syncwarp();
    // the buffer is free: stage the next step into it
    const int g1 = step_queue_next(w, kP2GQueue, lane, nsteps, nwarps, q_next, q_end);
    if (g1 >= 0) p2g_issue<NR>(sm, rows_map, w, g1, lane);

    if (act && (j < 0 || j >= n)) {
      bad |= MPM_STATUS_TABLE_OVERFLOW;
      act = false;
    }
    const int mat = matword & 0xFF;
    if (act) {
      // carried fields go to the sorted slot right away: the position words,
      // id and E unchanged, and a stationary particle's velocity (:722)
      nxt[j] = xw[0];
      nxt[cap + j] = xw[1];
      if (!Q) nxt[2 * cap + j] = x2w;
      nxt[R::Id * cap + j] = idf;
      if (HAS_EP) nxt[R::Ep * cap + j] = Ep;
      if (mat == 4) {
#pragma unroll
        for (int r = 0; r < (Q ? 2 : 3); ++r) nxt[(R::V + r) * cap + j] = vw[r];
      }
    }
    const MpmParams &S = scene_of_particle<BATCH>(P, tab, matword);
    uint32_t bad_base = 0;
    Base bs = particle_base(S, x[0], x[1], x[2], bad_base);
    if (act) bad |= bad_base;
    float mass = 0.f, q[3] = {0.f, 0.f, 0.f}, adx[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float wt[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    if (act) {
      const P2GOut out = constitutive(S, BATCH ? S.dt : dt, mat, Ep, F, Jp, C);
      st_F_mat<Q>(nxt, cap, j, F, matword);
      nxt[R::Jp * cap + j] = Jp;
      if (mat == 4) {  // stationary: G2P keeps v and C (:722)
#pragma unroll
        for (int a = 0; a < 9; ++a) nxt[(R::C + a) * cap + j] = C[a / 3][a % 3];
      }
      bspline_weights(bs.fx, wt);
      mass = out.mass;
      // APIC scatter, :576-584: node value = w * (m v + A (off - fx) dx)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        q[d] = out.mass * v[d] -
               S.dx * (out.affine[d][0] * bs.fx[0] + out.affine[d][1] * bs.fx[1] + out.affine[d][2] * bs.fx[2]);
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) adx[r][c] = out.affine[r][c] * S.dx;
    }
    p2g_scatter_step<false, ROLL>(P, w, sm.tile, o, anchored, act, bs, wt, mass, q, adx, lane);
    g0 = g1;
  }
  if (anchored) p2g_tile_flush<false>(P, w, sm.tile, o, lane);
  set_status(w, bad);
  step_queue_done(w, kP2GQueue, kP2GDone, lane, nwarps);
}

// --------------------------------------------------------------- grid ----

template <bool BATCH>
__global__ __launch_bounds__(256) void k_grid(const MpmParams P, const MpmParams *tab, const Ws w, float dt) {
  const int ng = w.counters[1];
  const int64_t total = (int64_t)ng * kBlockCells;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int blin = w.gblocks[t >> 6];
    const int l = (int)(t & 63);
    const int64_t addr = (int64_t)blin * kBlockCells + l;
    const float4 g = w.grid_mom[addr];
    w.grid_mom[addr] = make_float4(0.f, 0.f, 0.f, 0.f);
    // a fused substep flags the blocks it scatters into; the flags are used
    // up once the grid-active list is built
    if (l == 0) w.blk_flag[blin] = 0;
    int bx, by, bz;
    block_coords(P, blin, bx, by, bz);
    const MpmParams &S = scene_of_block<BATCH>(P, tab, bx, by, bz);
    const int I[3] = {S.win_lo[0] + bx * 4 + (l >> 4), S.win_lo[1] + by * 4 + ((l >> 2) & 3),
                      S.win_lo[2] + bz * 4 + (l & 3)};
    const float3 v = grid_node_update(S, I, g.x, make_float3(g.y, g.z, g.w), BATCH ? S.dt : dt);
    w.grid_vel[addr] = make_float4(v.x, v.y, v.z, g.x);
  }
}

// ---------------------------------------------------------------- G2P ----

// BIN selects the next substep's binning: kBinKeep - particles that stay in
// their cell keep their rank there (bin_one with the old key and rank; a
// particle that leaves marks its old rank in the old cell's leave mask, which
// k_scatter subtracts from the stayers'); kBinPlain - ranks from arrival
// order; kBinNone - no binning (the caller bins from scratch next time).
constexpr int kBinNone = 0, kBinPlain = 1, kBinKeep = 2;
template <bool BATCH, bool Q, int BIN>
__global__ __launch_bounds__(kG2PThreads, 8) void k_g2p(const MpmParams P, const MpmParams *tab, const Ws w,
                                                       float *__restrict__ st, int64_t cap, float dt,
                                                       float *maxv_out) {
  __shared__ float4 vt[kTileN];
  const int nitems = (int)min((int64_t)w.counters[2], w.items_cap);
  uint32_t bad = 0;
  float vmax = 0.0f;
  float bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
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
    __syncthreads();
    for (int j = start + threadIdx.x; j < end; j += blockDim.x) {
      float x[3];
      ld_x<Q>(st, cap, j, x);
      const int matword = ld_mat<Q>(st, cap, j);
      const int mat = matword & 0xFF;
      const MpmParams &S = scene_of_particle<BATCH>(P, tab, matword);
      const float s4 = 4.0f * S.inv_dx;
      const float dts = BATCH ? S.dt : dt;
      const Base b = particle_base(S, x[0], x[1], x[2], bad);
      float wt[3][3];
      bspline_weights(b.fx, wt);
      const int lx = b.b[0] - bx * 4, ly = b.b[1] - by * 4, lz = b.b[2] - bz * 4;
      if ((unsigned)lx > 3u || (unsigned)ly > 3u || (unsigned)lz > 3u) {  // moved since binning
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        continue;
      }
      // Gather, :711-721, in separable form.  Along each z-line (a, b) of
      // the stencil, T = sum_c w_c^z g and U = sum_c c w_c^z g; then with
      // W = w_a^x w_b^y:  v = sum W T,  C = 4 inv_dx (S - v (x) fx) where the
      // columns of S are sum a W T, sum b W T, sum W U.
      float nv[3] = {0.f, 0.f, 0.f}, sa[3] = {0.f, 0.f, 0.f}, sb[3] = {0.f, 0.f, 0.f},
            sc[3] = {0.f, 0.f, 0.f};
      const int base_node = (lx * kTileW + ly) * kTileW + lz;
      const float wz0 = wt[0][2], wz1 = wt[1][2], wz2x2 = 2.0f * wt[2][2], wz2 = wt[2][2];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) {
          const float4 *line = vt + base_node + (a * kTileW + bb) * kTileW;
          const float4 g0 = line[0], g1 = line[1], g2 = line[2];
          const float2 T01 = __ffma2_rn(f2(wz2, wz2), f2(g2.x, g2.y),
                                        __ffma2_rn(f2(wz1, wz1), f2(g1.x, g1.y), __fmul2_rn(f2(wz0, wz0), f2(g0.x, g0.y))));
          const float T2 = fmaf(wz2, g2.z, fmaf(wz1, g1.z, wz0 * g0.z));
          const float2 U01 = __ffma2_rn(f2(wz2x2, wz2x2), f2(g2.x, g2.y), __fmul2_rn(f2(wz1, wz1), f2(g1.x, g1.y)));
          const float U2 = fmaf(wz2x2, g2.z, wz1 * g1.z);
          const float W = wt[a][0] * wt[bb][1];
          const float T[3] = {T01.x, T01.y, T2}, U[3] = {U01.x, U01.y, U2};
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            nv[r] = fmaf(W, T[r], nv[r]);
            sc[r] = fmaf(W, U[r], sc[r]);
            if (a > 0) sa[r] = fmaf((float)a * W, T[r], sa[r]);
            if (bb > 0) sb[r] = fmaf((float)bb * W, T[r], sb[r]);
          }
        }
      float nC[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        nC[r][0] = s4 * fmaf(-nv[r], b.fx[0], sa[r]);
        nC[r][1] = s4 * fmaf(-nv[r], b.fx[1], sb[r]);
        nC[r][2] = s4 * fmaf(-nv[r], b.fx[2], sc[r]);
      }
      float vv[3];
      if (mat != 4) {  // :722-724; the advection reads the stored (rounded, when packed) v
#pragma unroll
        for (int d = 0; d < 3; ++d) vv[d] = nv[d];
        st_v<Q>(st, cap, j, vv, bad);
#pragma unroll
        for (int d = 0; d < 3; ++d) x[d] = x[d] + dts * vv[d];
        st_x<Q>(st, cap, j, x, bad);
#pragma unroll
        for (int a = 0; a < 9; ++a) st[(PRows<Q>::C + a) * cap + j] = nC[a / 3][a % 3];
      } else {
        ld_v<Q>(st, cap, j, vv);
      }
      vmax = fmaxf(vmax, fmaxf(fabsf(vv[0]), fmaxf(fabsf(vv[1]), fabsf(vv[2]))));
#pragma unroll
      for (int d = 0; d < 3; ++d) {  // fminf / fmaxf skip NaN positions
        bmin[d] = fminf(bmin[d], x[d]);
        bmax[d] = fmaxf(bmax[d], x[d]);
      }
      if (BIN == kBinKeep) {  // next substep's build_pid, keeping the rank of a stayer
        const int old_key = cell_key(P, b);
        const int r_old = w.slot_rank[j];
        const int key = bin_one<BATCH>(P, tab, w, j, x[0], x[1], x[2], matword, bad, old_key, r_old);
        if (key != old_key && (unsigned)r_old < 64u) atomicOr(&w.leave[old_key], 1ull << r_old);
      } else if (BIN == kBinPlain) {
        bin_one<BATCH>(P, tab, w, j, x[0], x[1], x[2], matword, bad);  // next substep's build_pid
      }
    }
    if (BATCH && maxv_out) {  // per-scene maximum, flushed per work item
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
      if ((threadIdx.x & 31) == 0 && vmax > 0.0f)
        atomicMax((int *)&maxv_out[scene_index_of_block<BATCH>(P, bx, by, bz)], __float_as_int(vmax));
      vmax = 0.0f;
    }
    __syncthreads();
  }
  set_status(w, bad);
  if (!BATCH && maxv_out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f) atomicMax((int *)maxv_out, __float_as_int(vmax));
  }
  if (!BATCH) {  // bounding box of the advected particles (the host sizes the grid window with it)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        bmin[d] = fminf(bmin[d], __shfl_xor_sync(0xffffffffu, bmin[d], o));
        bmax[d] = fmaxf(bmax[d], __shfl_xor_sync(0xffffffffu, bmax[d], o));
      }
      if ((threadIdx.x & 31) == 0 && bmin[d] <= bmax[d]) {
        atomicMin(&w.counters[kBoxMin + d], float_key_i32(bmin[d]));
        atomicMax(&w.counters[kBoxMax + d], float_key_i32(bmax[d]));
      }
    }
  }
}

// --------------------------------------------- fused plain substeps ----
//
// A frame of the plain substep loop (engine/mpm_solver.py:789-797) can run
// G2P of substep s-1 and P2G of substep s as one pass over the particles,
// with the state updated in place in its storage order:
//   sort       binning and the streaming P2G (k_p2g) into sorted order;
//   fused      k_fused: per warp step of 32 slots, G2P of the previous
//              substep at x (gather of the grid velocities through L1),
//              advection, the constitutive update with the new C and the
//              scatter at the new x into the warp's tile window; it flags the
//              blocks that receive momentum, which make the grid-active list;
//   close      k_g2p_stream: G2P of the last substep with the binning of the
//              next sort.
// The arithmetic is the plain substep's; only the order of the float32
// summations differs.  The storage order drifts from the positions while
// fused substeps run, so a frame re-sorts every few substeps.

constexpr int kFusedQueue = 7, kFusedDone = 8;  // counters[]: step queue, warps done

// Separable node addresses of the block-major grid around base b:
// addr(b + (a, bb, c)) = ax[a] + ay[bb] + az[c].
__device__ __forceinline__ void stencil_addresses(const MpmParams &P, const int (&b)[3], int (&ax)[3], int (&ay)[3],
                                                  int (&az)[3]) {
  const int SX = P.win_nb[1] * P.win_nb[2] * kBlockCells, SY = P.win_nb[2] * kBlockCells;
#pragma unroll
  for (int o = 0; o < 3; ++o) {
    const int gx = b[0] + o, gy = b[1] + o, gz = b[2] + o;
    ax[o] = (gx >> 2) * SX + (gx & 3) * 16;
    ay[o] = (gy >> 2) * SY + (gy & 3) * 4;
    az[o] = (gz >> 2) * kBlockCells + (gz & 3);
  }
}

// G2P gather (:711-721) straight from the grid velocities: v and C.
// ROLL: the x loop rolled (fewer registers, fewer loads in flight)
template <bool ROLL = false>
__device__ __forceinline__ void gather_vc(const MpmParams &P, float inv_dx, const float4 *__restrict__ gv,
                                          const Base &b, float (&nv)[3], float (&nC)[3][3]) {
  float wt[3][3];
  bspline_weights(b.fx, wt);
  int ax[3], ay[3], az[3];
  stencil_addresses(P, b.b, ax, ay, az);
  float sa[3] = {0.f, 0.f, 0.f}, sb[3] = {0.f, 0.f, 0.f}, sc[3] = {0.f, 0.f, 0.f};
  nv[0] = nv[1] = nv[2] = 0.0f;
  const float wz0 = wt[0][2], wz1 = wt[1][2], wz2 = wt[2][2], wz2x2 = 2.0f * wt[2][2];
#pragma unroll(ROLL ? 1 : 3)
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) {
      const int line = (a == 0 ? ax[0] : (a == 1 ? ax[1] : ax[2])) + ay[bb];
      const float4 g0 = __ldg(gv + line + az[0]), g1 = __ldg(gv + line + az[1]), g2 = __ldg(gv + line + az[2]);
      const float2 T01 =
          __ffma2_rn(f2(wz2, wz2), f2(g2.x, g2.y), __ffma2_rn(f2(wz1, wz1), f2(g1.x, g1.y), __fmul2_rn(f2(wz0, wz0), f2(g0.x, g0.y))));
      const float T2 = fmaf(wz2, g2.z, fmaf(wz1, g1.z, wz0 * g0.z));
      const float2 U01 = __ffma2_rn(f2(wz2x2, wz2x2), f2(g2.x, g2.y), __fmul2_rn(f2(wz1, wz1), f2(g1.x, g1.y)));
      const float U2 = fmaf(wz2x2, g2.z, wz1 * g1.z);
      const float W = (a == 0 ? wt[0][0] : (a == 1 ? wt[1][0] : wt[2][0])) * wt[bb][1];
      const float T[3] = {T01.x, T01.y, T2}, U[3] = {U01.x, U01.y, U2};
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        nv[r] = fmaf(W, T[r], nv[r]);
        sc[r] = fmaf(W, U[r], sc[r]);
        if (a > 0) sa[r] = fmaf((float)a * W, T[r], sa[r]);
        if (bb > 0) sb[r] = fmaf((float)bb * W, T[r], sb[r]);
      }
    }
  const float s4 = 4.0f * inv_dx;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    nC[r][0] = s4 * fmaf(-nv[r], b.fx[0], sa[r]);
    nC[r][1] = s4 * fmaf(-nv[r], b.fx[1], sb[r]);
    nC[r][2] = s4 * fmaf(-nv[r], b.fx[2], sc[r]);
  }
}

// Per-warp shared memory of the fused kernel: staged rows x (3) and F .. E
// (9 + Jp + material + id + E), the tile, the mbarrier.
constexpr int kFusedRowsF = 13;
struct __align__(128) FusedWarpSmem {
  float bx[3][32];  // 384 bytes: bf starts 128-byte aligned
  float bf[kFusedRowsF][32];
  float4 tile[kP2GTileN + 1];
  unsigned long long bar;
};
static_assert(offsetof(FusedWarpSmem, bf) % 128 == 0 && sizeof(FusedWarpSmem) % 128 == 0,
              "fused staging buffers must be 128-byte aligned");
constexpr size_t kFusedSmem = sizeof(FusedWarpSmem) * kP2GWarps;

// Stages step g of the fused kernel: rows x and F .. (NF rows from F on).
template <int NF>
__device__ __forceinline__ void fused_stage(FusedWarpSmem &sm, const CUtensorMap &map_x, const CUtensorMap &map_f,
                                            int g, int lane) {
  if (lane == 0) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&sm.bar, (3 + NF) * 128);
    tma_load_2d(sm.bx[0], &map_x, g * 32, 0, &sm.bar);
    tma_load_2d(sm.bf[0], &map_f, g * 32, PRows<false>::F, &sm.bar);
  }
}

// Scene index in the material word of a batched particle (bits 8..30).
__device__ __forceinline__ int scene_index_of_particle(const MpmParams &P, int matword) {
  return min(max(matword >> 8, 0), P.n_scenes - 1);
}

// The max |v| of a warp's particles into maxv_out: one slot, or in batched
// mode the slot of the scene each lane's maximum belongs to.
template <bool BATCH>
__device__ __forceinline__ void flush_vmax(float *maxv_out, float vmax, int vscene, int lane) {
  if (!maxv_out) return;
  if constexpr (BATCH) {
    if (vmax > 0.0f) atomicMax((int *)&maxv_out[vscene], __float_as_int(vmax));
  } else {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, d));
    if (lane == 0 && vmax > 0.0f) atomicMax((int *)maxv_out, __float_as_int(vmax));
  }
}

// Modes of the fused kernel: the plain loop in place (G2P of substep s-1,
// P2G of substep s), and the G2P2G mode (engine/mpm_solver.py:363-485) in
// place or writing every state row to the particle's sorted slot inv[i] of
// another buffer (the substep that re-sorts).
// In place the G2P2G mode stores v only at a frame's last substep
// (kFusedG2P2GLast): the next substep gathers v afresh, except for stationary
// particles, whose stored v never changes.
constexpr int kFusedPlain = 0, kFusedG2P2G = 1, kFusedG2P2GSorted = 2, kFusedG2P2GLast = 3;

template <bool HAS_EP, int MODE, bool BATCH = false, bool ROLL = false>
__global__ __launch_bounds__(kP2GThreads, ROLL ? 4 : MPM_P2G_MIN_CTAS) void k_fused(const MpmParams P,
                                                                                   const MpmParams *tab,
                                                                          const Ws w,
                                                                          const __grid_constant__ CUtensorMap map_x,
                                                                          const __grid_constant__ CUtensorMap map_f,
                                                                          float *__restrict__ st,
                                                                          float *__restrict__ out, int64_t cap,
                                                                          int64_t n, float dt, int64_t first_new,
                                                                          float *maxv_out) {
  using R = PRows<false>;
  constexpr bool G2P2G = MODE != kFusedPlain;
  constexpr bool SORTED = MODE == kFusedG2P2GSorted;
  // ROLL rolls the scatter's x loop (4 CTAs, 16 warps per SM).  The plain
  // mode without per-particle E keeps its gather unrolled within that budget
  // (8 B of spills; 16M / 2M scenes: 1.445 / 0.320 ms per launch against
  // 1.540 / 0.323 with both loops rolled); the other modes and the batched
  // form roll both (they would spill 24-66 B).
  constexpr bool ROLL_GATHER = ROLL && (G2P2G || HAS_EP || BATCH);
  static_assert(!(BATCH && G2P2G), "the batched form runs the plain loop");
  // staged rows from F on: F, Jp, material[, id][, E].  Only the sorted pass
  // needs the id: particles added since the last substep (id >= first_new)
  // exist only at a frame's first substep, which always sorts
  constexpr int NF = HAS_EP ? kFusedRowsF : (SORTED ? kFusedRowsF - 1 : kFusedRowsF - 2);
  extern __shared__ __align__(128) unsigned char fused_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  FusedWarpSmem &sm = reinterpret_cast<FusedWarpSmem *>(fused_smem)[warp];
  const int nsteps = (int)((n + 31) / 32);
  const int nwarps = (int)gridDim.x * kP2GWarps;
  uint32_t bad = 0;
  float vmax = 0.0f;
  int vscene = 0;  // batched: the scene vmax belongs to (per lane)
  for (int t = lane; t < kP2GTileN + 1; t += 32) sm.tile[t] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (lane == 0) {
    mbar_init(&sm.bar, 1);
    fence_mbar_init();
  }
  __syncwarp();
  int q_next = 0, q_end = 0;
  uint32_t parity = 0u;
  int g0 = step_queue_next(w, kFusedQueue, lane, nsteps, nwarps, q_next, q_end);
  if (g0 >= 0) fused_stage<NF>(sm, map_x, map_f, g0, lane);
  bool anchored = false;
  int o[3] = {0, 0, 0};
  while (g0 >= 0) {
    if (!mbar_wait(&sm.bar, parity)) {
      bad |= MPM_STATUS_TIMEOUT;
      anchored = false;
      break;
    }
    parity ^= 1u;
    float x[3], F[3][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) x[d] = sm.bx[d][lane];
#pragma unroll
    for (int a = 0; a < 9; ++a) F[a / 3][a % 3] = sm.bf[a][lane];
    float Jp = sm.bf[9][lane];
    const int matword = __float_as_int(sm.bf[10][lane]);
    const int idword = SORTED ? __float_as_int(sm.bf[11][lane]) : 0;
    const float Ep = HAS_EP ? sm.bf[12][lane] : 0.0f;
    __syncwarp();
    const int g1 = step_queue_next(w, kFusedQueue, lane, nsteps, nwarps, q_next, q_end);
    if (g1 >= 0) fused_stage<NF>(sm, map_x, map_f, g1, lane);
    const int64_t i = (int64_t)g0 * 32 + lane;
    bool act = i < n;
    int64_t j = i;  // where the particle's state goes
    if (SORTED && act) {
      j = w.inv[i];
      if (j < 0 || j >= n) {  // no sorted slot: the binning was not of this state
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        act = false;
      }
    }
    const int mat = matword & 0xFF;
    const MpmParams &S = scene_of_particle<BATCH>(P, tab, matword);
    const float dts = BATCH ? S.dt : dt;
    float v[3] = {0.f, 0.f, 0.f}, C[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    uint32_t bad_b = 0;
    if (act) {
      const Base b0 = particle_base(S, x[0], x[1], x[2], bad_b);
      if (!G2P2G) {
        // G2P of the previous substep, :694-724.  v and C feed this P2G only:
        // the next substep gathers them afresh and the frame's closing G2P
        // (k_g2p_stream) stores the final ones
        if (mat != 4) {
          gather_vc<ROLL_GATHER>(P, S.inv_dx, w.grid_vel, b0, v, C);
#pragma unroll
          for (int d = 0; d < 3; ++d) x[d] = x[d] + dts * v[d];
        } else {  // stationary: v, C and x stay
#pragma unroll
          for (int d = 0; d < 3; ++d) v[d] = st[(R::V + d) * cap + i];
#pragma unroll
          for (int a = 0; a < 9; ++a) C[a / 3][a % 3] = st[(R::C + a) * cap + i];
        }
      } else {
        // G2P from the previous substep's grid, :373-408: particles added
        // since then keep their v with C = 0; stationary particles gather C
        // but keep v and x
        const bool fresh = SORTED && (int64_t)(uint32_t)idword >= first_new;
        if (!fresh) gather_vc<ROLL_GATHER>(P, S.inv_dx, w.grid_vel, b0, v, C);
        if (mat == 4 || fresh) {
#pragma unroll
          for (int d = 0; d < 3; ++d) v[d] = st[(R::V + d) * cap + i];
        }
        if (mat != 4) {
#pragma unroll
          for (int d = 0; d < 3; ++d) x[d] = x[d] + dt * v[d];
        }
      }
      const float vm = fmaxf(fabsf(v[0]), fmaxf(fabsf(v[1]), fabsf(v[2])));
      if (BATCH) {
        const int sc = scene_index_of_particle(P, matword);
        if (sc != vscene) {  // per-scene maxima: flush when this lane's scene changes
          if (maxv_out && vmax > 0.0f) atomicMax((int *)&maxv_out[vscene], __float_as_int(vmax));
          vmax = 0.0f;
          vscene = sc;
        }
      }
      vmax = fmaxf(vmax, vm);
    }
    // P2G of this substep at the advected x, :487-584 (:410-485)
    Base bs = particle_base(S, x[0], x[1], x[2], bad_b);
    if (act) bad |= bad_b;
    float mass = 0.f, q[3] = {0.f, 0.f, 0.f}, adx[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float wt[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    if (act) {
      const P2GOut cu = constitutive<G2P2G, false>(S, dts, mat, Ep, F, Jp, C);
      float *dst = SORTED ? out : st;
#pragma unroll
      for (int a = 0; a < 9; ++a) dst[(R::F + a) * cap + j] = F[a / 3][a % 3];
      dst[R::Jp * cap + j] = Jp;
      if (!G2P2G && mat != 4) {  // the advected x
#pragma unroll
        for (int d = 0; d < 3; ++d) dst[(R::X + d) * cap + j] = x[d];
      }
      if (G2P2G && !SORTED && mat != 4) {  // in place: x, and v at the frame's last substep
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          dst[(R::X + d) * cap + j] = x[d];
          if (MODE == kFusedG2P2GLast) dst[(R::V + d) * cap + j] = v[d];
        }
      }
      if (SORTED) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          dst[(R::X + d) * cap + j] = x[d];
          dst[(R::V + d) * cap + j] = v[d];
        }
        dst[R::Mat * cap + j] = __int_as_float(matword);
        dst[R::Id * cap + j] = __int_as_float(idword);
        if (HAS_EP) dst[R::Ep * cap + j] = Ep;
      }
      bspline_weights(bs.fx, wt);
      mass = cu.mass;
#pragma unroll
      for (int d = 0; d < 3; ++d)
        q[d] = cu.mass * v[d] -
               S.dx * (cu.affine[d][0] * bs.fx[0] + cu.affine[d][1] * bs.fx[1] + cu.affine[d][2] * bs.fx[2]);
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) adx[r][c] = cu.affine[r][c] * S.dx;
    }
    p2g_scatter_step<true, ROLL>(P, w, sm.tile, o, anchored, act, bs, wt, mass, q, adx, lane);
    g0 = g1;
  }
  if (anchored) p2g_tile_flush<true>(P, w, sm.tile, o, lane);
  set_status(w, bad);
  flush_vmax<BATCH>(maxv_out, vmax, vscene, lane);
  step_queue_done(w, kFusedQueue, kFusedDone, lane, nwarps);
}

// Plain binning of every particle of `st` in storage order (the counts the
// next sort finalizes) and, when `box` is set, the particles' bounding box.
__global__ __launch_bounds__(256) void k_bin_box(const MpmParams P, const Ws w, const float *__restrict__ st,
                                                 int64_t cap, int64_t n, int box) {
  using R = PRows<false>;
  uint32_t bad = 0;
  float bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    float x[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      x[d] = st[(R::X + d) * cap + i];
      bmin[d] = fminf(bmin[d], x[d]);
      bmax[d] = fmaxf(bmax[d], x[d]);
    }
    bin_one<false>(P, nullptr, w, i, x[0], x[1], x[2], 0, bad);
  }
  set_status(w, bad);
  if (box) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        bmin[d] = fminf(bmin[d], __shfl_xor_sync(0xffffffffu, bmin[d], o));
        bmax[d] = fmaxf(bmax[d], __shfl_xor_sync(0xffffffffu, bmax[d], o));
      }
      if ((threadIdx.x & 31) == 0 && bmin[d] <= bmax[d]) {
        atomicMin(&w.counters[kBoxMin + d], float_key_i32(bmin[d]));
        atomicMax(&w.counters[kBoxMax + d], float_key_i32(bmax[d]));
      }
    }
  }
}

// G2P of the last substep of a fused run, in the storage order, with the
// plain binning for the next sort (in-cell ranks from arrival order: the
// storage order no longer matches the last sort's ranks), the max |v| and
// the particles' bounding box.
template <bool BATCH>
__global__ __launch_bounds__(128, 5) void k_g2p_stream(const MpmParams P, const MpmParams *tab, const Ws w,
                                                      float *__restrict__ st, int64_t cap, int64_t n, float dt,
                                                      float *maxv_out) {
  using R = PRows<false>;
  const int lane = threadIdx.x & 31;
  const int nsteps = (int)((n + 31) / 32);
  const int nwarps = (int)gridDim.x * (blockDim.x >> 5);
  uint32_t bad = 0;
  float vmax = 0.0f;
  int vscene = 0;
  float bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  int q_next = 0, q_end = 0;
  for (int g = step_queue_next(w, kFusedQueue, lane, nsteps, nwarps, q_next, q_end); g >= 0;
       g = step_queue_next(w, kFusedQueue, lane, nsteps, nwarps, q_next, q_end)) {
    const int64_t j = (int64_t)g * 32 + lane;
    if (j >= n) continue;
    float x[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) x[d] = st[(R::X + d) * cap + j];
    const int matword = __float_as_int(st[R::Mat * cap + j]);
    const MpmParams &S = scene_of_particle<BATCH>(P, tab, matword);
    const Base b = particle_base(S, x[0], x[1], x[2], bad);
    float vv[3];
    if ((matword & 0xFF) != 4) {
      float nC[3][3];
      gather_vc(P, S.inv_dx, w.grid_vel, b, vv, nC);
      const float dts = BATCH ? S.dt : dt;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        st[(R::V + d) * cap + j] = vv[d];
        x[d] = x[d] + dts * vv[d];
        st[(R::X + d) * cap + j] = x[d];
      }
#pragma unroll
      for (int a = 0; a < 9; ++a) st[(R::C + a) * cap + j] = nC[a / 3][a % 3];
    } else {
#pragma unroll
      for (int d = 0; d < 3; ++d) vv[d] = st[(R::V + d) * cap + j];
    }
    if (BATCH) {
      const int sc = scene_index_of_particle(P, matword);
      if (sc != vscene) {
        if (maxv_out && vmax > 0.0f) atomicMax((int *)&maxv_out[vscene], __float_as_int(vmax));
        vmax = 0.0f;
        vscene = sc;
      }
    }
    vmax = fmaxf(vmax, fmaxf(fabsf(vv[0]), fmaxf(fabsf(vv[1]), fabsf(vv[2]))));
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      bmin[d] = fminf(bmin[d], x[d]);
      bmax[d] = fmaxf(bmax[d], x[d]);
    }
    bin_one<BATCH>(P, tab, w, j, x[0], x[1], x[2], matword, bad);
  }
  set_status(w, bad);
  flush_vmax<BATCH>(maxv_out, vmax, vscene, lane);
  if constexpr (!BATCH) {  // the batched window is fixed by its slots: no bounding box
#pragma unroll
    for (int d = 0; d < 3; ++d) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        bmin[d] = fminf(bmin[d], __shfl_xor_sync(0xffffffffu, bmin[d], o));
        bmax[d] = fmaxf(bmax[d], __shfl_xor_sync(0xffffffffu, bmax[d], o));
      }
      if (lane == 0 && bmin[d] <= bmax[d]) {
        atomicMin(&w.counters[kBoxMin + d], float_key_i32(bmin[d]));
        atomicMax(&w.counters[kBoxMax + d], float_key_i32(bmax[d]));
      }
    }
  }
  step_queue_done(w, kFusedQueue, kFusedDone, lane, nwarps);
}

// -------------------------------------------------------------- G2P2G ----
//
// The fused substep of use_g2p2g=True (engine/mpm_solver.py:363-485): per
// particle, G2P from the grid velocities of the previous substep at x
// (particles added since then keep their v with C = 0, :401-404), advection,
// the constitutive update with the gathered C (C is not stored), and P2G at
// the advected position into the momentum grid of this substep.  Work items
// are the blocks of the particles' positions before advection, so the
// scatter reaches the nodes [-1, 6] of the block per axis: an 8^3 float4 tile
// per warp, flushed like P2G.  A particle that moved more than one cell
// scatters straight to the grid with global atomics.  The new positions are
// binned for the next substep, as in G2P.

__device__ __forceinline__ float4 f4add(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

constexpr int kFusedTileW = 8;
constexpr int kFusedTileN = kFusedTileW * kFusedTileW * kFusedTileW;

template <bool Q>
__global__ __launch_bounds__(kFusedThreads, MPM_FUSED_MIN_CTAS) void k_g2p2g(const MpmParams P, const Ws w,
                                                                         const float *__restrict__ cur,
                                                                         float *__restrict__ nxt, int64_t cap,
                                                                         float dt, int64_t first_new,
                                                                         float *maxv_out) {
  __shared__ float4 vt[kTileN];
  __shared__ float4 tiles[kFusedWarps][kFusedTileN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float4 *tile = tiles[warp];
  const int nitems = (int)min((int64_t)w.counters[2], w.items_cap);
  const float s4 = 4.0f * P.inv_dx;
  uint32_t bad = 0;
  float vmax = 0.0f;
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
    for (int t = lane; t < kFusedTileN; t += 32) tile[t] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    for (int j0 = start + warp * 32; j0 < end; j0 += kFusedThreads) {
      const int j = j0 + lane;
      bool active = j < end;
      int64_t i = active ? w.pid[j] : 0;
      if (active && (i < 0 || i >= cap)) {
        bad |= MPM_STATUS_TABLE_OVERFLOW;
        active = false;
      }
      int cell = -1 - lane;  // unique per inactive lane
      bool direct = false;   // moved more than a cell: scatter with global atomics
      float mass = 0.f, q[3] = {0.f, 0.f, 0.f}, adx[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      float wt[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
      int tx0 = 0, ty0 = 0, tz0 = 0, gb[3] = {0, 0, 0};
      if (active) {
        using R = PRows<Q>;
        float x[3], v[3], F[3][3];
        ld_x<Q>(cur, cap, i, x);
        ld_v<Q>(cur, cap, i, v);
        ld_F<Q>(cur, cap, i, F);
        float Jp = cur[R::Jp * cap + i];
        const int matword = ld_mat<Q>(cur, cap, i);
        const int mat = matword & 0xFF;
        const float idf = cur[R::Id * cap + i];
        const float Ep = P.has_Ep ? cur[R::Ep * cap + i] : 0.0f;
        // ---- G2P at x (:373-404) ----
        const Base b = particle_base(P, x[0], x[1], x[2], bad);
        const int lx = b.b[0] - bx * 4, ly = b.b[1] - by * 4, lz = b.b[2] - bz * 4;
        float C[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        float nv[3] = {v[0], v[1], v[2]};
        if ((unsigned)lx > 3u || (unsigned)ly > 3u || (unsigned)lz > 3u) {
          bad |= MPM_STATUS_TABLE_OVERFLOW;
          active = false;
        } else if ((int64_t)__float_as_int(idf) < first_new) {
          float gw[3][3];
          bspline_weights(b.fx, gw);
          nv[0] = nv[1] = nv[2] = 0.0f;
          const int base_node = (lx * kTileW + ly) * kTileW + lz;
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int bb = 0; bb < 3; ++bb)
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const float4 g = vt[base_node + (a * kTileW + bb) * kTileW + c];
                const float wgt = gw[a][0] * gw[bb][1] * gw[c][2];
                const float dp[3] = {(float)a - b.fx[0], (float)bb - b.fx[1], (float)c - b.fx[2]};
                const float gv[3] = {g.x, g.y, g.z};
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                  nv[r] += wgt * gv[r];
#pragma unroll
                  for (int cc = 0; cc < 3; ++cc) C[r][cc] += s4 * wgt * gv[r] * dp[cc];
                }
              }
        }
        if (active) {
          using R = PRows<Q>;
          if (mat != 4) {  // :406-408
#pragma unroll
            for (int d = 0; d < 3; ++d) v[d] = nv[d];
            st_v<Q>(nxt, cap, j, v, bad);  // packed: the advection and P2G read the rounded v
#pragma unroll
            for (int d = 0; d < 3; ++d) x[d] = x[d] + dt * v[d];
            st_x<Q>(nxt, cap, j, x, bad);
          } else {
            st_v<Q>(nxt, cap, j, v, bad);  // loaded values re-encode to the same words
            st_x<Q>(nxt, cap, j, x, bad);
          }
          // ---- constitutive update and P2G at the new x (:410-485) ----
          const P2GOut o = constitutive<true, Q>(P, dt, mat, Ep, F, Jp, C);
          st_F_mat<Q>(nxt, cap, j, F, matword);
          nxt[R::Jp * cap + j] = Jp;
          nxt[R::Id * cap + j] = idf;
          if (P.has_Ep) nxt[R::Ep * cap + j] = Ep;
          vmax = fmaxf(vmax, fmaxf(fabsf(v[0]), fmaxf(fabsf(v[1]), fabsf(v[2]))));
          const Base b2 = particle_base(P, x[0], x[1], x[2], bad);
          bspline_weights(b2.fx, wt);
          mass = o.mass;
#pragma unroll
          for (int d = 0; d < 3; ++d)
            q[d] = o.mass * v[d] -
                   P.dx * (o.affine[d][0] * b2.fx[0] + o.affine[d][1] * b2.fx[1] + o.affine[d][2] * b2.fx[2]);
#pragma unroll
          for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) adx[r][c] = o.affine[r][c] * P.dx;
          tx0 = b2.b[0] - bx * 4 + 1;
          ty0 = b2.b[1] - by * 4 + 1;
          tz0 = b2.b[2] - bz * 4 + 1;
#pragma unroll
          for (int d = 0; d < 3; ++d) gb[d] = b2.b[d];
          if ((unsigned)tx0 > 5u || (unsigned)ty0 > 5u || (unsigned)tz0 > 5u) {
            direct = true;
          } else {
            cell = (tx0 * kFusedTileW + ty0) * kFusedTileW + tz0;
          }
          {  // next substep's build_pid, keeping the rank of a stayer (as in k_g2p)
            const int old_key = cell_key(P, b);
            const int r_old = w.slot_rank[j];
            const int key = bin_one<false>(P, nullptr, w, j, x[0], x[1], x[2], matword, bad, old_key, r_old);
            if (key != old_key && (unsigned)r_old < 64u) atomicOr(&w.leave[old_key], 1ull << r_old);
          }
        }
      }
      if (active && direct) {  // rare: straight to the grid
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int bb = 0; bb < 3; ++bb)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const int gx = gb[0] + a, gy = gb[1] + bb, gz = gb[2] + c;
              if (gx < 0 || gy < 0 || gz < 0 || gx >= P.win_nb[0] * 4 || gy >= P.win_nb[1] * 4 ||
                  gz >= P.win_nb[2] * 4)
                continue;
              const float wgt = wt[a][0] * wt[bb][1] * wt[c][2];
              float4 g;
              g.x = wgt * mass;
              g.y = wgt * (q[0] + adx[0][0] * (float)a + adx[0][1] * (float)bb + adx[0][2] * (float)c);
              g.z = wgt * (q[1] + adx[1][0] * (float)a + adx[1][1] * (float)bb + adx[1][2] * (float)c);
              g.w = wgt * (q[2] + adx[2][0] * (float)a + adx[2][1] * (float)bb + adx[2][2] * (float)c);
              atomicAdd(&w.grid_mom[node_addr(P, gx, gy, gz)], g);
            }
      }
      const bool tiled = active && !direct;
      const unsigned peers = __match_any_sync(0xffffffffu, cell);
      const int round_of_lane = __popc(peers & ((1u << lane) - 1u));
      const int base_node = (tiled ? (tx0 * kFusedTileW + ty0) * kFusedTileW + tz0 : 0);
      for (int round = 0;; ++round) {
        const bool mine = tiled && round_of_lane == round;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int bb = 0; bb < 3; ++bb) {
            const float wab = tiled ? wt[a][0] * wt[bb][1] : 0.0f;
            float pab[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) pab[d] = q[d] + adx[d][0] * (float)a + adx[d][1] * (float)bb;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float wgt = wab * wt[c][2];
              float4 *nd = tile + base_node + (a * kFusedTileW + bb) * kFusedTileW + c;
              float4 g = *nd;
              g.x = fmaf(wgt, mass, g.x);
              g.y = fmaf(wgt, fmaf(adx[0][2], (float)c, pab[0]), g.y);
              g.z = fmaf(wgt, fmaf(adx[1][2], (float)c, pab[1]), g.z);
              g.w = fmaf(wgt, fmaf(adx[2][2], (float)c, pab[2]), g.w);
              if (mine) *nd = g;
              __syncwarp();
            }
          }
        if (!__any_sync(0xffffffffu, tiled && round_of_lane > round)) break;
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kFusedTileN; t += blockDim.x) {
      float4 g = tiles[0][t];
#pragma unroll
      for (int wq = 1; wq < kFusedWarps; ++wq) g = f4add(g, tiles[wq][t]);
      if (g.x != 0.0f) {
        const int tx = t / 64, ty = (t / 8) % 8, tz = t % 8;
        const int gx = bx * 4 - 1 + tx, gy = by * 4 - 1 + ty, gz = bz * 4 - 1 + tz;
        if (gx >= 0 && gy >= 0 && gz >= 0 && gx < P.win_nb[0] * 4 && gy < P.win_nb[1] * 4 && gz < P.win_nb[2] * 4)
          atomicAdd(&w.grid_mom[node_addr(P, gx, gy, gz)], g);
      }
    }
    __syncthreads();
  }
  set_status(w, bad);
  if (maxv_out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f) atomicMax((int *)maxv_out, __float_as_int(vmax));
  }
}

// compute_max_grid_velocity (engine/mpm_solver.py:737-746): the largest |v_d|
// over the nodes of the grid-active blocks of the last substep; *out (a
// non-negative float) is raised with an integer atomic max
__global__ __launch_bounds__(256) void k_max_grid_velocity(const MpmParams P, const Ws w, float *out) {
  const int ng = w.counters[1];
  const int64_t total = (int64_t)ng * kBlockCells;
  float m = 0.0f;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float4 g = w.grid_vel[(int64_t)w.gblocks[t >> 6] * kBlockCells + (t & 63)];
    m = fmaxf(m, fmaxf(fabsf(g.x), fmaxf(fabsf(g.y), fabsf(g.z))));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax((int *)out, __float_as_int(m));
}

// The constitutive update of P2G for n independent particles (the diagnostic
// entry mpm_constitutive_eval): F (row major), Jp updated in place, the APIC
// affine matrix written, by the same device code the P2G kernels run.
__global__ void k_constitutive_eval(const MpmParams P, int64_t n, const int32_t *__restrict__ material,
                                    float *__restrict__ F, const float *__restrict__ C, float *__restrict__ Jp,
                                    float *__restrict__ affine, float dt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float f[3][3], c[3][3];
#pragma unroll
  for (int a = 0; a < 9; ++a) {
    f[a / 3][a % 3] = F[9 * i + a];
    c[a / 3][a % 3] = C[9 * i + a];
  }
  float jp = Jp[i];
  const P2GOut o = constitutive<false, false>(P, dt, material[i] & 0xFF, 0.0f, f, jp, c);
#pragma unroll
  for (int a = 0; a < 9; ++a) {
    F[9 * i + a] = f[a / 3][a % 3];
    affine[9 * i + a] = o.affine[a / 3][a % 3];
  }
  Jp[i] = jp;
}

__global__ void k_gather_rows(const float *__restrict__ ps, int64_t cap, int64_t n, int row0, int ncols,
                              float *__restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int64_t id = __float_as_int(ps[kId * cap + j]);
  if (id < 0 || id >= n) return;  // corrupted id row: leave the slot untouched
  for (int c = 0; c < ncols; ++c) out[id * ncols + c] = ps[(row0 + c) * cap + j];
}

// ------------------------------------------------------------ host side --

// cuTensorMapEncodeTiled, looked up once through the runtime (no link
// against the driver library)
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// Tensor map of the first `rows` rows of a state buffer: a 2-D float32
// tensor of cap x rows elements (row stride cap), boxes of 32 slots x
// box_rows rows (box_rows = rows when 0).
static bool rows_tensor_map(CUtensorMap *map, const float *state, int64_t cap, int rows, int box_rows = 0) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cap, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cap * sizeof(float)};
  const cuuint32_t box[2] = {32u, (cuuint32_t)(box_rows > 0 ? box_rows : rows)};
  const cuuint32_t elem[2] = {1u, 1u};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(state), dims, strides, box, elem,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <bool HAS_EP, bool BATCH, bool Q, bool ROLL = BATCH>
static int launch_p2g(int ctas, cudaStream_t s, const MpmParams &p, const MpmParams *tab, const Ws &w,
                      const float *cur, float *nxt, int64_t cap, int64_t n, float dt) {
  if (n <= 0) return MPM_OK;
  CUtensorMap map;
  if (!rows_tensor_map(&map, cur, cap, P2GRows<Q, HAS_EP>::N)) return MPM_E_CUDA;
  k_p2g<HAS_EP, BATCH, Q, ROLL><<<ctas, kP2GThreads, kP2GSmem, s>>>(p, tab, w, map, cur, nxt, cap, n, dt);
  return MPM_OK;
}

template <bool HAS_EP, bool BATCH, bool Q, bool ROLL = BATCH>
static int p2g_occupancy() {
  auto k = k_p2g<HAS_EP, BATCH, Q, ROLL>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kP2GSmem);
  int c = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k, kP2GThreads, kP2GSmem);
  return c > 0 ? c : 1;
}

// P2G stages 128-byte row segments with bulk copies: row starts must be
// 16-byte aligned and whole 32-slot steps must lie inside the buffers.
static bool p2g_rows_ok(const void *cur, int64_t cap) {
  return cap % 32 == 0 && ((uintptr_t)cur & 15u) == 0;
}

struct DevInfo {
  int sms = 0;
  int p2g_ctas = 0, p2g_ep_ctas = 0, g2p_ctas = 0, g2p2g_ctas = 0;
  int p2g_b_ctas = 0, p2g_ep_b_ctas = 0, g2p_b_ctas = 0;
  int p2g_q_ctas = 0, p2g_ep_q_ctas = 0, g2p_q_ctas = 0, g2p2g_q_ctas = 0;  // packed storage
  int fused_ctas[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};  // k_fused [has_Ep][mode]
  int fused_b_ctas[2] = {0, 0};                    // batched k_fused [has_Ep]
  int fused_b_roll_ctas[2] = {0, 0};               // batched rolled k_fused [has_Ep]
  int fused_roll_ctas[2][2] = {{0, 0}, {0, 0}};    // rolled k_fused [has_Ep][plain, G2P2G in place]
  int p2g_roll_ctas[2] = {0, 0};                   // rolled k_p2g [has_Ep]
  int g2ps_ctas = 0, g2ps_b_ctas = 0, binbox_ctas = 0;
};

// CTAs of one full wave of k_fused<HAS_EP, MODE, BATCH> (its dynamic shared
// memory opted in first)
template <bool HAS_EP, int MODE, bool BATCH = false, bool ROLL = false>
static void fused_occupancy(int sms, int &ctas) {
  int k = 0;
  auto kern = k_fused<HAS_EP, MODE, BATCH, ROLL>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFusedSmem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, kern, kP2GThreads, kFusedSmem);
  ctas = sms * (k > 0 ? k : 1);
}

static DevInfo g_dev[64];
static std::mutex g_dev_mu;

static const DevInfo *dev_info() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  DevInfo &d = g_dev[dev];
  if (d.sms == 0) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return nullptr;
    int a = 0, b = 0, c = 0, a2 = 0, b2 = 0, c2 = 0;
    a = p2g_occupancy<false, false, false>();
    b = p2g_occupancy<true, false, false>();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_g2p<false, false, kBinKeep>, kG2PThreads, 0);
    a2 = p2g_occupancy<false, true, false>();
    b2 = p2g_occupancy<true, true, false>();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c2, k_g2p<true, false, kBinPlain>, kG2PThreads, 0);
    int f = 0, aq = 0, bq = 0, cq = 0, fq = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, k_g2p2g<false>, kFusedThreads, 0);
    aq = p2g_occupancy<false, false, true>();
    bq = p2g_occupancy<true, false, true>();
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cq, k_g2p<false, true, kBinKeep>, kG2PThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fq, k_g2p2g<true>, kFusedThreads, 0);
    d.g2p2g_ctas = sms * (f > 0 ? f : 1);
    d.p2g_q_ctas = sms * (aq > 0 ? aq : 1);
    d.p2g_ep_q_ctas = sms * (bq > 0 ? bq : 1);
    d.g2p_q_ctas = sms * (cq > 0 ? cq : 1);
    d.g2p2g_q_ctas = sms * (fq > 0 ? fq : 1);
    d.p2g_ctas = sms * (a > 0 ? a : 1);
    d.p2g_ep_ctas = sms * (b > 0 ? b : 1);
    d.g2p_ctas = sms * (c > 0 ? c : 1);
    d.p2g_b_ctas = sms * (a2 > 0 ? a2 : 1);
    d.p2g_ep_b_ctas = sms * (b2 > 0 ? b2 : 1);
    d.g2p_b_ctas = sms * (c2 > 0 ? c2 : 1);
    {
      fused_occupancy<false, kFusedPlain>(sms, d.fused_ctas[0][0]);
      fused_occupancy<true, kFusedPlain>(sms, d.fused_ctas[1][0]);
      fused_occupancy<false, kFusedG2P2G>(sms, d.fused_ctas[0][1]);
      fused_occupancy<true, kFusedG2P2G>(sms, d.fused_ctas[1][1]);
      fused_occupancy<false, kFusedG2P2GSorted>(sms, d.fused_ctas[0][2]);
      fused_occupancy<true, kFusedG2P2GSorted>(sms, d.fused_ctas[1][2]);
      fused_occupancy<false, kFusedG2P2GLast>(sms, d.fused_ctas[0][3]);
      fused_occupancy<true, kFusedG2P2GLast>(sms, d.fused_ctas[1][3]);
      fused_occupancy<false, kFusedPlain, true>(sms, d.fused_b_ctas[0]);
      fused_occupancy<true, kFusedPlain, true>(sms, d.fused_b_ctas[1]);
      fused_occupancy<false, kFusedPlain, false, true>(sms, d.fused_roll_ctas[0][0]);
      fused_occupancy<true, kFusedPlain, false, true>(sms, d.fused_roll_ctas[1][0]);
      fused_occupancy<false, kFusedG2P2G, false, true>(sms, d.fused_roll_ctas[0][1]);
      fused_occupancy<true, kFusedG2P2G, false, true>(sms, d.fused_roll_ctas[1][1]);
      fused_occupancy<false, kFusedPlain, true, true>(sms, d.fused_b_roll_ctas[0]);
      fused_occupancy<true, kFusedPlain, true, true>(sms, d.fused_b_roll_ctas[1]);
      d.p2g_roll_ctas[0] = sms * p2g_occupancy<false, false, false, true>();
      d.p2g_roll_ctas[1] = sms * p2g_occupancy<true, false, false, true>();
      int gs = 0, gsb = 0, bb = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gs, k_g2p_stream<false>, 128, 0);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gsb, k_g2p_stream<true>, 128, 0);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bb, k_bin_box, 256, 0);
      d.g2ps_ctas = sms * (gs > 0 ? gs : 1);
      d.g2ps_b_ctas = sms * (gsb > 0 ? gsb : 1);
      d.binbox_ctas = sms * (bb > 0 ? bb : 1);
    }
    d.sms = sms;
  }
  return &d;
}

// P2G of a single scene in the parameters' storage layout
static int launch_p2g_single(const DevInfo *di, cudaStream_t s, const MpmParams &p, const Ws &w, const float *cur,
                             float *nxt, int64_t cap, int64_t n, float dt) {
  if (p.quant)
    return p.has_Ep ? launch_p2g<true, false, true>(di->p2g_ep_q_ctas, s, p, nullptr, w, cur, nxt, cap, n, dt)
                    : launch_p2g<false, false, true>(di->p2g_q_ctas, s, p, nullptr, w, cur, nxt, cap, n, dt);
  if (p.occupancy)  // rolled, 16 warps per SM
    return p.has_Ep ? launch_p2g<true, false, false, true>(di->p2g_roll_ctas[1], s, p, nullptr, w, cur, nxt, cap, n, dt)
                    : launch_p2g<false, false, false, true>(di->p2g_roll_ctas[0], s, p, nullptr, w, cur, nxt, cap, n,
                                                            dt);
  return p.has_Ep ? launch_p2g<true, false, false>(di->p2g_ep_ctas, s, p, nullptr, w, cur, nxt, cap, n, dt)
                  : launch_p2g<false, false, false>(di->p2g_ctas, s, p, nullptr, w, cur, nxt, cap, n, dt);
}

static bool params_ok(const MpmParams *p) {
  if (!p || p->version != MPM_ABI_VERSION) return false;
  for (int d = 0; d < 3; ++d) {
    if (p->win_nb[d] <= 0 || (p->win_lo[d] & 3) != 0) return false;
  }
  const int64_t nblk = (int64_t)p->win_nb[0] * p->win_nb[1] * p->win_nb[2];
  if (nblk * kBlockCells >= (int64_t)INT32_MAX) return false;
  if (p->chunk < 32 || (p->chunk & 31) != 0) return false;
  if (p->n_colliders < 0 || p->n_colliders > MPM_MAX_COLLIDERS) return false;
  return true;
}

static int last_error() { return cudaGetLastError() == cudaSuccess ? MPM_OK : MPM_E_CUDA; }

// ------------------------------------------- allocation-free substep ----
//
// Scratch of mpm_substep_noalloc: a file-scope device array, so callers that
// cannot allocate device memory can still run a substep.  Every device that
// loads this library keeps these bytes for the life of the process.  Host
// code must not use `g_static_scratch` as a pointer (on the host it names a
// stand-in object); its device address is looked up once per device with
// cudaGetSymbolAddress and passed to the kernels.
constexpr size_t kStaticScratchBytes = size_t(16) << 20;  // 16 MiB
constexpr int64_t kStaticMaxParticles = 65536;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static void *g_static_addr[64];
static std::mutex g_static_mu;

// Device address of the static scratch on the current device (set up on the
// first call per device).
static int static_scratch_addr(void **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MPM_E_CUDA;
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_addr[dev]) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_static_scratch) != cudaSuccess || !ptr) return MPM_E_CUDA;
    g_static_addr[dev] = ptr;
  }
  *out = g_static_addr[dev];
  return MPM_OK;
}

}  // namespace mpm

using namespace mpm;

extern "C" {

int mpm_abi_version(void) { return MPM_ABI_VERSION; }

int mpm_workspace_bytes(const MpmParams *p, int64_t cap, size_t *bytes_out) {
  if (!params_ok(p) || cap <= 0 || cap >= (int64_t)INT32_MAX || !bytes_out) return MPM_E_INVALID;
  *bytes_out = ws_layout(*p, cap, nullptr, nullptr);
  return MPM_OK;
}

int mpm_workspace_init(const MpmParams *p, void *ws, int64_t cap, void *stream) {
  if (!params_ok(p) || !ws) return MPM_E_INVALID;
  const size_t bytes = ws_layout(*p, cap, nullptr, nullptr);
  if (cudaMemsetAsync(ws, 0, bytes, (cudaStream_t)stream) != cudaSuccess) return MPM_E_CUDA;
  return MPM_OK;
}

int mpm_bin_count(const MpmParams *p, void *ws, int64_t cap, const float *pstate, int64_t begin, int64_t end,
                  void *stream) {
  if (!params_ok(p) || !ws || !pstate || begin < 0 || end > cap || begin > end) return MPM_E_INVALID;
  if (end == begin) return MPM_OK;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  const int64_t n = end - begin;
  const unsigned nb = (unsigned)((n + 255) / 256);
  if (p->quant)
    k_bin_count<false, true><<<nb, 256, 0, (cudaStream_t)stream>>>(*p, nullptr, w, pstate, cap, begin, end);
  else
    k_bin_count<false, false><<<nb, 256, 0, (cudaStream_t)stream>>>(*p, nullptr, w, pstate, cap, begin, end);
  return last_error();
}

int mpm_bin_finalize(const MpmParams *p, void *ws, int64_t cap, int64_t n, void *stream) {
  if (!params_ok(p) || !ws || n < 0 || n > cap) return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  cudaStream_t s = (cudaStream_t)stream;
  k_flags_count<<<w.nflagtiles, 256, 0, s>>>(*p, w);
  k_flags_write<<<w.nflagtiles, 256, 0, s>>>(*p, w);
  k_pb_stats<<<w.nstattiles, 256, 0, s>>>(*p, w);
  k_pb_scan<<<w.nstattiles, 256, 0, s>>>(*p, w);
  k_pb_levels<<<di->sms * 8, 256, 0, s>>>(*p, w, cap);
  if (n > 0) k_scatter<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(*p, w, n);
  k_cell_clear<<<di->sms * 8, 256, 0, s>>>(*p, w);
  return last_error();
}

int mpm_p2g(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float *nxt, float dt,
            void *stream) {
  if (!params_ok(p) || !ws || !cur || !nxt || n < 0 || n > cap || !p2g_rows_ok(cur, cap)) return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  cudaStream_t s = (cudaStream_t)stream;
  const int rc = launch_p2g_single(di, s, *p, w, cur, nxt, cap, n, dt);
  return rc ? rc : last_error();
}

int mpm_grid_update(const MpmParams *p, void *ws, int64_t cap, float dt, void *stream) {
  if (!params_ok(p) || !ws) return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  k_grid<false><<<di->sms * 8, 256, 0, (cudaStream_t)stream>>>(*p, nullptr, w, dt);
  return last_error();
}

int mpm_g2p(const MpmParams *p, void *ws, int64_t cap, int64_t n, float *nxt, float dt, float *maxv_out,
            void *stream) {
  if (!params_ok(p) || !ws || !nxt || n < 0 || n > cap) return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  if (p->quant)
    k_g2p<false, true, kBinKeep><<<di->g2p_q_ctas, kG2PThreads, 0, (cudaStream_t)stream>>>(*p, nullptr, w, nxt, cap, dt,
                                                                                 maxv_out);
  else
    k_g2p<false, false, kBinKeep><<<di->g2p_ctas, kG2PThreads, 0, (cudaStream_t)stream>>>(*p, nullptr, w, nxt, cap, dt,
                                                                                maxv_out);
  return last_error();
}

int mpm_g2p_bin_into(const MpmParams *p, void *ws, void *ws_bins, int64_t cap, int64_t n, float *nxt, float dt,
                     float *maxv_out, void *stream) {
  if (!params_ok(p) || p->quant || !ws || !ws_bins || !nxt || n < 0 || n > cap) return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w, wb;
  ws_layout(*p, cap, (char *)ws, &w);
  ws_layout(*p, cap, (char *)ws_bins, &wb);
  // the grid, sorted order and status stay with `ws`; only the next
  // substep's cell counts, block flags, cell keys and rank records go to
  // `ws_bins`
  w.cell_cnt = wb.cell_cnt;
  w.blk_flag = wb.blk_flag;
  w.cellkey = wb.cellkey;
  w.stay_rank = wb.stay_rank;
  w.arr_cnt = wb.arr_cnt;
  k_g2p<false, false, kBinPlain><<<di->g2p_ctas, kG2PThreads, 0, (cudaStream_t)stream>>>(*p, nullptr, w, nxt, cap,
                                                                                         dt, maxv_out);
  return last_error();
}

int mpm_g2p2g_substep(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float *nxt,
                      float dt, int64_t first_new, int32_t finalize_first, float *maxv_out, void *stream) {
  if (!params_ok(p) || p->n_scenes > 0 || !ws || !cur || !nxt || n < 0 || n > cap || first_new < 0)
    return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  int rc = MPM_OK;
  if (finalize_first) {
    rc = mpm_bin_finalize(p, ws, cap, n, stream);
    if (rc) return rc;
  }
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  if (p->quant)
    k_g2p2g<true><<<di->g2p2g_q_ctas, kFusedThreads, 0, (cudaStream_t)stream>>>(*p, w, cur, nxt, cap, dt, first_new,
                                                                              maxv_out);
  else
    k_g2p2g<false><<<di->g2p2g_ctas, kFusedThreads, 0, (cudaStream_t)stream>>>(*p, w, cur, nxt, cap, dt, first_new,
                                                                             maxv_out);
  rc = last_error();
  if (rc) return rc;
  rc = mpm_bin_finalize(p, ws, cap, n, stream);
  if (rc) return rc;
  return mpm_grid_update(p, ws, cap, dt, stream);
}

int mpm_substep(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float *nxt, float dt,
                float *maxv_out, void *stream) {
  if (!cur || !p2g_rows_ok(cur, cap)) return MPM_E_INVALID;  // checked before any device work
  int rc = mpm_bin_finalize(p, ws, cap, n, stream);
  if (rc) return rc;
  rc = mpm_p2g(p, ws, cap, n, cur, nxt, dt, stream);
  if (rc) return rc;
  rc = mpm_grid_update(p, ws, cap, dt, stream);
  if (rc) return rc;
  return mpm_g2p(p, ws, cap, n, nxt, dt, maxv_out, stream);
}

// The particle kernel of a fused substep on `st`: the G2P of the previous
// substep, advection, the constitutive update and the P2G of this one (MODE:
// the plain loop in place, or the G2P2G mode in place or into `out` sorted;
// BATCH: the plain loop over the scenes of a batch, `tab` their parameters).
extern "C++" {
template <int MODE, bool BATCH = false>
static int fused_particles(const DevInfo *di, cudaStream_t s, const MpmParams &p, const MpmParams *tab, const Ws &w,
                           float *st, float *out, int64_t cap, int64_t n, float dt, int64_t first_new, float *maxv) {
  CUtensorMap mx, mf;
  const int nf = p.has_Ep ? kFusedRowsF : (MODE == kFusedG2P2GSorted ? kFusedRowsF - 1 : kFusedRowsF - 2);
  if (!rows_tensor_map(&mx, st, cap, MPM_NROWS, 3) || !rows_tensor_map(&mf, st, cap, MPM_NROWS, nf))
    return MPM_E_CUDA;
  const int ep = p.has_Ep ? 1 : 0;
  if constexpr (!BATCH && (MODE == kFusedPlain || MODE == kFusedG2P2G)) {
    if (p.occupancy) {  // rolled, 16 warps per SM
      constexpr int R = MODE == kFusedPlain ? 0 : 1;
      if (p.has_Ep)
        k_fused<true, MODE, false, true><<<di->fused_roll_ctas[1][R], kP2GThreads, kFusedSmem, s>>>(
            p, tab, w, mx, mf, st, out, cap, n, dt, first_new, maxv);
      else
        k_fused<false, MODE, false, true><<<di->fused_roll_ctas[0][R], kP2GThreads, kFusedSmem, s>>>(
            p, tab, w, mx, mf, st, out, cap, n, dt, first_new, maxv);
      return MPM_OK;
    }
  }
  if constexpr (BATCH && MODE == kFusedPlain) {
    if (p.occupancy) {  // rolled, 16 warps per SM
      if (p.has_Ep)
        k_fused<true, MODE, true, true><<<di->fused_b_roll_ctas[1], kP2GThreads, kFusedSmem, s>>>(
            p, tab, w, mx, mf, st, out, cap, n, dt, first_new, maxv);
      else
        k_fused<false, MODE, true, true><<<di->fused_b_roll_ctas[0], kP2GThreads, kFusedSmem, s>>>(
            p, tab, w, mx, mf, st, out, cap, n, dt, first_new, maxv);
      return MPM_OK;
    }
  }
  const int ctas = BATCH ? di->fused_b_ctas[ep] : di->fused_ctas[ep][MODE];
  if (p.has_Ep)
    k_fused<true, MODE, BATCH><<<ctas, kP2GThreads, kFusedSmem, s>>>(p, tab, w, mx, mf, st, out, cap, n, dt,
                                                                    first_new, maxv);
  else
    k_fused<false, MODE, BATCH><<<ctas, kP2GThreads, kFusedSmem, s>>>(p, tab, w, mx, mf, st, out, cap, n, dt,
                                                                     first_new, maxv);
  return MPM_OK;
}
}  // extern "C++"

// The grid half of a fused substep: the blocks the particles marked become
// the grid-active list, then the grid update over them (`tab`: the scene
// table of a batch, else null).
static void fused_grid(cudaStream_t s, const DevInfo *di, const MpmParams &p, const MpmParams *tab, const Ws &w,
                       float dt) {
  k_flags_count<<<w.nflagtiles, 256, 0, s>>>(p, w);
  k_flags_write<<<w.nflagtiles, 256, 0, s>>>(p, w);
  if (tab)
    k_grid<true><<<di->sms * 8, 256, 0, s>>>(p, tab, w, 0.0f);
  else
    k_grid<false><<<di->sms * 8, 256, 0, s>>>(p, nullptr, w, dt);
}

static bool batch_ok(const MpmParams *p) {
  if (!params_ok(p) || p->n_scenes < 1 || p->quant) return false;
  int64_t slots = 1;
  for (int d = 0; d < 3; ++d) {
    if (p->slot_nb[d] <= 0 || p->slots[d] <= 0) return false;
    if ((int64_t)p->slot_nb[d] * p->slots[d] > p->win_nb[d]) return false;
    slots *= p->slots[d];
  }
  return slots >= p->n_scenes;
}

int mpm_batch_bin_count(const MpmParams *p, const MpmParams *scenes, void *ws, int64_t cap, const float *pstate,
                        int64_t begin, int64_t end, void *stream) {
  if (!batch_ok(p) || !scenes || !ws || !pstate || begin < 0 || end > cap || begin > end) return MPM_E_INVALID;
  if (end == begin) return MPM_OK;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  const int64_t n = end - begin;
  k_bin_count<true, false><<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(*p, scenes, w, pstate, cap,
                                                                                         begin, end);
  return last_error();
}

int mpm_batch_substep(const MpmParams *p, const MpmParams *scenes, void *ws, int64_t cap, int64_t n,
                      const float *cur, float *nxt, float *maxv_out, void *stream) {
  if (!batch_ok(p) || !scenes || !ws || !cur || !nxt || n < 0 || n > cap || !p2g_rows_ok(cur, cap))
    return MPM_E_INVALID;
  int rc = mpm_bin_finalize(p, ws, cap, n, stream);
  if (rc) return rc;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  cudaStream_t s = (cudaStream_t)stream;
  rc = p->has_Ep ? launch_p2g<true, true, false>(di->p2g_ep_b_ctas, s, *p, scenes, w, cur, nxt, cap, n, 0.0f)
                 : launch_p2g<false, true, false>(di->p2g_b_ctas, s, *p, scenes, w, cur, nxt, cap, n, 0.0f);
  if (rc) return rc;
  k_grid<true><<<di->sms * 8, 256, 0, s>>>(*p, scenes, w, 0.0f);
  k_g2p<true, false, kBinPlain><<<di->g2p_b_ctas, kG2PThreads, 0, s>>>(*p, scenes, w, nxt, cap, 0.0f, maxv_out);
  return last_error();
}

int mpm_substep_noalloc(const MpmParams *p, int64_t cap, int64_t n, const float *cur, float *nxt, float dt,
                        float *maxv_out, void *stream) {
  if (!params_ok(p) || p->quant || p->n_scenes > 0 || !cur || !nxt || n < 0 || n > cap) return MPM_E_INVALID;
  if (n > kStaticMaxParticles) return MPM_E_CAPACITY;
  const size_t bytes = ws_layout(*p, kStaticMaxParticles, nullptr, nullptr);
  if (bytes > kStaticScratchBytes) return MPM_E_CAPACITY;
  if (!p2g_rows_ok(cur, cap)) return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  void *base = nullptr;
  const int rc = static_scratch_addr(&base);
  if (rc) return rc;
  Ws w;
  ws_layout(*p, kStaticMaxParticles, (char *)base, &w);
  cudaStream_t s = (cudaStream_t)stream;
  // The scratch keeps whatever the previous call left: zero the counters,
  // block flags, cell counters and grids this call relies on.
  if (cudaMemsetAsync(base, 0, bytes, s) != cudaSuccess) return MPM_E_CUDA;
  if (n > 0) {
    k_bin_count<false, false><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(*p, nullptr, w, cur, cap, 0, n);
    k_flags_count<<<w.nflagtiles, 256, 0, s>>>(*p, w);
    k_flags_write<<<w.nflagtiles, 256, 0, s>>>(*p, w);
    k_pb_stats<<<w.nstattiles, 256, 0, s>>>(*p, w);
    k_pb_scan<<<w.nstattiles, 256, 0, s>>>(*p, w);
    k_pb_levels<<<di->sms * 8, 256, 0, s>>>(*p, w, kStaticMaxParticles);
    k_scatter<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(*p, w, n);
    k_cell_clear<<<di->sms * 8, 256, 0, s>>>(*p, w);
    const int rc_p = launch_p2g_single(di, s, *p, w, cur, nxt, cap, n, dt);
    if (rc_p) return rc_p;
    k_grid<false><<<di->sms * 8, 256, 0, s>>>(*p, nullptr, w, dt);
    // the next call bins from scratch, so G2P skips the binning
    k_g2p<false, false, kBinNone><<<di->g2p_ctas, kG2PThreads, 0, s>>>(*p, nullptr, w, nxt, cap, dt, maxv_out);
  }
  return last_error();
}

// The frame driver of mpm_frame (G2P2G false), mpm_g2p2g_frame and, with a
// scene table `tab`, mpm_batch_frame (the plain loop over a batch; `maxv`
// then holds n_scenes floats per substep).
// events[5k + j]: substep k's start, after the binning of the state (a sort
// substep of the G2P2G mode) or the closing G2P of the previous plain run,
// after the finalize, after the particle kernel, after the grid update;
// events[5 count], [5 count + 1] bracket the frame's closing pass.
extern "C++" {
template <bool G2P2G, bool BATCH>
static int run_frame(const MpmParams *p, const MpmParams *tab, void *ws, int64_t cap, int64_t n, float *a, float *b,
                     float dt, int32_t count, int32_t resort, int64_t first_new, float *maxv, int32_t *in_b,
                     void *const *events, void *stream) {
  const bool params = BATCH ? (batch_ok(p) && tab != nullptr) : (params_ok(p) && p->n_scenes == 0);
  if (!params || p->quant || !ws || !a || !b || !maxv || !in_b || n < 0 || n > cap || count < 1 || resort < 1 ||
      first_new < 0 || !p2g_rows_ok(a, cap) || !p2g_rows_ok(b, cap))
    return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  cudaStream_t s = (cudaStream_t)stream;
  auto mark = [&](int64_t e) {
    if (events) cudaEventRecord((cudaEvent_t)events[e], s);
  };
  const int64_t mv_stride = BATCH ? p->n_scenes : 1;  // maxv floats per substep
  auto close_g2p = [&](float *st, float *mv) {
    if (BATCH)
      k_g2p_stream<true><<<di->g2ps_b_ctas, 128, 0, s>>>(*p, tab, w, st, cap, n, dt, mv);
    else
      k_g2p_stream<false><<<di->g2ps_ctas, 128, 0, s>>>(*p, nullptr, w, st, cap, n, dt, mv);
  };
  float *cur = a, *oth = b;
  int rc = MPM_OK;
  for (int k = 0; k < count; ++k) {
    mark(5 * k);
    const bool sort = k % resort == 0;
    if (sort) {
      // the binning of the state for this sort: the previous plain run's
      // closing G2P bins as it goes; the G2P2G mode bins in a pass of its own
      if (k > 0 && n > 0) {
        if (G2P2G)
          k_bin_box<<<di->binbox_ctas, 256, 0, s>>>(*p, w, cur, cap, n, 0);
        else
          close_g2p(cur, maxv + (k - 1) * mv_stride);
      }
      mark(5 * k + 1);
      rc = mpm_bin_finalize(p, ws, cap, n, stream);
      if (rc) return rc;
      mark(5 * k + 2);
      if (G2P2G) {
        if (n > 0) {
          rc = fused_particles<kFusedG2P2GSorted>(di, s, *p, nullptr, w, cur, oth, cap, n, dt,
                                                  k == 0 ? first_new : n, maxv + k);
          if (rc) return rc;
        }
        mark(5 * k + 3);
        fused_grid(s, di, *p, nullptr, w, dt);
      } else {
        if (BATCH)
          rc = p->has_Ep ? launch_p2g<true, true, false>(di->p2g_ep_b_ctas, s, *p, tab, w, cur, oth, cap, n, 0.0f)
                         : launch_p2g<false, true, false>(di->p2g_b_ctas, s, *p, tab, w, cur, oth, cap, n, 0.0f);
        else
          rc = launch_p2g_single(di, s, *p, w, cur, oth, cap, n, dt);
        if (rc) return rc;
        mark(5 * k + 3);
        if (BATCH)
          k_grid<true><<<di->sms * 8, 256, 0, s>>>(*p, tab, w, 0.0f);
        else
          k_grid<false><<<di->sms * 8, 256, 0, s>>>(*p, nullptr, w, dt);
      }
      float *t = cur;
      cur = oth;
      oth = t;
    } else {
      mark(5 * k + 1);
      mark(5 * k + 2);
      if (n > 0) {
        if (G2P2G)
          rc = k + 1 < count ? fused_particles<kFusedG2P2G>(di, s, *p, nullptr, w, cur, nullptr, cap, n, dt,
                                                            k == 0 ? first_new : n, maxv + k)
                             : fused_particles<kFusedG2P2GLast>(di, s, *p, nullptr, w, cur, nullptr, cap, n, dt,
                                                                k == 0 ? first_new : n, maxv + k);
        else
          rc = fused_particles<kFusedPlain, BATCH>(di, s, *p, tab, w, cur, nullptr, cap, n, dt, 0,
                                                   maxv + (k - 1) * mv_stride);
        if (rc) return rc;
      }
      mark(5 * k + 3);
      if (n > 0) fused_grid(s, di, *p, BATCH ? tab : nullptr, w, dt);
    }
    mark(5 * k + 4);
  }
  mark(5 * (int64_t)count);
  if (n > 0) {
    if (G2P2G)
      k_bin_box<<<di->binbox_ctas, 256, 0, s>>>(*p, w, cur, cap, n, 1);
    else
      close_g2p(cur, maxv + (count - 1) * mv_stride);
  }
  mark(5 * (int64_t)count + 1);
  *in_b = cur == b;
  return last_error();
}
}  // extern "C++"


int mpm_frame(const MpmParams *p, void *ws, int64_t cap, int64_t n, float *a, float *b, float dt, int32_t count,
              int32_t resort, float *maxv, int32_t *in_b, void *const *events, void *stream) {
  return run_frame<false, false>(p, nullptr, ws, cap, n, a, b, dt, count, resort, 0, maxv, in_b, events, stream);
}

int mpm_batch_frame(const MpmParams *p, const MpmParams *scenes, void *ws, int64_t cap, int64_t n, float *a,
                    float *b, int32_t count, int32_t resort, float *maxv, int32_t *in_b, void *const *events,
                    void *stream) {
  return run_frame<false, true>(p, scenes, ws, cap, n, a, b, 0.0f, count, resort, 0, maxv, in_b, events, stream);
}

int mpm_g2p2g_frame(const MpmParams *p, void *ws, int64_t cap, int64_t n, float *a, float *b, float dt,
                    int32_t count, int32_t resort, int64_t first_new, float *maxv, int32_t *in_b,
                    void *const *events, void *stream) {
  return run_frame<true, false>(p, nullptr, ws, cap, n, a, b, dt, count, resort, first_new, maxv, in_b, events,
                                stream);
}

int mpm_max_grid_velocity(const MpmParams *p, void *ws, int64_t cap, float *out, void *stream) {
  if (!params_ok(p) || !ws || !out) return MPM_E_INVALID;
  const DevInfo *di = dev_info();
  if (!di) return MPM_E_CUDA;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  k_max_grid_velocity<<<di->sms * 4, 256, 0, (cudaStream_t)stream>>>(*p, w, out);
  return last_error();
}

int mpm_constitutive_eval(const MpmParams *p, int64_t n, const int32_t *material, float *F, const float *C,
                          float *Jp, float *affine, float dt, void *stream) {
  if (!params_ok(p) || p->n_scenes > 0 || n < 0 || (n > 0 && (!material || !F || !C || !Jp || !affine)))
    return MPM_E_INVALID;
  if (n == 0) return MPM_OK;
  k_constitutive_eval<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(*p, n, material, F, C, Jp,
                                                                                      affine, dt);
  return last_error();
}

int mpm_gather_rows(const float *pstate, int64_t cap, int64_t n, int32_t row0, int32_t ncols, float *out,
                    void *stream) {
  if (!pstate || !out || n < 0 || n > cap || row0 < 0 || ncols <= 0 || row0 + ncols > MPM_NROWS)
    return MPM_E_INVALID;
  if (n == 0) return MPM_OK;
  k_gather_rows<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(pstate, cap, n, row0, ncols, out);
  return last_error();
}

int mpm_status_ptr(const MpmParams *p, void *ws, int64_t cap, uint32_t **status_out) {
  if (!params_ok(p) || !ws || !status_out) return MPM_E_INVALID;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  *status_out = (uint32_t *)&w.counters[3];
  return MPM_OK;
}

int mpm_views(const MpmParams *p, void *ws, int64_t cap, MpmViews *out) {
  if (!params_ok(p) || !ws || !out) return MPM_E_INVALID;
  Ws w;
  ws_layout(*p, cap, (char *)ws, &w);
  out->counters = w.counters;
  out->pblocks = w.pblocks;
  out->gblocks = w.gblocks;
  out->pblock_count = w.pb_count;
  out->pblock_start = w.pb_start;
  out->pid = w.pid;
  out->cellkey = w.cellkey;
  out->grid_mom = (float *)w.grid_mom;
  out->grid_vel = (float *)w.grid_vel;
  return MPM_OK;
}

}  // extern "C"
