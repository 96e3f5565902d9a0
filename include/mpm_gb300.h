/*
 * mpm_gb300.h - C ABI of the GB300-native MLS-MPM engine (libmpm_gb300.so).
 *
 * The reference (taichi-dev/taichi_elements) has no FFI: its operator API is
 * the Python class engine.mpm_solver.MPMSolver, whose @ti.kernel methods are
 * the hot path.  Each entry point below replaces one of those kernels (or a
 * piece of the Taichi runtime they rely on) and is called through ctypes by
 * taichi_elements_gb300/mpm_solver.py, the drop-in MPMSolver.
 *
 * Conventions
 *  - Every entry point returns 0 on success or a negative MPM_E_* code; it
 *    never allocates device memory.  All buffers are owned by the caller.
 *  - Pointers are device pointers unless named host_*; `stream` is a
 *    cudaStream_t passed as void*.  Launches are asynchronous.
 *  - Device-side faults (positions outside the grid window, NaN/Inf, table
 *    overflow) are reported through the status word of the workspace
 *    (MPM_STATUS_* bits), never by trapping.
 *
 * Particle state ("pstate") is one float32 buffer of MPM_NROWS rows of `cap`
 * elements (structure of arrays, row r starts at pstate + r*cap):
 *   rows 0-2 x, 3-5 v, 6-14 C (row-major 3x3), 15-23 F (row-major 3x3),
 *   24 Jp, 25 material (int32 bits), 26 original particle id (int32 bits),
 *   27 per-particle Young's modulus (used only when MpmParams.has_Ep != 0).
 * The engine ping-pongs between two such buffers: a substep reads buffer
 * `cur` in any order and writes buffer `nxt` sorted by grid block.  `cap`
 * must be a multiple of 32 and the buffers 16-byte aligned: P2G stages
 * 128-byte segments of the rows with bulk copies (entry points that run P2G
 * return MPM_E_INVALID otherwise).
 *
 * With MpmParams.quant != 0 (MPMSolver(quant=True), engine/mpm_solver.py
 * :106-127 and :216-262) the buffers hold MPM_QROWS rows of 32-bit words:
 *   rows 0-1 x as three signed 21-bit fixed-point values of scale 2^-19,
 *   rows 2-3 v as a 7-bit shared exponent (bias 100) and three signed 19-bit
 *   mantissas, rows 4-8 F as nine signed 16-bit fixed-point values of scale
 *   4.1/2^15 two per word, the last word's high half holding the 16-bit
 *   material, 9 Jp, 10 id, 11 Young's modulus, 12-20 C (float32).
 * mpm_quant_pack / mpm_quant_unpack convert between the two layouts.
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPM_ABI_VERSION 6
#define MPM_NROWS 28
#define MPM_QROWS 21
#define MPM_MAX_COLLIDERS 16 /* post-process records, box included */

/* status bits (workspace status word) */
#define MPM_STATUS_OUT_OF_GRID 1u  /* a stencil left the grid window (clamped) */
#define MPM_STATUS_NONFINITE 2u    /* NaN/Inf particle position */
#define MPM_STATUS_TABLE_OVERFLOW 4u
#define MPM_STATUS_UNSUPPORTED 8u     /* adjoint met a material it does not differentiate */
#define MPM_STATUS_TIMEOUT 16u        /* a bounded wait for staged data gave up (results invalid) */

/* error codes */
#define MPM_OK 0
#define MPM_E_INVALID (-1)
#define MPM_E_CUDA (-2)
#define MPM_E_VERSION (-3)
#define MPM_E_CAPACITY (-4)

/* Grid post-process record, applied in list order after gravity, as the
 * reference's grid_postprocess list (engine/mpm_solver.py:300-302, 794-795).
 * kind 0 = surface (half-space) collider, engine/mpm_solver.py:647-687
 * (add_surface_collider); kind 1 = sphere, :618-642 (add_sphere_collider);
 * kind 2 = bounding box, :600-616 and :689-692 (add_bounding_box), whose
 * `surface` field holds the `unbounded` flag.  surface: 0 sticky, 1 slip,
 * 2 separate (engine/mpm_solver.py:29-42). */
typedef struct MpmCollider {
  int32_t kind;
  int32_t surface;
  float point[3];  /* plane point / sphere centre */
  float normal[3]; /* unit normal (plane) */
  float radius;    /* sphere radius */
  float friction;  /* plane friction */
} MpmCollider;

/* Solver constants, engine/mpm_solver.py:44-310.  All float fields are the
 * float32 values of the reference's Python-double constants. */
typedef struct MpmParams {
  int32_t version; /* MPM_ABI_VERSION */
  int32_t res[3];
  int32_t padding;
  int32_t unbounded;
  int32_t grid_size; /* reference grid_size (4096, grown when unbounded) */
  int32_t n_colliders;
  int32_t win_lo[3]; /* grid window origin, node index, multiple of 4 */
  int32_t win_nb[3]; /* grid window extent in 4^3 blocks */
  int32_t has_Ep;    /* per-particle Young's modulus in pstate row 27 */
  int32_t chunk;     /* particles per P2G/G2P work item (multiple of 32) */
  int32_t plasticity; /* support_plasticity (mpm_solver.py:62): 0 = no Jp
                       * updates, h = 1, water restarts from F = I and sand
                       * carries no stress */
  int32_t quant;      /* quant=True (mpm_solver.py:106-127, :216-262): pstate
                       * holds the packed 21-row layout (MPM_QROWS) */
  int32_t occupancy;  /* register budget of the fused and streaming P2G
                       * kernels: 0 = stencil loops fully unrolled, 3 CTAs
                       * (12 warps) per SM; 1 = 4 CTAs (16 warps) per SM, the
                       * scatter's x loop rolled (and the gather's, except in
                       * the plain loop's single-scene fused kernel without
                       * per-particle E).  Results are the same; which is
                       * faster depends on the scene (measured per scene by
                       * the Python autotuner).  In a batch header it selects
                       * the budget of mpm_batch_frame's fused kernel */
  float dx, inv_dx, p_vol, p_mass;
  float mu0, la0, nu, alpha; /* Lame parameters, Poisson ratio, sand alpha */
  float water_density;
  float gravity[3];
  float stress_k; /* p_vol * 4 * inv_dx^2            (mpm_solver.py:569) */
  float sand_k;   /* (3 la0 + 2 mu0) / (2 mu0)        (mpm_solver.py:335-337) */
  float v_clamp_k; /* dx * g2p2g_allowed_cfl when the fused G2P2G mode clamps
                    * grid velocities to +-v_clamp_k / dt per component after
                    * gravity (mpm_solver.py:589-598); 0 = no clamp */
  /* Batched mode only (zero otherwise).  Scenes live side by side in one
   * grid window, scene s in slot (s % slots[0], s / slots[0] % slots[1],
   * s / (slots[0]*slots[1])) of slot_nb blocks per axis.  Each scene's row of
   * the scene table repeats win_nb/chunk/slots and shifts win_lo so that its
   * own grid frame maps into its slot; particles carry their scene index in
   * bits 8..30 of the material word. */
  int32_t n_scenes;
  int32_t slot_nb[3];
  int32_t slots[3];
  float dt; /* batched mode: this scene's substep dt */
  MpmCollider colliders[MPM_MAX_COLLIDERS];
} MpmParams;

/* Library ABI version (MPM_ABI_VERSION). */
int mpm_abi_version(void);

/* Bytes of scratch (workspace) a solver with this grid window and particle
 * capacity needs.  Replaces the Taichi SNode tree of
 * engine/mpm_solver.py:161-196 (pointer/dense grid and per-block pid lists)
 * and the particle dynamic SNode chunking of :212-214. */
int mpm_workspace_bytes(const MpmParams *p, int64_t cap, size_t *bytes_out);

/* Zero the persistent parts of a fresh workspace (cell counters, block
 * flags, grids, status).  Call once after allocating it. */
int mpm_workspace_init(const MpmParams *p, void *ws, int64_t cap, void *stream);

/* Bin particles [begin, end) of `pstate` into the grid: per-particle cell key
 * and rank within the cell.  Replaces build_pid, engine/mpm_solver.py:344-361
 * (the substep engine does this for the next substep inside mpm_g2p; this
 * entry point bins freshly seeded particles, engine/mpm_solver.py:840-850,
 * 969-978, 1081-1144). */
int mpm_bin_count(const MpmParams *p, void *ws, int64_t cap, const float *pstate, int64_t begin,
                  int64_t end, void *stream);

/* Turn the counts into the active-block list, the dilated grid-block list,
 * per-block particle ranges and the sorted particle order (`pid`).  Second
 * half of build_pid (engine/mpm_solver.py:344-361) plus the sparse grid
 * activation of grid.deactivate_all()/P2G writes (:789, :582-584). */
int mpm_bin_finalize(const MpmParams *p, void *ws, int64_t cap, int64_t n, void *stream);

/* P2G: engine/mpm_solver.py:487-584 (with sand_projection :321-342).  Reads
 * `cur` through the sorted order, writes the updated F/Jp and the carried
 * particle fields into `nxt` in sorted order, and scatters mass and momentum
 * into the grid. */
int mpm_p2g(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float *nxt,
            float dt, void *stream);

/* Grid update: engine/mpm_solver.py:586-616 (momentum to velocity, gravity,
 * bounding box) and :618-687 (colliders in insertion order), fused, over the
 * active grid blocks only. Also clears the momentum grid for the next P2G. */
int mpm_grid_update(const MpmParams *p, void *ws, int64_t cap, float dt, void *stream);

/* G2P: engine/mpm_solver.py:694-724, in place on `nxt`, fused with the next
 * substep's binning (build_pid, :344-361) and the max-|v| reduction
 * (compute_max_velocity, :726-735) into `maxv_out` (may be NULL). */
int mpm_g2p(const MpmParams *p, void *ws, int64_t cap, int64_t n, float *nxt, float dt,
            float *maxv_out, void *stream);

/* One substep = finalize + p2g + grid update + g2p; engine/mpm_solver.py:789-799.
 * After it returns (on the stream), `nxt` holds the state. */
int mpm_substep(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float *nxt,
                float dt, float *maxv_out, void *stream);

/* `count` plain substeps of one frame: the substep loop of step(),
 * engine/mpm_solver.py:748-799, with the same per-substep arithmetic as
 * mpm_substep.  Every `resort` substeps (and at the first) the particles are
 * re-sorted by grid block (finalize + p2g into the other buffer); between
 * sorts the G2P of one substep and the P2G of the next run as one kernel in
 * place, with the grid's active blocks marked by the particles as they
 * scatter.  The last substep's G2P bins the state for the next call.
 * Preconditions: the workspace holds the binning counts of the state in `a`
 * (mpm_bin_count of every particle, or a previous mpm_substep / mpm_g2p /
 * mpm_frame on it); both buffers satisfy mpm_p2g's layout rules; no
 * quantized state, no batch (n_scenes == 0).  `maxv` receives the max |v|
 * after each substep (count floats).  On return `*in_b` is 1 when the state
 * ends in `b`, 0 when in `a`.  `events` is NULL, or 5 * count + 2 cudaEvent_t
 * recorded on the stream for timing: events[5k .. 5k+4] at substep k's start,
 * after the previous run's closing G2P (a sort substep; else at once), after
 * the finalize (likewise), after the particle kernel (P2G of a sort, or the
 * fused G2P+P2G) and after the grid update; events[5 count] and
 * [5 count + 1] bracket the frame's closing G2P.  No single counterpart in
 * the reference, whose loop launches the four kernels of each substep
 * separately. */
int mpm_frame(const MpmParams *p, void *ws, int64_t cap, int64_t n, float *a, float *b, float dt, int32_t count,
              int32_t resort, float *maxv, int32_t *in_b, void *const *events, void *stream);

/* `count` substeps of the fused G2P2G mode (MPMSolver(use_g2p2g=True)):
 * engine/mpm_solver.py:773-787 with the g2p2g kernel :363-485, per substep
 * G2P from the previous substep's grid velocities, advection, the fused
 * constitutive update and P2G at the new positions, then the grid update
 * (with the mode's velocity clamp, MpmParams.v_clamp_k).  Every `resort`
 * substeps (and at the first) the particle kernel reads `a`/`b` in storage
 * order and writes each particle to its slot sorted by grid block in the
 * other buffer; in between it runs in place.  The state after the call is
 * binned (counts) and its bounding box reduced, as after mpm_frame.
 * Particles with id >= first_new skip the first substep's gather (they keep
 * their v with C = 0), as particles added since the last substep do in the
 * reference (last_time_final_particles); first_new = 0 before the first
 * substep of a solver.  C is not stored in this mode.  Preconditions as for
 * mpm_frame, plus: the workspace's grid velocities are those of the previous
 * substep for the particles with id < first_new.  `maxv` receives max |v|
 * per substep; `events` as for mpm_frame (events[5k+1] after the binning
 * pass of a sort substep, [5 count] and [5 count + 1] around the frame's
 * closing binning pass). */
int mpm_g2p2g_frame(const MpmParams *p, void *ws, int64_t cap, int64_t n, float *a, float *b, float dt,
                    int32_t count, int32_t resort, int64_t first_new, float *maxv, int32_t *in_b,
                    void *const *events, void *stream);

/* One substep of the fused G2P2G mode (MPMSolver(use_g2p2g=True),
 * engine/mpm_solver.py:363-485 and :773-787): G2P from the grid velocities of
 * the previous substep, advection, the constitutive update and P2G at the new
 * positions in one kernel, then the binning of the new positions and the grid
 * update with dt.  Particles with id >= first_new skip the gather (they keep
 * their v, C = 0), as particles added since the last substep do in the
 * reference (last_time_final_particles).  C is not stored in this mode.
 * The workspace must hold the binning of `cur`: finalized lists when
 * finalize_first == 0 (the state after a previous call), or the counts of
 * every particle when finalize_first != 0.  After the call it holds the
 * finalized lists of `nxt` and the grid velocities the next call gathers. */
int mpm_g2p2g_substep(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float *nxt,
                      float dt, int64_t first_new, int32_t finalize_first, float *maxv_out, void *stream);

/* Batched form: bins particles [begin, end) of a multi-scene state.  `p` is
 * the batch header (window, chunk, slot layout, n_scenes) and `scenes` a
 * device array of n_scenes per-scene MpmParams rows (see MpmParams).  No
 * counterpart in the reference, which runs one MPMSolver per scene; this is
 * build_pid (engine/mpm_solver.py:344-361) for many scenes in one launch. */
int mpm_batch_bin_count(const MpmParams *p, const MpmParams *scenes, void *ws, int64_t cap, const float *pstate,
                        int64_t begin, int64_t end, void *stream);

/* Batched substep: one substep of every scene (each with its own dt, E,
 * gravity, grid resolution and post-process list from its `scenes` row) in
 * the same kernel launches as a single scene.  maxv_out: device float array
 * of n_scenes (per-scene max |v|, zeroed by the caller), or NULL.  Replaces a
 * host loop of engine/mpm_solver.py:789-799 over independent solvers. */
int mpm_batch_substep(const MpmParams *p, const MpmParams *scenes, void *ws, int64_t cap, int64_t n,
                      const float *cur, float *nxt, float *maxv_out, void *stream);

/* Batched frame: `count` substeps of every scene of the batch (each at its
 * own MpmParams.dt), as mpm_frame does for one scene: re-sorted every
 * `resort` substeps (and at the first), the G2P of one substep fused with
 * the P2G of the next in between.  Preconditions as for mpm_batch_substep
 * (the workspace holds the binning counts of the state in `a`) and
 * mpm_frame's buffer rules.  `maxv` receives n_scenes floats per substep
 * (the scenes' max |v|); on return `*in_b` is 1 when the state ends in `b`.
 * `events` as for mpm_frame.  No counterpart in the reference, which runs
 * one MPMSolver per scene. */
int mpm_batch_frame(const MpmParams *p, const MpmParams *scenes, void *ws, int64_t cap, int64_t n, float *a,
                    float *b, int32_t count, int32_t resort, float *maxv, int32_t *in_b, void *const *events,
                    void *stream);

/* ---- Adjoint of one substep (water and elastic) ----------------------
 * No counterpart in the reference, which has no autodiff.  Gradient buffers
 * `gin` / `gout` have 26 float32 rows of `cap` columns: dL/dx (rows 0-2),
 * dL/dv (3-5), dL/dC (6-14), dL/dF (15-23), dL/dJp (24) and dL/dE of the
 * per-particle Young's modulus (25); `gin` holds the gradient with respect to
 * the state after substep t, `gout` receives the one before it (distinct
 * buffers).  Columns are original particle ids when `by_id` is nonzero;
 * otherwise `gin` is in the order of the substep's sorted output (the order
 * mpm_p2g wrote `nxt` in) and `gout` in the order of `cur`, so all gradient
 * traffic is coalesced.  `gmid` (3 rows of `cap`) carries the position
 * gradient from mpm_g2p_adj to mpm_p2g_adj.  `keep` and `ggrid` are float4
 * arrays shaped like the workspace grid (see mpm_workspace_bytes: window
 * blocks * 64 nodes).
 * `cur` is the particle state before substep t.  The workspace `ws` must
 * hold the binning and grid of the forward substep t: run its forward
 * (bin count, finalize, p2g from `cur`), then
 *   mpm_grid_snapshot(keep)      - between mpm_p2g and mpm_grid_update
 *   mpm_grid_update
 * (a caller may do this during a checkpoint-segment recompute and keep one
 * workspace + snapshot per substep), and then for the adjoint:
 *   zero ggrid; mpm_g2p_adj      - writes gmid, scatters dL/dv_grid
 *   mpm_grid_adj                 - dL/dv_grid -> dL/d(m, mv) in place
 *   mpm_p2g_adj                  - writes all rows of gout */
int mpm_grid_snapshot(const MpmParams *p, void *ws, int64_t cap, float *keep, void *stream);
/* Move `rows` gradient rows (row stride cap) between original-id columns and
 * the column order of particle state `state`: with to_state_order nonzero
 * dst[r][j] = src[r][id_j], else dst[r][id_j] = src[r][j], where id_j is the
 * id row of `state` at column j.  src and dst must differ. */
int mpm_grad_reorder(const float *state, int64_t cap, int64_t n, int32_t rows, const float *src, float *dst,
                     int32_t to_state_order, void *stream);
/* mpm_g2p with the next substep's binning (cell counts, block flags, cell
 * keys) written to the workspace `ws_bins` instead of `ws`, so that a
 * checkpoint-segment recompute can keep one workspace per substep.  The cell
 * counts and block flags of `ws_bins` must be zero: a freshly initialised
 * workspace, or one whose own substep (bin finalize) has run since it was
 * last binned into. */
int mpm_g2p_bin_into(const MpmParams *p, void *ws, void *ws_bins, int64_t cap, int64_t n, float *nxt, float dt,
                     float *maxv_out, void *stream);
int mpm_g2p_adj(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float dt, const float *gin,
                float *gmid, float *ggrid, int32_t by_id, void *stream);
int mpm_grid_adj(const MpmParams *p, void *ws, int64_t cap, const float *keep, float *ggrid, float dt,
                 void *stream);
int mpm_p2g_adj(const MpmParams *p, void *ws, int64_t cap, int64_t n, const float *cur, float dt, const float *gin,
                const float *gmid, float *gout, const float *ggrid, int32_t by_id, void *stream);

/* One substep that allocates nothing and needs no caller-provided workspace.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc (or a caching allocator) at the point they step the simulation,
 * for example code running inside someone else's stream capture or memory
 * pool, or a host application that hands the engine only its particle
 * buffers.  All scratch (binning tables, grids, status) lives in one static
 * device array of the library, 16 MiB, which every GPU that loads the library
 * holds until the process exits.
 *   - The caller passes `cur` and `nxt` (pstate layout, row stride `cap`);
 *     `nxt` receives the state sorted by grid block, as with mpm_substep.
 *   - Limits: at most 65,536 particles, and a grid window whose workspace
 *     fits 16 MiB (about 4,000 blocks of 4^3 nodes, e.g. a 48^3 grid with the
 *     solver's default margins).  Larger inputs return MPM_E_CAPACITY before
 *     any device work.
 *   - The first call on a device looks up the array's device address and
 *     keeps it for the life of the process; make that first call before any
 *     stream capture, and do not use the library across a cudaDeviceReset
 *     (the kept address would then be stale).
 *   - Single scenes only: batched parameter blocks (n_scenes > 0) and packed
 *     storage (quant) return MPM_E_INVALID.
 *   - Every call bins all particles itself and clears the scratch it uses,
 *     since the array keeps the previous call's contents; calls that overlap
 *     on the GPU (other streams, other threads) share the array and race.
 *   - The status word of this scratch is not exposed; check results on the
 *     host (finite positions) when that matters. */
int mpm_substep_noalloc(const MpmParams *p, int64_t cap, int64_t n, const float *cur, float *nxt, float dt,
                        float *maxv_out, void *stream);

/* Copy rows of the sorted state back to original particle order:
 * out[id[j]*ncols + c] = pstate[(row0 + c)*cap + j] for c < ncols.
 * Replaces copy_dynamic_nd / copy_dynamic, engine/mpm_solver.py:1146-1191. */
int mpm_gather_rows(const float *pstate, int64_t cap, int64_t n, int32_t row0, int32_t ncols,
                    float *out, void *stream);

/* Packed particle storage (quant=True).  mpm_quant_pack encodes `count`
 * slots of a float32-layout buffer (MPM_NROWS rows of stride rows_cap, slot
 * t at column t) into slots begin + t of the packed buffer (MPM_QROWS rows of
 * stride cap), rounding to the nearest representable value (ties away from
 * zero); positions outside [-2, 2) are clamped and OR MPM_STATUS_OUT_OF_GRID
 * into *status (device int32, may be null), non-finite values
 * MPM_STATUS_NONFINITE.  mpm_quant_unpack decodes packed slots begin + t
 * into column t of a float32-layout buffer (rows 25 and 26 carry the
 * material and id as int32 bits). */
int mpm_quant_pack(const float *rows, int64_t rows_cap, int64_t count, float *packed, int64_t cap, int64_t begin,
                   int32_t *status, void *stream);
int mpm_quant_unpack(const float *packed, int64_t cap, int64_t begin, int64_t count, float *rows, int64_t rows_cap,
                     void *stream);

/* ---- Particle output (engine/particle_io.py:12-76, ParticleIO.write_particles)
 * The quantised frame format: per dimension, positions and velocities are
 * mapped to their [min, max] range over all particles (max raised to
 * min + 1e-5 when narrower, :48-50), quantised to 24 and 8 bits with the
 * reference's float32 expression and packed into one uint32 per component,
 * (qx << 8) + qv (uint32 wrap-around).
 * mpm_particle_ranges: `keys` is a device uint32[12] scratch, `ranges_out` a
 *   device float[12] laid out as the reference's (2, 3, 2) `ranges` array
 *   (positions then velocities; per dimension min, max).  n >= 1.
 * mpm_quantize_particles: `x_and_v` is a device uint32[n * 3] in ORIGINAL
 *   particle order (rows scattered by the id row of `pstate`).
 * mpm_unpack_colors: 24-bit colours (device int32[n], original order) to a
 *   device uint8[n * 3] of R, G, B (:62-74). */
int mpm_particle_ranges(const float *pstate, int64_t cap, int64_t n, uint32_t *keys, float *ranges_out,
                        void *stream);
int mpm_quantize_particles(const float *pstate, int64_t cap, int64_t n, const float *ranges, uint32_t *x_and_v,
                           void *stream);
int mpm_unpack_colors(const int32_t *color, int64_t n, uint8_t *rgb, void *stream);

/* ---- Mesh emitter (engine/voxelizer.py:46-126, engine/mpm_solver.py:1017-1079)
 * mpm_voxelize: triangles (device float64[ntri * 9], vertex-major xyz) into
 *   the dense voxel grid `voxels` (device int32[rx * ry * rz], index
 *   (p * ry + q) * rz + k, zeroed here): per voxel the signed count of
 *   triangle crossings above it along z, as Voxelizer.voxelize_triangles.
 *   dx is the voxel size (solver dx / super_sample), padding the voxelizer's.
 * mpm_voxel_seed_count / mpm_voxel_seed_emit: particles of seed_from_voxels
 *   (mpm_solver.py:1017-1047).  Count pass: particles per voxel column into
 *   col_count (int32[rx * ry]); the caller scans them into col_offset
 *   (int64, exclusive) and sizes x_out (float32[n_out * 3]); the emit pass
 *   writes positions (rand + (i, j, k)) * voxel_dx + (tx, ty, tz).  Random
 *   numbers come from a counter-based hash of `seed`, the voxel and the draw
 *   (deterministic per seed; not Taichi's ti.random stream). */
int mpm_voxelize(const double *triangles, int64_t ntri, int32_t rx, int32_t ry, int32_t rz, double dx,
                 int32_t padding, int32_t *voxels, void *stream);
int mpm_voxel_seed_count(const int32_t *voxels, int32_t rx, int32_t ry, int32_t rz, int32_t sample_density,
                         int32_t super_sample, int32_t grid_size, int32_t padding, uint64_t seed, int32_t *col_count,
                         void *stream);
int mpm_voxel_seed_emit(const int32_t *voxels, int32_t rx, int32_t ry, int32_t rz, int32_t sample_density,
                        int32_t super_sample, int32_t grid_size, int32_t padding, uint64_t seed, float voxel_dx,
                        float tx, float ty, float tz, const int64_t *col_offset, int64_t n_out, float *x_out,
                        void *stream);

/* ---- Particle path tracer (engine/renderer.py, engine/renderer_utils.py)
 * `scene` points to a host RenderScene (layout in csrc/mpm_render.cu,
 * mirrored by taichi_elements_gb300/renderer.py; its size is
 * mpm_render_scene_bytes()).  Cell lists over the particle bounding box:
 * mpm_render_cell_count adds each particle's cells to `count`
 * (int32[cells], zeroed by the caller); the caller scans them into `start`
 * (int64[cells], exclusive) and sizes `list` (int32[list_len]);
 * mpm_render_cell_fill writes the particle indices (`fill`, int32[cells],
 * zeroed).  x, v: float32[n * 3] (v may be NULL: no motion blur); rgb:
 * uint8[n * 3].  mpm_render_occupancy packs one bit per cell (count > 0)
 * into `occ` (uint32[(cells + 31) / 32]), which the tracing calls read
 * before touching a cell's list.  mpm_render_samples adds `spp` path-traced samples
 * (sample indices sample0 ..) of every pixel to color_buffer
 * (float32[res0 * res1 * 3], pixel (u, v) at (u * res1 + v) * 3);
 * mpm_render_tonemap writes the displayed image (vignette, exposure,
 * square root) for `samples` accumulated samples; mpm_render_first_hits
 * evaluates the nearest hit (distance, normal, colour: float32[7] per ray)
 * of given rays. */
int mpm_render_scene_bytes(void);
int mpm_render_cell_count(const void *scene, const float *x, const float *v, int64_t n, int32_t *count,
                          void *stream);
int mpm_render_cell_fill(const void *scene, const float *x, const float *v, int64_t n, const int64_t *start,
                         int32_t *fill, int64_t list_len, int32_t *list, void *stream);
int mpm_render_occupancy(const int32_t *count, int64_t ncells, uint32_t *occ, void *stream);
int mpm_render_samples(const void *scene, const uint32_t *occ, const int64_t *start, const int32_t *count,
                       const int32_t *list, const float *x, const float *v, const uint8_t *rgb, int32_t sample0,
                       int32_t spp, float *color_buffer, void *stream);
int mpm_render_tonemap(int32_t rx, int32_t ry, const float *color_buffer, float vignette_strength,
                       float vignette_radius, float vcx, float vcy, float exposure, int32_t samples, float *img,
                       void *stream);
int mpm_render_first_hits(const void *scene, const uint32_t *occ, const int64_t *start, const int32_t *count,
                          const int32_t *list, const float *x, const float *v, const uint8_t *rgb, const float *orig,
                          const float *dir, int64_t nrays, float t, float *out, void *stream);

/* compute_max_grid_velocity (engine/mpm_solver.py:737-746): raises *out
 * (device float, zeroed by the caller) to the largest |v_d| over the nodes of
 * the grid-active blocks of the last substep (0 before the first).  Used by
 * the adaptive time step (use_adaptive_dt, :761-766). */
int mpm_max_grid_velocity(const MpmParams *p, void *ws, int64_t cap, float *out, void *stream);

/* The constitutive update of P2G (engine/mpm_solver.py:506-574, with
 * sand_projection :321-342) for n independent particles, by the device code
 * the P2G kernels run: material[i] (0-4), F[9 i .. 9 i + 8] (row major) and
 * Jp[i] updated in place, C[9 i ..] read, affine[9 i ..] written with the
 * APIC matrix -dt p_vol 4 inv_dx^2 stress + mass C (:569-574).  A diagnostic
 * entry point for tests on chosen deformation gradients (inverted, nearly
 * singular, clamped); device pointers; single-scene parameters. */
int mpm_constitutive_eval(const MpmParams *p, int64_t n, const int32_t *material, float *F, const float *C,
                          float *Jp, float *affine, float dt, void *stream);

/* Pointer to the device status word inside the workspace (uint32). */
int mpm_status_ptr(const MpmParams *p, void *ws, int64_t cap, uint32_t **status_out);

/* Diagnostics views inside the workspace (device pointers), used by the
 * parity tests: counters (int32[16]: 0 #particle blocks, 1 #grid blocks,
 * 2 #work items, 3 status, 4 #particles binned), the particle-block list,
 * the grid-block list, per-particle-block counts and starts, and the sorted
 * order. */
typedef struct MpmViews {
  int32_t *counters;
  int32_t *pblocks;
  int32_t *gblocks;
  int32_t *pblock_count;
  int32_t *pblock_start;
  int32_t *pid;
  int32_t *cellkey;
  float *grid_mom; /* float4 per node (m, mv) in window block-major order */
  float *grid_vel; /* float4 per node (v, m) */
} MpmViews;
int mpm_views(const MpmParams *p, void *ws, int64_t cap, MpmViews *out);

#ifdef __cplusplus
}
#endif
#endif
