/*
 * Oracle for the MLS-MPM substep: CPU restatement of taichi-dev/taichi_elements
 * engine/mpm_solver.py (p2g :487-584, sand_projection :321-342, grid update
 * :586-616, colliders :618-692, g2p :694-724, substep loop :789-797).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, by the smoke check and by the
 * benchmark's CPU-baseline leg.  The product package never loads it.
 *
 * Exported symbols carry a _d (float64) or _f (float32) suffix.
 *
 * `pd` (double[17]) layout, ORACLE_PD_*:
 *   0 dx, 1 inv_dx, 2 p_vol, 3 p_mass, 4 mu0, 5 la0, 6 alpha (sand),
 *   7 water_density, 8..10 gravity, 11 p_vol*4*inv_dx^2, 12 (3la0+2mu0)/(2mu0),
 *   13 nu, 14 support_plasticity (0 or 1), 15 dx * g2p2g_allowed_cfl of the
 *   fused mode's grid velocity clamp (0 = none), 16 quant (0 or 1: stored
 *   x, v and F take the values of the packed fields)
 * Post-process records (double[12] each), applied in list order like the
 *   reference's grid_postprocess list: 0 kind (0 plane, 1 sphere,
 *   2 bounding box), 1 surface (0 sticky, 1 slip, 2 separate; for the box:
 *   the unbounded flag), 2..4 point/centre,
 *   5..7 unit normal (plane), 8 radius (sphere), 9 friction, 10..11 unused.
 * Grids are dense windows: node (i,j,k) of the reference grid frame lives at
 *   ((i-lo0)*W1 + (j-lo1))*W2 + (k-lo2); momentum/velocity is AoS (n*3).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define REAL double
#define SFX _d
#include "mpm_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX _f
#define ORACLE_IS_FLOAT 1
#include "mpm_oracle_impl.h"
#undef ORACLE_IS_FLOAT
#undef REAL
#undef SFX

int oracle_abi_version(void) { return 1; }
