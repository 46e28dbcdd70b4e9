// fv_kernels.h -- host-side launchers of the GB300 hydro kernels.
#pragma once

#include <cuda_runtime.h>

#include "fv_device.cuh"

namespace fv {

// Pointers to the five field arrays of one state, in storage order
// (rho, m_a, m_b, m_c, E): m_a = x-momentum, m_b = momentum along the second
// active axis (y or z), m_c = momentum along the degenerate axis.
struct Fields {
  double* f[5];
};

// Tile of the 2-D FP64 stage kernel.
constexpr int kTileX = 32;
constexpr int kTileY = 16;

// One fused stage (Euler step, RK2 stage 1 or RK2 stage 2) over a 2-D plane.
//   uin  : the stage's input state (read with a 2-cell ghost halo)
//   u0   : U^n for STAGE_RK_2 (read at own cell only); unused otherwise
//   uout : output state (may alias u0 for STAGE_RK_2; never uin)
// dt and the active flag come from ctrl (set by launch_control); STAGE_EULER
// and STAGE_RK_2 also reduce max inv_dt_hyp of their output into
// ctrl->slot[parity ^ 1].
cudaError_t launch_stage2d(const Grid2D& G, int riemann_solver, int kind, bool wact, Fields uin, Fields u0,
                           Fields uout, StepCtrl* ctrl, cudaStream_t stream);

// Reduce max inv_dt_hyp of state u into ctrl->slot[slot] (caller zeroes it).
cudaError_t launch_reduce2d(const Grid2D& G, bool wact, Fields u, StepCtrl* ctrl, int slot, cudaStream_t stream);

// Per-step control for n problems: choose dt (CFL from the reduced max, or
// dt_given when mode_override == 0), set active and parity, advance t and the
// step counter, zero the next reduction slot.  mode_override < 0 uses each
// control block's own mode; 2 takes the CFL dt with no time bound.
cudaError_t launch_control(StepCtrl* ctrl, int n, int mode_override, double dt_given, cudaStream_t stream);

// In-place conversions on a state whose arrays hold primitive / conserved
// values in storage order (primToCons / consToPrim, States.h:20-45, with the
// reference's rounding: no contraction).
cudaError_t launch_prim_to_cons2d(const Grid2D& G, Fields u, cudaStream_t stream);
cudaError_t launch_cons_to_prim2d(const Grid2D& G, Fields src, Fields dst, cudaStream_t stream);

// Compensated per-block partial sums of the five conserved fields:
// partial[(blk*5 + v)*2 + {0,1}] = (sum, compensation).  Returns the block
// count through nblocks.
cudaError_t launch_totals2d(const Grid2D& G, Fields u, double* partial, int max_blocks, int* nblocks,
                            cudaStream_t stream);

}  // namespace fv
