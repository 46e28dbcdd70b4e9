// fv_kernels.h -- host-side launchers of the GB300 hydro kernels.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "fv3d_gb300.h"
#include "fv_device.cuh"
#include "fv_grid.cuh"
#include "fv_tma.cuh"

namespace fv {

#ifndef FV_PDL
#define FV_PDL 1  // 0: plain stream order for the step-loop kernels
#endif

// Launches a step-loop kernel (one that waits with pdl_wait) with
// programmatic stream serialisation, so that its launch overlaps the tail of
// the previous kernel in the stream.
template <class... KArgs, class... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = FV_PDL;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// Pointers to the five field arrays of one state, in storage order
// (rho, m_a, m_b, m_c, E): m_a = x-momentum, m_b = momentum along the second
// active axis (y or z), m_c = momentum along the degenerate axis.
struct Fields {
  double* f[5];
};

// Tile of the 2-D FP64 stage kernel, and the resident CTAs per SM its
// register allocation targets (without / with the third momentum).
#ifndef FV_TILE2D_X
#define FV_TILE2D_X 32
#endif
#ifndef FV_TILE2D_Y
#define FV_TILE2D_Y 16
#endif
#ifndef FV_FP64_MIN_CTAS
#define FV_FP64_MIN_CTAS 3
#endif
#ifndef FV_FP64_MIN_CTAS_W
#define FV_FP64_MIN_CTAS_W 2
#endif
constexpr int kTileX = FV_TILE2D_X;
constexpr int kTileY = FV_TILE2D_Y;

// One fused stage (Euler step, RK2 stage 1 or RK2 stage 2) over a 2-D plane.
//   uin  : the stage's input state (read with a 2-cell ghost halo)
//   u0   : U^n for STAGE_RK_2 (read at own cell only); unused otherwise
//   uout : output state (may alias u0 for STAGE_RK_2; never uin)
// dt and the active flag come from ctrl (set by launch_control); STAGE_EULER
// and STAGE_RK_2 also reduce max inv_dt_hyp of their output into
// ctrl->slot[parity ^ 1].  hout (optional, STAGE_EULER / STAGE_RK_2 only):
// the stage also writes the primitives of its result, storage order, to
// unpadded arrays of na x rows values that the GPU can address (device or
// host memory).
// tin (optional): TMA descriptors of uin (encode_tma_state); interior
// blocks are then staged by tensor copies instead of per-thread loads.
// prims (optional): a padded primitive copy Q of the state (same layout as
// the conserved fields).  A stage given qout writes the primitives of its
// result there and sets ctrl->q_valid; a stage given qin reads its halo
// from Q instead of converting uin when ctrl->q_valid is set (the host
// clears it whenever it writes the state).  Q holds the same bits
// consToPrim gives, so the results are unchanged.
struct PrimCopy {
  const Fields* qin = nullptr;   // read by this stage (Q == primitives of uin)
  const Fields* qout = nullptr;  // written by this stage (primitives of uout)
  const TmaState* tq = nullptr;  // TMA descriptors of Q (with qin)
};
cudaError_t launch_stage2d(const Grid& G, int riemann_solver, int kind, bool wact, Fields uin, Fields u0,
                           Fields uout, StepCtrl* ctrl, cudaStream_t stream, const Fields* hout = nullptr,
                           const TmaState* tin = nullptr, const PrimCopy* prims = nullptr);

// Encodes the TMA descriptors of state u of the 2-D problem G for the stage
// kernel (tensor na x rows of doubles, row pitch G.pitch, boxes of
// (kTileX + 4) x kTmaRows).  False when the driver's encoder is unavailable
// or refuses the layout; the stage kernel then loads with plain loads.
bool encode_tma_state(const Grid& G, const Fields& u, TmaState* tin);

// The same stage over a 3-D grid (G.ndim == 3): 16 x 16 blocks of columns
// marched over z, the (column block, layer) units split evenly over the
// resident CTAs; always carries w.
cudaError_t launch_stage3d(const Grid& G, int riemann_solver, int kind, Fields uin, Fields u0, Fields uout,
                           StepCtrl* ctrl, cudaStream_t stream, const Fields* hout = nullptr,
                           const PrimCopy* prims = nullptr);

// The stage kernel the grid needs (2-D plane kernel or 3-D kernel).
inline cudaError_t launch_stage(const Grid& G, int riemann_solver, int kind, bool wact, Fields uin, Fields u0,
                                Fields uout, StepCtrl* ctrl, cudaStream_t stream, const Fields* hout = nullptr,
                                const TmaState* tin = nullptr, const PrimCopy* prims = nullptr) {
  if (G.ndim == 3) return launch_stage3d(G, riemann_solver, kind, uin, u0, uout, ctrl, stream, hout, prims);
  return launch_stage2d(G, riemann_solver, kind, wact, uin, u0, uout, ctrl, stream, hout, tin, prims);
}

// primToCons (States.h:20-31) from primitive arrays the GPU can address
// (unpadded rows of na values, storage order, a null field reads as 0) into
// the padded conserved state dst; with ctrl, also the CFL maximum of
// consToPrim of the result into ctrl->slot[slot] (ComputeDt.h:28-54, the
// reference's dt after its set-up).  qout (optional): also the primitive
// copy of dst (PrimCopy), with *q_valid set once it is written.
cudaError_t launch_prim_to_cons_from(const Grid& G, bool wact, Fields src, Fields dst, StepCtrl* ctrl, int slot,
                                     cudaStream_t stream, const Fields* qout = nullptr, int* q_valid = nullptr);

// Reduce max inv_dt_hyp of state u into ctrl->slot[slot] (caller zeroes it).
cudaError_t launch_reduce2d(const Grid& G, bool wact, Fields u, StepCtrl* ctrl, int slot, cudaStream_t stream);

// Per-step control for n problems: choose dt (CFL from the reduced max, or
// dt_given when mode_override == 0), set active and parity, advance t and the
// step counter, zero the next reduction slot.  mode_override < 0 uses each
// control block's own mode; 2 takes the CFL dt with no time bound.
cudaError_t launch_control(StepCtrl* ctrl, int n, int mode_override, double dt_given, cudaStream_t stream);

// In-place conversions on a state whose arrays hold primitive / conserved
// values in storage order (primToCons / consToPrim, States.h:20-45, with the
// reference's rounding: no contraction).
cudaError_t launch_prim_to_cons2d(const Grid& G, Fields u, cudaStream_t stream);
cudaError_t launch_cons_to_prim2d(const Grid& G, Fields src, Fields dst, cudaStream_t stream);

// Compensated per-block partial sums of the five conserved fields:
// partial[(blk*5 + v)*2 + {0,1}] = (sum, compensation).  Returns the block
// count through nblocks.
cudaError_t launch_totals2d(const Grid& G, Fields u, double* partial, int max_blocks, int* nblocks,
                            cudaStream_t stream);

// ---- batches of independent problems ----------------------------------

enum Precision : int { PREC_FP64 = 0, PREC_MIXED = 1 };

// One problem of a batch as the persistent kernels see it.  FP64: A = U^n,
// B = U* (Euler: ping-pong).  FP32-mixed: A = U^n as float2 (hi, lo) pairs,
// B = U* as float (RK2) or the second pair buffer (Euler).  Q (FP64 2-D RK2
// only, else null): the primitive copy of A (PrimCopy), valid while
// ctrl->q_valid is set.
struct BatchInst {
  Grid G;
  Fields A, B, Q;
  StepCtrl* ctrl;
  int tiles_x;  // tiles along a
  int tile0;    // first tile of this problem in its group's tile numbering
  int rs;       // 0 HLL, 1 HLLC
  int tiles_y;  // tiles along b (3-D: column blocks along y)
  int tz;       // 3-D: z layers per work item (work item = column block x z chunk)
  int pad;
};

// Tile shapes the autotuner chooses from (cells along a x along b).
struct TileShape {
  int tx, ty;
};
int batch_tile_shapes64(const TileShape** shapes);
int batch_tile_shapes32(const TileShape** shapes);
// The kernel of FP32-mixed shape `shape`: its index (shapes of one kernel
// differ only in their starting rows), its block rows (8 or 16) and whether
// it computes the viscous fluxes in a per-face pass (1) or per cell (0).
int batch_shape_kernel32(int shape, int* block_rows, int* vface);

// Persistent stage kernel over a group of problems sharing plane and third
// momentum: `grid` CTAs pull tiles from the work-queue counter *queue (reset
// by launch_batch_control) until `ntiles` are done.  flip selects the Euler
// ping-pong direction (B -> A when set); tc sizes shared memory for the
// temperature tile.  Shape indexes batch_tile_shapes64/32.
cudaError_t launch_batch_stage64(int plane, bool wact, int shape, const BatchInst* insts, int ninst, int ntiles,
                                 unsigned* queue, int kind, int flip, int grid, bool tc, cudaStream_t stream);
cudaError_t launch_batch_stage32(int plane, bool wact, int shape, const BatchInst* insts, int ninst, int ntiles,
                                 unsigned* queue, int kind, int flip, int grid, bool tc, cudaStream_t stream);
// Resident CTAs per SM of one batch stage kernel (0 on error).
int batch_stage_occupancy64(int plane, bool wact, int shape, bool tc);
int batch_stage_occupancy32(int plane, bool wact, int shape, bool tc);

// Persistent stage kernels for groups of 3-D problems sharing a Riemann
// solver (rs): a work item is a 16 x 16 column block and a chunk of tz z
// layers of one problem (numbered x fastest, then y, then z); same body as
// launch_stage3d, so a problem in a batch is bit-identical to the same
// problem alone (FP64).
int batch3d_columns();  // column-block side (16)
cudaError_t launch_batch_stage3d64(const BatchInst* insts, int ninst, int ntiles, unsigned* queue, int kind, int flip,
                                   int rs, int grid, bool tc, cudaStream_t stream);
cudaError_t launch_batch_stage3d32(const BatchInst* insts, int ninst, int ntiles, unsigned* queue, int kind, int flip,
                                   int rs, int grid, bool tc, cudaStream_t stream);
// rs: Riemann solver (bit 0), corrected physics (bit 1).
int batch_stage3d_occupancy64(int rs, bool tc);
int batch_stage3d_occupancy32(int rs, bool tc);

// Several RK2 steps of a group of FP32-mixed 2-D problems in one cooperative
// launch (fv_batch32.cu, batch_multi32): for small grids, whose steps are
// bound by launch latency.  At most batch_multi_problems32() problems; grid
// at most batch_multi_occupancy32() x SMs CTAs (all resident); the barrier
// counter and abort flag of gb zeroed before the launch; a grid-barrier wait
// that runs out sets bit 1 of every problem's error flag.  mode_override as
// launch_control.
int batch_multi_problems32();
int batch_multi_occupancy32(int plane, bool wact, int shape, bool tc);
cudaError_t launch_batch_multi32(int plane, bool wact, int shape, const BatchInst* insts, int ninst, int ntiles,
                                 int nsteps, int mode_override, GridBarrier gb, int grid, bool tc,
                                 cudaStream_t stream);

// launch_control for n problems plus a reset of nq work-queue counters.
cudaError_t launch_batch_control(StepCtrl* ctrl, int n, unsigned* queue, int nq, int mode_override, double dt_given,
                                 cudaStream_t stream);

// FP32-mixed helpers: CFL max of (hi, lo) pairs; pairs <-> FP64 values.
cudaError_t launch_reduce2d_mixed(const Grid& G, bool wact, Fields pairs, StepCtrl* ctrl, int slot,
                                  cudaStream_t stream);
cudaError_t launch_pairs_from_double(const Grid& G, Fields src, Fields dst_pairs, cudaStream_t stream);
cudaError_t launch_double_from_pairs(const Grid& G, Fields src_pairs, Fields dst, cudaStream_t stream);

// The reference's problem generators (Init.h:18-209) on the GPU (fv_init.cu).
enum InitKind : int {
  INIT_SOD_X, INIT_SOD_Y, INIT_SOD_Z, INIT_BLAST, INIT_RT, INIT_DIFFUSION, INIT_H84, INIT_C91
};
struct InitSpec {
  int kind;                  // InitKind
  int nx, ny, rows;          // Nx, Ny and rows = Ny * Nz
  double xmin, ymin, zmin, dx, dy, dz;
  double xmid, ymid, zmid;   // 0.5 * (min + max) per axis
  double m1;                 // polytropic index (H84, C91)
  double c0;                 // 0.1 g (rayleigh-taylor), theta1 (C91)
  double c1, c2;             // 4 pi and 3 pi (rayleigh-taylor)
  double pert;               // perturbation amplitude (H84, C91)
  unsigned long long key;    // perturbation stream key
};
// FV_OK, or FV_ERR_PARAM for a problem name Init.h does not know.
int make_init_spec(const fv_params& p, InitSpec* spec);
// Writes the primitives of every interior cell to out (reference variable
// order rho, u, v, w, p; element (k * Ny + j) * pitch + i) and ORs bit v of
// *flags when field v has a non-zero value.
cudaError_t launch_generate(const InitSpec& spec, const Fields& out, int pitch, int* flags, cudaStream_t stream);

}  // namespace fv
