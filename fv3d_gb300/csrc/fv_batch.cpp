// fv_batch.cpp -- extern "C" entry points for batches of independent problems
// (fvgpu_batch_*).  No counterpart in the reference, which runs one problem
// per process (main.cpp:25-30).
//
// A batch owns one device allocation holding every problem's two state
// buffers, one control block per problem (each problem has its own dt, time
// and CFL reduction) and a few work-queue counters.  Problems that share the
// plane and the third-momentum layout form a group; one persistent kernel
// launch per RK stage advances a whole group (fv_batch64.cu /
// fv_batch32.cu).  Steps are replayed from a captured CUDA graph of
// kGraphSteps steps.  The tile shape of each group is chosen by timing the
// candidate shapes on the group's own data (autotuner), and remembered per
// (precision, plane, layout, problem sizes) in memory and in a small cache
// file (FV3D_TILE_CACHE, default $XDG_CACHE_HOME/fv3d_gb300/tiles.txt).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include <cuda_runtime.h>

#include "fv3d_gb300.h"
#include "fv_kernels.h"

namespace fv {
int configure_grid(const fv_params& p, Grid* G, double* inv_tc, double* inv_visc, int* deg_bc,
                   std::string* err);
}

using fv::BatchInst;
using fv::Fields;
using fv::Grid;
using fv::StepCtrl;

namespace {

constexpr int kGraphSteps = 8;
constexpr int kMaxGroups = 8;  // two work-queue counters each
// Problems of at most this many cells in all run several steps per launch
// (FP32-mixed RK2, one group of 2-D problems): their steps are bound by
// launch latency, not by the GPU's throughput.
constexpr long long kMultiMaxCells = 1LL << 21;
constexpr int kMultiChunk = 256;  // steps per multi-step launch of a loop with a time bound

struct Group {
  int ndim = 2;     // 3: 3-D problems (one kernel shape, grouped by solver)
  int rs = -1;      // 3-D groups: the shared Riemann solver (bit 0) and corrected physics (bit 1)
  int plane = 0;
  bool wact = false;
  bool tc = false;
  std::vector<int> members;
  int shape = 0;
  int rows = 0;     // 2-D: rows per work item (0: the shape's)
  int ntiles = 0;
  int grid = 0;
  BatchInst* d_inst = nullptr;
};

}  // namespace

struct fv_batch {
  int n = 0;
  int precision = FV_PREC_FP64;
  int ts = FV_TS_RK2;
  std::vector<fv_params> p;
  std::vector<Grid> G;
  std::vector<int> deg_bc;
  std::vector<double> inv_tc, inv_visc;
  std::vector<char> wact, state_set, slot_valid;
  std::vector<Fields> A, B, Q;  // Q: primitive copy of A (FP64 2-D RK2), else null
  double* buf = nullptr;
  double* scratch = nullptr;
  long long max_fstride = 0;
  StepCtrl* d_ctrl = nullptr;
  StepCtrl* h_ctrl = nullptr;
  unsigned* d_queue = nullptr;  // 2 per group, then the grid barrier's counter and abort flag
  std::vector<Group> groups;
  bool prepared = false;
  int flip = 0;  // Euler: current states are in B
  cudaStream_t own_stream = nullptr, stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaGraphExec_t graph_loop = nullptr;  // steps in each control block's own mode
  BatchInst* d_inst_multi = nullptr;     // descriptors of the multi-step launch
  int ntiles_multi = 0, grid_multi = 0, rows_multi = 0;
  long launches = 0;
  std::string err;
};

namespace {

int Fail(fv_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCUDA(b, call)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return Fail((b), FV_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Device allocations of one scope, freed when it ends (early returns
// included; cudaFree waits for the work that may still use them).
struct ScopedDevice {
  std::vector<void*> ptrs;
  ScopedDevice() = default;
  ScopedDevice(const ScopedDevice&) = delete;
  ScopedDevice& operator=(const ScopedDevice&) = delete;
  ~ScopedDevice() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** p, size_t bytes) {
    void* q = nullptr;
    const cudaError_t e = cudaMalloc(&q, bytes);
    *p = e == cudaSuccess ? static_cast<T*>(q) : nullptr;
    if (e == cudaSuccess) ptrs.push_back(q);
    return e;
  }
};

void StorageOrder(int plane, int slot_of[5]) {
  slot_of[0] = 0;
  slot_of[1] = 1;
  slot_of[2] = plane == fv::PLANE_XY ? 2 : 3;
  slot_of[3] = plane == fv::PLANE_XY ? 3 : 2;
  slot_of[4] = 4;
}

const Fields& Current(const fv_batch* b, int i) { return b->flip ? b->B[i] : b->A[i]; }

// FP64 2-D RK2 problems keep a primitive copy of U^n (BatchInst::Q).
bool WithPrimCopy(const fv_batch* b, int i) {
  return b->precision == FV_PREC_FP64 && b->ts == FV_TS_RK2 && b->G[i].ndim == 2;
}

// ---- tile-shape cache --------------------------------------------------

// A group's schedule: strip width, rows per work item, and for the
// FP32-mixed kernels the rows per marched block (cells per thread) and the
// viscous form (1: per-face pass, 0: fused per cell).
struct Schedule {
  int tx = 0, rows = 0, block_rows = 16, vface = 0;
};

std::mutex g_cache_mutex;
std::map<std::string, Schedule> g_cache;
bool g_cache_loaded = false;

std::string CachePath() {
  if (const char* f = std::getenv("FV3D_TILE_CACHE")) return f;
  std::string dir;
  if (const char* x = std::getenv("XDG_CACHE_HOME")) dir = x;
  else if (const char* h = std::getenv("HOME")) dir = std::string(h) + "/.cache";
  else return "";
  return dir + "/fv3d_gb300/tiles.txt";
}

void LoadCache() {
  if (g_cache_loaded) return;
  g_cache_loaded = true;
  std::ifstream in(CachePath());
  std::string key;
  int tx, ty;
  // lines: key tx rows [block_rows vface]
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    Schedule sc;
    if (!(ls >> key >> sc.tx >> sc.rows)) continue;
    int br = 0, vf = 0;
    if (ls >> br >> vf) {
      sc.block_rows = br;
      sc.vface = vf;
    }
    g_cache[key] = sc;
  }
  (void)tx;
  (void)ty;
}

void SaveCacheEntry(const std::string& key, const Schedule& sc) {
  const std::string path = CachePath();
  if (path.empty()) return;
  const std::string dir = path.substr(0, path.find_last_of('/'));
  const std::string parent = dir.substr(0, dir.find_last_of('/'));
  mkdir(parent.c_str(), 0755);
  mkdir(dir.c_str(), 0755);
  std::ofstream out(path, std::ios::app);
  if (out) out << key << " " << sc.tx << " " << sc.rows << " " << sc.block_rows << " " << sc.vface << "\n";
}

// Key of a group: precision, plane, layout, conduction, solver mix and the
// multiset of problem sizes (hashed).
std::string GroupKey(const fv_batch* b, const Group& g) {
  std::vector<std::pair<int, int>> sizes;
  int rs_mask = 0;
  bool visc = false;
  for (int i : g.members) {
    sizes.push_back({b->G[i].na, b->G[i].nb * b->G[i].nc});
    rs_mask |= 1 << (b->p[i].riemann_solver == FV_HLL ? 0 : 1);
    visc = visc || b->G[i].visc;
  }
  std::sort(sizes.begin(), sizes.end());
  unsigned long long h = 1469598103934665603ull;
  long long cells = 0;
  for (auto& s : sizes) {
    h = (h ^ (unsigned long long)s.first) * 1099511628211ull;
    h = (h ^ (unsigned long long)s.second) * 1099511628211ull;
    cells += (long long)s.first * s.second;
  }
  std::ostringstream k;
  k << "p" << b->precision << "_d" << g.ndim << "_co" << (g.rs >= 2) << "_pl" << g.plane << "_w" << g.wact << "_tc" << g.tc << "_v" << visc << "_rs"
    << rs_mask << "_ts" << b->ts << "_n" << g.members.size() << "_c" << cells << "_h" << std::hex << h;
  return k.str();
}

int NumShapes(int precision, const fv::TileShape** shapes) {
  return precision == FV_PREC_FP64 ? fv::batch_tile_shapes64(shapes) : fv::batch_tile_shapes32(shapes);
}

// The schedule a shape stands for (rows: the shape's own).  FP64 kernels:
// blocks of 512 cells, viscous fluxes of the face-only branches shared per
// face (fv_tile64.cuh).
Schedule ShapeSchedule(const fv_batch* b, int shape) {
  const fv::TileShape* shapes;
  NumShapes(b->precision, &shapes);
  Schedule sc;
  sc.tx = shapes[shape].tx;
  sc.rows = shapes[shape].ty;
  if (b->precision == FV_PREC_FP64) {
    sc.block_rows = 512 / sc.tx;
    sc.vface = 1;
  } else {
    fv::batch_shape_kernel32(shape, &sc.block_rows, &sc.vface);
  }
  return sc;
}

// The schedule of a 3-D group: 16 x 16 column blocks, z layers per work item;
// the FP64 kernel shares the x / y faces' viscous fluxes.
Schedule Schedule3d(const fv_batch* b, int layers) {
  Schedule sc;
  sc.tx = fv::batch3d_columns();
  sc.rows = layers > 0 ? layers : 16;
  sc.block_rows = 0;
  sc.vface = b->precision == FV_PREC_FP64 ? 1 : 0;
  return sc;
}

int Occupancy(const fv_batch* b, const Group& g, int shape) {
  if (g.ndim == 3)
    return b->precision == FV_PREC_FP64 ? fv::batch_stage3d_occupancy64(g.rs, g.tc)
                                        : fv::batch_stage3d_occupancy32(g.rs, g.tc);
  return b->precision == FV_PREC_FP64 ? fv::batch_stage_occupancy64(g.plane, g.wact, shape, g.tc)
                                      : fv::batch_stage_occupancy32(g.plane, g.wact, shape, g.tc);
}

cudaError_t LaunchStage(const fv_batch* b, const Group& g, const BatchInst* insts, int ntiles, int grid,
                        unsigned* queue, int kind, int flip) {
  if (g.ndim == 3)
    return b->precision == FV_PREC_FP64
               ? fv::launch_batch_stage3d64(insts, (int)g.members.size(), ntiles, queue, kind, flip, g.rs, grid, g.tc,
                                            b->stream)
               : fv::launch_batch_stage3d32(insts, (int)g.members.size(), ntiles, queue, kind, flip, g.rs, grid, g.tc,
                                            b->stream);
  return b->precision == FV_PREC_FP64
             ? fv::launch_batch_stage64(g.plane, g.wact, g.shape, insts, (int)g.members.size(), ntiles, queue, kind,
                                        flip, grid, g.tc, b->stream)
             : fv::launch_batch_stage32(g.plane, g.wact, g.shape, insts, (int)g.members.size(), ntiles, queue, kind,
                                        flip, grid, g.tc, b->stream);
}

// Descriptors of group g for work-item shape `shape` with `rows` rows per
// item (0: the shape's), work items numbered per group.  2-D items are strip
// segments (BatchInst::tz = rows per item); 3-D groups: 16 x 16 column
// blocks and chunks of up to 16 z layers.
std::vector<BatchInst> Describe(const fv_batch* b, const Group& g, int shape, StepCtrl* ctrl_base, int* ntiles,
                                int rows = 0) {
  const fv::TileShape* shapes;
  NumShapes(b->precision, &shapes);
  const int tx = g.ndim == 3 ? fv::batch3d_columns() : shapes[shape].tx;
  const int ty = g.ndim == 3 ? fv::batch3d_columns() : (rows > 0 ? rows : shapes[shape].ty);
  std::vector<BatchInst> out;
  int t0 = 0;
  for (int i : g.members) {
    BatchInst I;
    std::memset(&I, 0, sizeof(I));
    I.G = b->G[i];
    I.A = b->A[i];
    I.B = b->B[i];
    I.Q = b->Q[i];
    I.ctrl = ctrl_base + i;
    I.tiles_x = (I.G.na + tx - 1) / tx;
    I.tiles_y = (I.G.nb + ty - 1) / ty;
    I.tz = g.ndim == 3 ? std::min(I.G.nc, rows > 0 ? rows : 16) : ty;  // 3-D: z layers per item
    const int chunks = g.ndim == 3 ? (I.G.nc + I.tz - 1) / I.tz : 1;
    I.tile0 = t0;
    I.rs = b->p[i].riemann_solver == FV_HLL ? 0 : 1;
    t0 += I.tiles_x * I.tiles_y * chunks;
    out.push_back(I);
  }
  *ntiles = t0;
  return out;
}

int SmCount() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// Times the candidate shapes of a group on its own data, one whole step per
// run (RK2: both stages; Euler: its one stage, which writes the idle
// buffer), against scratch control blocks.  RK2 stage 2 overwrites U^n, so
// the group's U^n is copied aside first and put back afterwards; without
// room for that copy only stage 1 is timed.  The problems' state and clocks
// are left as they were, and the tuning descriptors carry no primitive copy.
int Autotune(fv_batch* b, Group& g) {
  const bool d3 = g.ndim == 3;  // one kernel: 16 x 16 column blocks; tuned: z layers per item
  if (d3 && Occupancy(b, g, 0) <= 0) return Fail(b, FV_ERR_CUDA, "the 3-D batch kernel cannot be launched");
  const fv::TileShape* shapes;
  const int ns = d3 ? 1 : NumShapes(b->precision, &shapes);
  bool visc = false;  // the viscous form matters only with viscosity
  for (int i : g.members) visc = visc || b->G[i].visc;
  // the first shape of a kernel (it serves every row count): strip width,
  // block rows and viscous form
  auto shape_of = [&](const Schedule& sc) {
    if (d3) return sc.tx == fv::batch3d_columns() ? 0 : -1;
    for (int s = 0; s < ns; ++s) {
      const Schedule k = ShapeSchedule(b, s);
      if (k.tx == sc.tx && k.block_rows == sc.block_rows && k.vface == sc.vface && Occupancy(b, g, s) > 0) return s;
    }
    return -1;
  };
  auto take = [&](const Schedule& sc) {
    const int s = shape_of(sc);
    if (s < 0) return false;
    g.shape = s;
    g.rows = sc.rows;
    return true;
  };
  if (const char* force = std::getenv("FV3D_TILE")) {  // WxH, WxH/B, WxHv, WxH/Bv
    Schedule sc;
    char rest[16] = "";
    const int got = std::sscanf(force, "%dx%d%15s", &sc.tx, &sc.rows, rest);
    if (got >= 2 && sc.rows > 0) {
      char* r = rest;
      if (*r == '/') sc.block_rows = (int)std::strtol(r + 1, &r, 10);
      sc.vface = *r == 'v' ? 1 : 0;
      if (d3) {
        sc = Schedule3d(b, sc.rows);
      } else if (b->precision == FV_PREC_FP64) {  // one kernel per strip width
        const int rows = sc.rows;
        for (int s = 0; s < ns; ++s)
          if (shapes[s].tx == sc.tx) sc = ShapeSchedule(b, s);
        sc.rows = rows;
      }
      if (take(sc)) return FV_OK;
    }
  }
  const std::string key = GroupKey(b, g);
  {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    LoadCache();
    auto it = g_cache.find(key);
    if (it != g_cache.end() && it->second.rows > 0 && take(it->second)) return FV_OK;
  }
  // Candidates: every shape with its own rows, and per strip width the rows
  // that give each resident CTA one work item's worth of strip rows (the
  // balanced split for a few large problems).
  std::vector<std::pair<int, int>> cand;
  int max_nc = 1;
  for (int i : g.members) max_nc = std::max(max_nc, b->G[i].nc);
  if (d3) {  // z layers per work item; a 4-layer prologue is converted per item
    for (int z : {8, 16, 32, 64})
      if (z == 8 || z <= max_nc) cand.push_back({0, z});
    // and the chunk lengths that make the work items fill 1-4 rounds of the
    // resident CTAs (the fewest layers with at most r rounds of items)
    const long long slots = (long long)Occupancy(b, g, 0) * SmCount();
    const int side = fv::batch3d_columns();
    auto items = [&](int z) {
      long long n = 0;
      for (int i : g.members)
        n += (long long)((b->G[i].na + side - 1) / side) * ((b->G[i].nb + side - 1) / side) *
             ((b->G[i].nc + z - 1) / z);
      return n;
    };
    for (int r = 1; r <= 4 && slots > 0; ++r) {
      int z = 4;
      while (z < max_nc && items(z) > r * slots) ++z;
      bool dup = false;
      for (auto& c : cand) dup = dup || c.second == z;
      if (!dup && items(z) <= r * slots) cand.push_back({0, z});
    }
  }
  for (int s = 0; s < ns && !d3; ++s)
    if (visc || !ShapeSchedule(b, s).vface || b->precision == FV_PREC_FP64) cand.push_back({s, shapes[s].ty});
  for (int s = 0; s < ns && !d3; ++s) {
    const Schedule ks = ShapeSchedule(b, s);
    if ((ks.vface && !visc && b->precision != FV_PREC_FP64) || shape_of(ks) != s) continue;
    long long units = 0;
    for (int i : g.members) units += (long long)((b->G[i].na + shapes[s].tx - 1) / shapes[s].tx) * b->G[i].nb;
    const long long slots = (long long)Occupancy(b, g, s) * SmCount();
    if (slots <= 0) continue;
    const int rows = (int)std::max(4LL, (units + slots - 1) / slots);
    bool dup = false;
    for (auto& c : cand) dup = dup || (shape_of(ShapeSchedule(b, c.first)) == s && c.second == rows);
    if (!dup) cand.push_back({s, rows});
  }
  StepCtrl* tune_ctrl = nullptr;
  BatchInst* tune_inst = nullptr;
  unsigned* tune_queue = nullptr;
  const size_t nm = g.members.size();
  ScopedDevice scratch;
  BCUDA(b, scratch.alloc(&tune_ctrl, sizeof(StepCtrl) * b->n));
  BCUDA(b, scratch.alloc(&tune_inst, sizeof(BatchInst) * nm * cand.size()));
  BCUDA(b, scratch.alloc(&tune_queue, 2 * sizeof(unsigned)));
  std::vector<StepCtrl> hc(b->n);
  for (int i = 0; i < b->n; ++i) {
    std::memset(&hc[i], 0, sizeof(StepCtrl));
    hc[i].active = 1;
    hc[i].dt_cur = 1.0e-9;
  }
  cudaMemcpyAsync(tune_ctrl, hc.data(), sizeof(StepCtrl) * b->n, cudaMemcpyHostToDevice, b->stream);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int kind = b->ts == FV_TS_RK2 ? fv::STAGE_RK_1 : fv::STAGE_EULER;
  const int saved = g.shape;
  // Each candidate's descriptors get their own slice of tune_inst (host
  // vectors kept alive until the copies are done).
  std::vector<std::vector<BatchInst>> descs(cand.size());
  std::vector<int> ntiles(cand.size(), 0), grid(cand.size(), 0);
  for (size_t c = 0; c < cand.size(); ++c) {
    const int s = cand[c].first;
    const int occ = Occupancy(b, g, s);
    if (occ <= 0) continue;
    descs[c] = Describe(b, g, s, tune_ctrl, &ntiles[c], cand[c].second);
    for (auto& I : descs[c]) I.Q = Fields{};
    cudaMemcpyAsync(tune_inst + c * nm, descs[c].data(), sizeof(BatchInst) * descs[c].size(),
                    cudaMemcpyHostToDevice, b->stream);
    grid[c] = std::min(occ * SmCount(), ntiles[c]);
  }
  // U^n of the group aside (RK2), when a quarter of the free memory holds it
  double* backup = nullptr;
  std::vector<size_t> a_doubles(nm);
  size_t backup_doubles = 0;
  if (b->ts == FV_TS_RK2) {
    for (size_t m = 0; m < nm; ++m) {
      a_doubles[m] = (size_t)5 * b->G[g.members[m]].fstride;  // A: 5 fields of fstride 8-byte values
      backup_doubles += a_doubles[m];
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && backup_doubles * sizeof(double) <= free_b / 4 &&
        cudaMalloc(&backup, backup_doubles * sizeof(double)) == cudaSuccess) {
      size_t at = 0;
      for (size_t m = 0; m < nm; ++m) {
        cudaMemcpyAsync(backup + at, b->A[g.members[m]].f[0], a_doubles[m] * sizeof(double),
                        cudaMemcpyDeviceToDevice, b->stream);
        at += a_doubles[m];
      }
    } else {
      cudaGetLastError();  // a refused allocation leaves no sticky error
      backup = nullptr;
    }
  }
  const bool both_stages = backup != nullptr;
  // Rounds over all candidates (so that clock and power drift hits each
  // alike), one warm-up round first; a candidate's time is its fastest run.
  constexpr int kRounds = 5;
  std::vector<float> best_ms(cand.size(), 1e30f);
  for (int round = 0; round <= kRounds; ++round) {
    for (size_t c = 0; c < cand.size(); ++c) {
      if (!grid[c]) continue;
      g.shape = cand[c].first;
      cudaMemsetAsync(tune_queue, 0, 2 * sizeof(unsigned), b->stream);
      cudaEventRecord(e0, b->stream);
      cudaError_t e = LaunchStage(b, g, tune_inst + c * nm, ntiles[c], grid[c], tune_queue, kind, b->flip);
      if (e == cudaSuccess && both_stages)
        e = LaunchStage(b, g, tune_inst + c * nm, ntiles[c], grid[c], tune_queue + 1, fv::STAGE_RK_2, 0);
      cudaEventRecord(e1, b->stream);
      if (e != cudaSuccess) {
        grid[c] = 0;  // not launchable: drop it
        continue;
      }
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (round > 0 && ms < best_ms[c]) best_ms[c] = ms;
    }
  }
  float best = 1e30f;
  int best_c = -1;
  const bool log = std::getenv("FV3D_TILE_LOG") != nullptr;
  for (size_t c = 0; c < cand.size(); ++c) {
    if (log) {
      const Schedule k = d3 ? Schedule3d(b, cand[c].second) : ShapeSchedule(b, cand[c].first);
      std::fprintf(stderr, "fv3d tile candidate %dx%d/%d%s: %.4f ms (%d items, %d CTAs)\n", k.tx, cand[c].second,
                   k.block_rows, k.vface ? "v" : "", grid[c] ? best_ms[c] : -1.0f, ntiles[c], grid[c]);
    }
    if (grid[c] && best_ms[c] < best) {
      best = best_ms[c];
      best_c = (int)c;
    }
  }
  g.shape = best_c < 0 ? saved : cand[best_c].first;
  g.rows = best_c < 0 ? 0 : cand[best_c].second;
  if (backup) {  // U^n back in place
    size_t at = 0;
    for (size_t m = 0; m < nm; ++m) {
      cudaMemcpyAsync(b->A[g.members[m]].f[0], backup + at, a_doubles[m] * sizeof(double), cudaMemcpyDeviceToDevice,
                      b->stream);
      at += a_doubles[m];
    }
  }
  cudaStreamSynchronize(b->stream);
  if (backup) cudaFree(backup);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best_c < 0) return Fail(b, FV_ERR_CUDA, "no tile shape could be launched for a batch group");
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  Schedule chosen = d3 ? Schedule3d(b, g.rows) : ShapeSchedule(b, g.shape);
  chosen.rows = g.rows;
  g_cache[key] = chosen;
  SaveCacheEntry(key, chosen);
  return FV_OK;
}

void ReleaseGroups(fv_batch* b) {
  for (auto& g : b->groups)
    if (g.d_inst) cudaFree(g.d_inst);
  if (b->d_inst_multi) cudaFree(b->d_inst_multi);
  b->d_inst_multi = nullptr;
  b->groups.clear();
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graph_loop) cudaGraphExecDestroy(b->graph_loop);
  b->graph = nullptr;
  b->graph_loop = nullptr;
  b->prepared = false;
}

// Groups problems by (plane, third-momentum layout), picks tile shapes and
// uploads the descriptors.
int Prepare(fv_batch* b) {
  if (b->prepared) return FV_OK;
  ReleaseGroups(b);
  for (int i = 0; i < b->n; ++i) {
    const int ndim = b->G[i].ndim;
    const int rs = ndim == 3 ? (b->p[i].riemann_solver == FV_HLL ? 0 : 1) + (b->G[i].corrected ? 2 : 0) : -1;
    Group* g = nullptr;
    for (auto& h : b->groups)
      if (h.ndim == ndim && h.rs == rs && h.plane == b->G[i].plane && h.wact == (bool)b->wact[i]) g = &h;
    if (!g) {
      b->groups.push_back(Group());
      g = &b->groups.back();
      g->ndim = ndim;
      g->rs = rs;
      g->plane = b->G[i].plane;
      g->wact = b->wact[i];
    }
    g->members.push_back(i);
    g->tc = g->tc || b->G[i].tc;
  }
  if ((int)b->groups.size() > kMaxGroups) return Fail(b, FV_ERR_UNSUPPORTED, "more than %d batch groups", kMaxGroups);
  for (auto& g : b->groups) {
    int rc = Autotune(b, g);
    if (rc) return rc;
    std::vector<BatchInst> d = Describe(b, g, g.shape, b->d_ctrl, &g.ntiles, g.rows);
    BCUDA(b, cudaMalloc(&g.d_inst, sizeof(BatchInst) * d.size()));
    BCUDA(b, cudaMemcpyAsync(g.d_inst, d.data(), sizeof(BatchInst) * d.size(), cudaMemcpyHostToDevice, b->stream));
    g.grid = std::max(1, std::min(Occupancy(b, g, g.shape) * SmCount(), g.ntiles));
  }
  BCUDA(b, cudaStreamSynchronize(b->stream));
  b->prepared = true;
  return FV_OK;
}

// The error status of a control block's sticky flag: bit 1 a bounded wait
// that gave up, bit 0 a non-finite state or dt.
int ErrStatus(int err) { return (err & 2) ? FV_ERR_TIMEOUT : FV_ERR_NONFINITE; }

// Whether run / advance take several steps per launch (batch_multi32): the
// FP32-mixed RK2 form, one group of 2-D problems, few cells in all.
// FV3D_MULTISTEP=0 keeps the per-stage launches, =1 takes the multi-step
// launch whatever the size.
bool MultiEligible(const fv_batch* b) {
  if (b->precision != FV_PREC_FP32_MIXED || b->ts != FV_TS_RK2 || b->groups.size() != 1) return false;
  const Group& g = b->groups[0];
  if (g.ndim != 2 || (int)g.members.size() > fv::batch_multi_problems32()) return false;
  if (ShapeSchedule(b, g.shape).vface) return false;  // multi-step kernels: the fused viscous form
  const char* env = std::getenv("FV3D_MULTISTEP");
  if (env && env[0] == '0') return false;
  long long cells = 0;
  for (int i : g.members) cells += (long long)b->G[i].na * b->G[i].nb;
  return cells <= kMultiMaxCells || (env && env[0] == '1');
}

// Descriptors of the multi-step launch: the group's strip width, rows per
// work item that give each resident CTA about one item (4 to 64; measured on
// Sedov 128^2 / 256^2 / 512^2 and 16 Sod tubes of 96^2, this count was the
// fastest of 4 / 8 / 16 / 32 rows each time; FV3D_MULTI_ROWS forces it).
int PrepareMulti(fv_batch* b) {
  if (b->d_inst_multi) return FV_OK;
  Group& g = b->groups[0];
  const int occ = fv::batch_multi_occupancy32(g.plane, g.wact, g.shape, g.tc);
  if (occ <= 0) return Fail(b, FV_ERR_CUDA, "the multi-step kernel cannot be launched");
  const fv::TileShape* shapes;
  NumShapes(b->precision, &shapes);
  const int tx = shapes[g.shape].tx;
  long long units = 0;
  for (int i : g.members) units += (long long)((b->G[i].na + tx - 1) / tx) * b->G[i].nb;
  const long long slots = (long long)occ * SmCount();
  int rows = (int)std::min(64LL, std::max(4LL, (units + slots - 1) / slots));
  if (const char* f = std::getenv("FV3D_MULTI_ROWS")) rows = std::max(1, std::atoi(f));
  std::vector<BatchInst> d = Describe(b, g, g.shape, b->d_ctrl, &b->ntiles_multi, rows);
  BCUDA(b, cudaMalloc(&b->d_inst_multi, sizeof(BatchInst) * d.size()));
  BCUDA(b, cudaMemcpyAsync(b->d_inst_multi, d.data(), sizeof(BatchInst) * d.size(), cudaMemcpyHostToDevice,
                           b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  b->rows_multi = rows;
  b->grid_multi = (int)std::max(1LL, std::min((long long)b->ntiles_multi, slots));
  return FV_OK;
}

// nsteps steps of the (single) group in one cooperative launch.
int RunMulti(fv_batch* b, int nsteps, int mode_override) {
  const Group& g = b->groups[0];
  unsigned* bar = b->d_queue + 2 * kMaxGroups;
  BCUDA(b, cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), b->stream));
  const fv::GridBarrier gb{bar, reinterpret_cast<int*>(bar + 1)};
  const cudaError_t e = fv::launch_batch_multi32(g.plane, g.wact, g.shape, b->d_inst_multi, (int)g.members.size(),
                                                 b->ntiles_multi, nsteps, mode_override, gb, b->grid_multi, g.tc,
                                                 b->stream);
  if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "multi-step launch: %s", cudaGetErrorString(e));
  b->launches += 1;
  return FV_OK;
}

int ReadCtrl(fv_batch* b) {
  BCUDA(b, cudaMemcpyAsync(b->h_ctrl, b->d_ctrl, sizeof(StepCtrl) * b->n, cudaMemcpyDeviceToHost, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return FV_OK;
}

// Makes every problem's reduction slot for its next step hold the CFL max
// of its current state.
int EnsureSlots(fv_batch* b) {
  bool any = false;
  for (int i = 0; i < b->n; ++i) any = any || !b->slot_valid[i];
  if (!any) return FV_OK;
  int rc = ReadCtrl(b);
  if (rc) return rc;
  for (int i = 0; i < b->n; ++i) {
    if (b->slot_valid[i]) continue;
    const int slot = (int)(b->h_ctrl[i].step & 1);
    BCUDA(b, cudaMemsetAsync(&b->d_ctrl[i].slot[slot], 0, sizeof(unsigned long long), b->stream));
    cudaError_t e = b->precision == FV_PREC_FP64
                        ? fv::launch_reduce2d(b->G[i], b->wact[i], Current(b, i), b->d_ctrl + i, slot, b->stream)
                        : fv::launch_reduce2d_mixed(b->G[i], b->wact[i], Current(b, i), b->d_ctrl + i, slot,
                                                    b->stream);
    if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "batch dt reduction: %s", cudaGetErrorString(e));
    b->launches += 1;
    b->slot_valid[i] = 1;
  }
  return FV_OK;
}

int KernelsPerStep(const fv_batch* b) {
  return 1 + (int)b->groups.size() * (b->ts == FV_TS_RK2 ? 2 : 1);
}

// Control + stages of one step for every group.
// mode_override: 2 = CFL dt, no time bound (fvgpu_batch_run); 0 = the given
// dt; -1 = each control block's own mode (the main.cpp loop of batch_advance).
int EnqueueStep(fv_batch* b, int mode_override = 2, double dt = 0.0) {
  const int nq = 2 * (int)b->groups.size();
  cudaError_t e = fv::launch_batch_control(b->d_ctrl, b->n, b->d_queue, nq, mode_override, dt, b->stream);
  for (size_t gi = 0; gi < b->groups.size() && e == cudaSuccess; ++gi) {
    const Group& g = b->groups[gi];
    unsigned* q = b->d_queue + 2 * gi;
    if (b->ts == FV_TS_RK2) {
      e = LaunchStage(b, g, g.d_inst, g.ntiles, g.grid, q, fv::STAGE_RK_1, 0);
      if (e == cudaSuccess) e = LaunchStage(b, g, g.d_inst, g.ntiles, g.grid, q + 1, fv::STAGE_RK_2, 0);
    } else {
      e = LaunchStage(b, g, g.d_inst, g.ntiles, g.grid, q, fv::STAGE_EULER, b->flip);
    }
  }
  if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "batch step launch: %s", cudaGetErrorString(e));
  if (b->ts != FV_TS_RK2) b->flip ^= 1;
  return FV_OK;
}

}  // namespace

extern "C" {

int fvgpu_batch_create(const fv_params* params, int n, fv_batch** out) {
  if (!out) return FV_ERR_PARAM;
  *out = nullptr;
  fv_batch* b = new fv_batch();
  *out = b;
  if (!params || n <= 0) return Fail(b, FV_ERR_PARAM, "need n > 0 parameter sets");
  b->n = n;
  b->precision = params[0].precision;
  b->ts = params[0].time_stepping;
  if (b->precision != FV_PREC_FP64 && b->precision != FV_PREC_FP32_MIXED)
    return Fail(b, FV_ERR_PARAM, "unknown precision %d", b->precision);
  b->p.assign(params, params + n);
  b->G.resize(n);
  b->deg_bc.resize(n);
  b->inv_tc.resize(n);
  b->inv_visc.resize(n);
  b->wact.assign(n, 0);
  b->state_set.assign(n, 0);
  b->slot_valid.assign(n, 0);
  std::vector<size_t> off(n);
  size_t total = 0;
  for (int i = 0; i < n; ++i) {
    if (params[i].precision != b->precision || params[i].time_stepping != b->ts)
      return Fail(b, FV_ERR_UNSUPPORTED, "problem %d: all problems of a batch share precision and time stepping", i);
    fv_params q = params[i];
    q.precision = FV_PREC_FP64;  // the grid checks are those of the FP64 handle
    std::string err;
    int rc = fv::configure_grid(q, &b->G[i], &b->inv_tc[i], &b->inv_visc[i], &b->deg_bc[i], &err);
    if (rc) return Fail(b, rc, "problem %d: %s", i, err.c_str());
    if (b->G[i].ndim == 3) {
      const int n_ax[3] = {params[i].Nx, params[i].Ny, params[i].Nz};
      const int bc_ax[3] = {params[i].boundary_x, params[i].boundary_y, params[i].boundary_z};
      for (int a = 0; a < 3; ++a)
        if (n_ax[a] == 1 && bc_ax[a] == FV_BC_REFLECTING)
          return Fail(b, FV_ERR_UNSUPPORTED, "problem %d: a reflecting one-cell axis runs with fvgpu_create", i);
    }
    if (params[i].thermal_conductivity_active && params[i].thermal_conductivity_mode == FV_TCM_B02)
      return Fail(b, FV_ERR_UNSUPPORTED, "problem %d: B02 conductivity runs with the FP64 handle (fvgpu_create)", i);
    if (b->precision != FV_PREC_FP64 && b->G[i].fstride >= (1LL << 32))
      return Fail(b, FV_ERR_UNSUPPORTED, "problem %d: the FP32-mixed kernels address fields below 2^32 cells", i);
    b->wact[i] = (params[i].viscosity_active || b->G[i].ndim == 3) ? 1 : 0;
    off[i] = total;
    total += (size_t)(WithPrimCopy(b, i) ? 15 : 10) * b->G[i].fstride;
    b->max_fstride = std::max(b->max_fstride, b->G[i].fstride);
  }
  if (cudaMalloc(&b->buf, total * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&b->scratch, (size_t)5 * b->max_fstride * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&b->d_ctrl, sizeof(StepCtrl) * n) != cudaSuccess ||
      cudaMallocHost(&b->h_ctrl, sizeof(StepCtrl) * n) != cudaSuccess ||
      cudaMalloc(&b->d_queue, sizeof(unsigned) * (2 * kMaxGroups + 2)) != cudaSuccess)
    return Fail(b, FV_ERR_NOMEM, "batch allocation of %zu bytes failed", total * sizeof(double));
  // Initialisation is ordered on the batch's own non-blocking stream (a
  // legacy-stream cudaMemset would not be ordered with it) and waited for
  // below.
  if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return Fail(b, FV_ERR_CUDA, "stream creation failed");
  b->stream = b->own_stream;
  BCUDA(b, cudaMemsetAsync(b->buf, 0, total * sizeof(double), b->stream));
  BCUDA(b, cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned) * (2 * kMaxGroups + 2), b->stream));
  b->A.resize(n);
  b->B.resize(n);
  b->Q.assign(n, Fields{});
  for (int i = 0; i < n; ++i)
    for (int v = 0; v < 5; ++v) {
      b->A[i].f[v] = b->buf + off[i] + (size_t)v * b->G[i].fstride;
      b->B[i].f[v] = b->buf + off[i] + (size_t)(5 + v) * b->G[i].fstride;
      if (WithPrimCopy(b, i)) b->Q[i].f[v] = b->buf + off[i] + (size_t)(10 + v) * b->G[i].fstride;
    }
  std::vector<StepCtrl> hc(n);
  for (int i = 0; i < n; ++i) {
    std::memset(&hc[i], 0, sizeof(StepCtrl));
    hc[i].cfl = params[i].CFL;
    hc[i].inv_tc = b->inv_tc[i];
    hc[i].inv_visc = b->inv_visc[i];
    hc[i].epsilon = params[i].epsilon;
    hc[i].mode = 2;
  }
  BCUDA(b, cudaMemcpyAsync(b->d_ctrl, hc.data(), sizeof(StepCtrl) * n, cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return FV_OK;
}

int fvgpu_batch_destroy(fv_batch* b) {
  if (!b) return FV_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  ReleaseGroups(b);
  if (b->buf) cudaFree(b->buf);
  if (b->scratch) cudaFree(b->scratch);
  if (b->d_ctrl) cudaFree(b->d_ctrl);
  if (b->h_ctrl) cudaFreeHost(b->h_ctrl);
  if (b->d_queue) cudaFree(b->d_queue);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return FV_OK;
}

const char* fvgpu_batch_last_error(const fv_batch* b) { return b ? b->err.c_str() : "null handle"; }

int fvgpu_batch_set_prim(fv_batch* b, int inst, const double* rho, const double* u, const double* v,
                         const double* w, const double* pr) {
  if (!b || !b->buf) return b ? Fail(b, FV_ERR_STATE, "batch not configured") : FV_ERR_PARAM;
  if (inst < 0 || inst >= b->n) return Fail(b, FV_ERR_PARAM, "problem index %d out of range", inst);
  const Grid& G = b->G[inst];
  int slot_of[5];
  StorageOrder(G.plane, slot_of);
  const double* ref[5] = {rho, u, v, w, pr};
  const double* src[5];
  for (int k = 0; k < 5; ++k) src[slot_of[k]] = ref[k];
  if (!src[0] || !src[4]) return Fail(b, FV_ERR_PARAM, "density and pressure arrays are required");
  bool nonzero = false;
  if (src[3] && G.ndim == 2)
    for (long long c = 0; c < (long long)G.na * G.rows && !nonzero; ++c) nonzero = src[3][c] != 0.0;
  const bool wact = b->p[inst].viscosity_active || nonzero || G.ndim == 3;
  if (G.ndim == 2 && wact && b->deg_bc[inst] == FV_BC_REFLECTING)
    return Fail(b, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting degenerate axis is not built");
  if ((bool)b->wact[inst] != wact) b->prepared = false;
  b->wact[inst] = wact;
  if (!b->prepared) ReleaseGroups(b);
  if (b->Q[inst].f[0])  // the primitive copy no longer matches the state
    BCUDA(b, cudaMemsetAsync(&b->d_ctrl[inst].q_valid, 0, sizeof(int), b->stream));
  // FP64 values into the staging buffer (the current state for FP64, scratch
  // for the mixed form), primToCons in place, then split into pairs (mixed)
  Fields stage = b->precision == FV_PREC_FP64 ? Current(b, inst) : Fields();
  if (b->precision != FV_PREC_FP64)
    for (int k = 0; k < 5; ++k) stage.f[k] = b->scratch + (size_t)k * G.fstride;
  const size_t rowb = (size_t)G.na * sizeof(double);
  for (int k = 0; k < 5; ++k) {
    if (src[k])
      BCUDA(b, cudaMemcpy2DAsync(stage.f[k], (size_t)G.pitch * sizeof(double), src[k], rowb, rowb, G.rows,
                                 cudaMemcpyHostToDevice, b->stream));
    else
      BCUDA(b, cudaMemsetAsync(stage.f[k], 0, (size_t)G.fstride * sizeof(double), b->stream));
  }
  cudaError_t e = fv::launch_prim_to_cons2d(G, stage, b->stream);
  if (e == cudaSuccess && b->precision != FV_PREC_FP64)
    e = fv::launch_pairs_from_double(G, stage, Current(b, inst), b->stream);
  if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "set_prim: %s", cudaGetErrorString(e));
  b->launches += b->precision == FV_PREC_FP64 ? 1 : 2;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  b->state_set[inst] = 1;
  b->slot_valid[inst] = 0;
  return FV_OK;
}

int fvgpu_batch_init_problem(fv_batch* b, int inst) {
  if (!b || !b->buf) return b ? Fail(b, FV_ERR_STATE, "batch not configured") : FV_ERR_PARAM;
  if (inst < 0 || inst >= b->n) return Fail(b, FV_ERR_PARAM, "problem index %d out of range", inst);
  fv::InitSpec spec;
  if (fv::make_init_spec(b->p[inst], &spec) != FV_OK)
    return Fail(b, FV_ERR_PARAM, "problem %d: unknown problem '%.63s'", inst, b->p[inst].problem);
  const Grid& G = b->G[inst];
  int slot_of[5];
  StorageOrder(G.plane, slot_of);
  // the generator writes FP64 primitives where set_prim's copies land
  Fields stage = b->precision == FV_PREC_FP64 ? Current(b, inst) : Fields();
  if (b->precision != FV_PREC_FP64)
    for (int k = 0; k < 5; ++k) stage.f[k] = b->scratch + (size_t)k * G.fstride;
  Fields out;
  for (int v = 0; v < 5; ++v) out.f[v] = stage.f[slot_of[v]];
  b->state_set[inst] = 0;
  int* d_flags = nullptr;
  int flags = 0;
  BCUDA(b, cudaMallocAsync(&d_flags, sizeof(int), b->stream));
  cudaError_t e = cudaMemsetAsync(d_flags, 0, sizeof(int), b->stream);
  if (e == cudaSuccess) e = fv::launch_generate(spec, out, G.pitch, d_flags, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, d_flags, sizeof(int), cudaMemcpyDeviceToHost, b->stream);
  cudaFreeAsync(d_flags, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "generator: %s", cudaGetErrorString(e));
  b->launches += 1;
  // the velocity checks of set_prim, from the generator's flags
  const int out_of_plane = G.plane == fv::PLANE_XY ? 3 : 2;  // w, or v of an x-z run
  const bool wact = b->p[inst].viscosity_active || (G.ndim == 2 && (flags >> out_of_plane & 1)) || G.ndim == 3;
  if (G.ndim == 2 && wact && b->deg_bc[inst] == FV_BC_REFLECTING)
    return Fail(b, FV_ERR_UNSUPPORTED, "a non-zero velocity along a reflecting degenerate axis is not built");
  if ((bool)b->wact[inst] != wact) b->prepared = false;
  b->wact[inst] = wact;
  if (!b->prepared) ReleaseGroups(b);
  if (b->Q[inst].f[0]) BCUDA(b, cudaMemsetAsync(&b->d_ctrl[inst].q_valid, 0, sizeof(int), b->stream));
  e = fv::launch_prim_to_cons2d(G, stage, b->stream);
  if (e == cudaSuccess && b->precision != FV_PREC_FP64)
    e = fv::launch_pairs_from_double(G, stage, Current(b, inst), b->stream);
  if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "init_problem: %s", cudaGetErrorString(e));
  b->launches += b->precision == FV_PREC_FP64 ? 1 : 2;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  b->state_set[inst] = 1;
  b->slot_valid[inst] = 0;
  return FV_OK;
}

int fvgpu_batch_get_prim(fv_batch* b, int inst, double* rho, double* u, double* v, double* w, double* pr) {
  if (!b || !b->buf) return b ? Fail(b, FV_ERR_STATE, "batch not configured") : FV_ERR_PARAM;
  if (inst < 0 || inst >= b->n) return Fail(b, FV_ERR_PARAM, "problem index %d out of range", inst);
  if (!b->state_set[inst]) return Fail(b, FV_ERR_STATE, "problem %d has no state", inst);
  const Grid& G = b->G[inst];
  int slot_of[5];
  StorageOrder(G.plane, slot_of);
  double* ref[5] = {rho, u, v, w, pr};
  double* dst[5];
  for (int k = 0; k < 5; ++k) dst[slot_of[k]] = ref[k];
  Fields S;
  for (int k = 0; k < 5; ++k) S.f[k] = b->scratch + (size_t)k * G.fstride;
  cudaError_t e;
  if (b->precision == FV_PREC_FP64) {
    e = fv::launch_cons_to_prim2d(G, Current(b, inst), S, b->stream);
  } else {
    e = fv::launch_double_from_pairs(G, Current(b, inst), S, b->stream);
    if (e == cudaSuccess) e = fv::launch_cons_to_prim2d(G, S, S, b->stream);
  }
  if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "get_prim: %s", cudaGetErrorString(e));
  if (!b->wact[inst]) BCUDA(b, cudaMemsetAsync(S.f[3], 0, (size_t)G.fstride * sizeof(double), b->stream));
  const size_t rowb = (size_t)G.na * sizeof(double);
  for (int k = 0; k < 5; ++k)
    if (dst[k])
      BCUDA(b, cudaMemcpy2DAsync(dst[k], rowb, S.f[k], (size_t)G.pitch * sizeof(double), rowb, G.rows,
                                 cudaMemcpyDeviceToHost, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return FV_OK;
}

int fvgpu_batch_run(fv_batch* b, long nsteps) {
  if (!b || !b->buf) return b ? Fail(b, FV_ERR_STATE, "batch not configured") : FV_ERR_PARAM;
  if (nsteps < 0) return Fail(b, FV_ERR_PARAM, "nsteps must be >= 0");
  for (int i = 0; i < b->n; ++i)
    if (!b->state_set[i]) return Fail(b, FV_ERR_STATE, "problem %d has no state", i);
  int rc = Prepare(b);
  if (rc) return rc;
  rc = EnsureSlots(b);
  if (rc) return rc;
  if (MultiEligible(b)) {  // small problems: every step in one launch
    rc = PrepareMulti(b);
    if (rc == FV_OK && nsteps > 0) rc = RunMulti(b, (int)std::min<long>(nsteps, 1L << 30), 2);
    return rc;
  }
  long done = 0;
  // Euler ping-pong: graphs are captured for an even start (state in A)
  if (b->ts != FV_TS_RK2 && b->flip && nsteps > 0) {
    rc = EnqueueStep(b);
    if (rc) return rc;
    b->launches += KernelsPerStep(b);
    done = 1;
  }
  if (nsteps - done >= kGraphSteps) {
    if (!b->graph) {
      cudaGraph_t g;
      const int flip0 = b->flip;
      BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < kGraphSteps; ++k) {
        rc = EnqueueStep(b);
        if (rc) {
          cudaStreamEndCapture(b->stream, &g);
          return rc;
        }
      }
      BCUDA(b, cudaStreamEndCapture(b->stream, &g));
      cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
      b->flip = flip0;
    }
    while (nsteps - done >= kGraphSteps) {
      BCUDA(b, cudaGraphLaunch(b->graph, b->stream));
      b->launches += (long)kGraphSteps * KernelsPerStep(b);
      done += kGraphSteps;
    }
  }
  for (; done < nsteps; ++done) {
    rc = EnqueueStep(b);
    if (rc) return rc;
    b->launches += KernelsPerStep(b);
  }
  return FV_OK;
}

int fvgpu_batch_times(fv_batch* b, double* t) {
  if (!b || !t) return b ? Fail(b, FV_ERR_PARAM, "null argument") : FV_ERR_PARAM;
  int rc = ReadCtrl(b);
  if (rc) return rc;
  int bad = -1;
  for (int i = 0; i < b->n; ++i) {
    t[i] = b->h_ctrl[i].t;
    if (b->h_ctrl[i].err && bad < 0) bad = i;
  }
  if (bad >= 0)
    return Fail(b, ErrStatus(b->h_ctrl[bad].err), "problem %d met a non-finite state or dt, or a wait gave up", bad);
  return FV_OK;
}

int fvgpu_batch_set_stream(fv_batch* b, void* stream) {
  if (!b) return FV_ERR_PARAM;
  if (b->stream) cudaStreamSynchronize(b->stream);
  b->stream = stream ? (cudaStream_t)stream : b->own_stream;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graph_loop) cudaGraphExecDestroy(b->graph_loop);
  b->graph = nullptr;
  b->graph_loop = nullptr;
  return FV_OK;
}

int fvgpu_batch_synchronize(fv_batch* b) {
  if (!b) return FV_ERR_PARAM;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return FV_OK;
}

int fvgpu_batch_launch_count(const fv_batch* b, long* count) {
  if (!b || !count) return FV_ERR_PARAM;
  *count = b->launches;
  return FV_OK;
}

int fvgpu_batch_schedule(fv_batch* b, int* ngroups, int* tx, int* rows, int* block_rows, int* split_viscous,
                         int max_groups) {
  if (!b || !ngroups) return FV_ERR_PARAM;
  for (int i = 0; i < b->n; ++i)
    if (!b->state_set[i]) return Fail(b, FV_ERR_STATE, "problem %d has no state", i);
  int rc = Prepare(b);
  if (rc) return rc;
  *ngroups = (int)b->groups.size();
  for (int gi = 0; gi < *ngroups && gi < max_groups; ++gi) {
    const Group& g = b->groups[gi];
    Schedule sc;
    if (g.ndim == 3) {  // column blocks of 16 x 16 marched over chunks of `rows` z layers
      sc = Schedule3d(b, g.rows);
    } else {
      sc = ShapeSchedule(b, g.shape);
      if (g.rows > 0) sc.rows = g.rows;
    }
    if (tx) tx[gi] = sc.tx;
    if (rows) rows[gi] = sc.rows;
    if (block_rows) block_rows[gi] = sc.block_rows;
    if (split_viscous) split_viscous[gi] = sc.vface;
  }
  return FV_OK;
}

int fvgpu_batch_tiling(fv_batch* b, int* ngroups, int* tx, int* ty, int max_groups) {
  if (!b || !ngroups) return FV_ERR_PARAM;
  for (int i = 0; i < b->n; ++i)
    if (!b->state_set[i]) return Fail(b, FV_ERR_STATE, "problem %d has no state", i);
  int rc = Prepare(b);
  if (rc) return rc;
  const fv::TileShape* shapes;
  NumShapes(b->precision, &shapes);
  *ngroups = (int)b->groups.size();
  for (int g = 0; g < *ngroups && g < max_groups; ++g) {
    const bool d3 = b->groups[g].ndim == 3;
    if (tx) tx[g] = d3 ? fv::batch3d_columns() : shapes[b->groups[g].shape].tx;
    if (ty) ty[g] = d3 ? fv::batch3d_columns()
                       : (b->groups[g].rows > 0 ? b->groups[g].rows : shapes[b->groups[g].shape].ty);
  }
  return FV_OK;
}

}  // extern "C"

// ---- one problem through the batch machinery --------------------------------
// fvgpu_create hands a problem in the FP32-mixed form to a batch of one; these
// give that handle the single-problem calls the batch API does not have.

namespace fv {

const char* batch_error(const fv_batch* b) { return b ? b->err.c_str() : "null handle"; }

// ComputeDtFunctor::computeDt of problem i's current state.
int batch_compute_dt(fv_batch* b, int i, double* dt, double inv[3]) {
  if (!b->state_set[i]) return Fail(b, FV_ERR_STATE, "no state set");
  int rc = Prepare(b);
  if (rc) return rc;
  rc = EnsureSlots(b);
  if (rc) return rc;
  rc = ReadCtrl(b);
  if (rc) return rc;
  const StepCtrl& c = b->h_ctrl[i];
  double inv_hyp;
  const unsigned long long bits = c.slot[c.step & 1];
  std::memcpy(&inv_hyp, &bits, sizeof(inv_hyp));
  double m = inv_hyp;
  if (b->inv_tc[i] > m) m = b->inv_tc[i];
  if (b->inv_visc[i] > m) m = b->inv_visc[i];
  const double d = b->p[i].CFL / m;
  if (inv) {
    inv[0] = inv_hyp;
    inv[1] = b->inv_tc[i];
    inv[2] = b->inv_visc[i];
  }
  if (dt) *dt = d;
  if (c.err) return Fail(b, ErrStatus(c.err), "non-finite state or a wait that gave up (dt = %g)", d);
  if (!std::isfinite(d)) return Fail(b, FV_ERR_NONFINITE, "non-finite state or dt (dt = %g)", d);
  return FV_OK;
}

// One step of every problem with the given dt (UpdateFunctor::update(Q, U, dt)).
int batch_step_dt(fv_batch* b, double dt) {
  for (int i = 0; i < b->n; ++i)
    if (!b->state_set[i]) return Fail(b, FV_ERR_STATE, "problem %d has no state", i);
  int rc = Prepare(b);
  if (rc) return rc;
  rc = EnqueueStep(b, 0, dt);
  if (rc) return rc;
  b->launches += KernelsPerStep(b);
  for (int i = 0; i < b->n; ++i) b->slot_valid[i] = 1;  // the last stage reduced the next slot
  return FV_OK;
}

// The main.cpp:51-74 loop (while t + epsilon < tend, at most max_steps) for
// a batch of one, steps replayed from a graph in the control blocks' own
// mode, the control block read back between replays.
int batch_advance(fv_batch* b, double tend, long max_steps, double* t, long* nsteps) {
  if (b->n != 1) return Fail(b, FV_ERR_PARAM, "batch_advance runs a batch of one");
  if (!b->state_set[0]) return Fail(b, FV_ERR_STATE, "no state set");
  int rc = Prepare(b);
  if (rc) return rc;
  rc = EnsureSlots(b);
  if (rc) return rc;
  rc = ReadCtrl(b);
  if (rc) return rc;
  StepCtrl c = b->h_ctrl[0];
  const long long step0 = c.step;
  c.mode = 1;
  c.t = *t;
  c.tend = tend;
  c.max_steps = max_steps > 0 ? step0 + max_steps : 0;
  BCUDA(b, cudaMemcpyAsync(b->d_ctrl, &c, sizeof(StepCtrl), cudaMemcpyHostToDevice, b->stream));
  const bool short_run = max_steps > 0 && max_steps < kGraphSteps;
  const bool multi = MultiEligible(b);
  if (multi) {
    rc = PrepareMulti(b);
    if (rc) return rc;
  }
  for (;;) {
    if (multi) {  // the kernel stops by itself at the time bound or max_steps
      rc = RunMulti(b, kMultiChunk, -1);
      if (rc) return rc;
      rc = ReadCtrl(b);
      if (rc) return rc;
      if (b->h_ctrl[0].err || !b->h_ctrl[0].active) break;
      continue;
    }
    if (short_run) {
      for (long k = 0; k < max_steps; ++k) {
        rc = EnqueueStep(b, -1, 0.0);
        if (rc) return rc;
        b->launches += KernelsPerStep(b);
      }
    } else {
      if (!b->graph_loop || (b->ts != FV_TS_RK2 && b->flip)) {
        // Euler ping-pong: a graph is captured for an even start (state in A)
        if (b->ts != FV_TS_RK2 && b->flip) {
          rc = EnqueueStep(b, -1, 0.0);
          if (rc) return rc;
          b->launches += KernelsPerStep(b);
        }
        if (!b->graph_loop) {
          cudaGraph_t g;
          const int flip0 = b->flip;
          BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
          for (int k = 0; k < kGraphSteps; ++k) {
            rc = EnqueueStep(b, -1, 0.0);
            if (rc) {
              cudaStreamEndCapture(b->stream, &g);
              return rc;
            }
          }
          BCUDA(b, cudaStreamEndCapture(b->stream, &g));
          cudaError_t e = cudaGraphInstantiate(&b->graph_loop, g, 0);
          cudaGraphDestroy(g);
          if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
          b->flip = flip0;
        }
      }
      BCUDA(b, cudaGraphLaunch(b->graph_loop, b->stream));
      b->launches += (long)kGraphSteps * KernelsPerStep(b);
      if (b->ts != FV_TS_RK2 && (kGraphSteps & 1)) b->flip ^= 1;
    }
    rc = ReadCtrl(b);
    if (rc) return rc;
    if (short_run || b->h_ctrl[0].err || !b->h_ctrl[0].active) break;
  }
  b->slot_valid[0] = 1;
  *t = b->h_ctrl[0].t;
  if (nsteps) *nsteps = (long)(b->h_ctrl[0].step - step0);
  if (b->h_ctrl[0].err) return Fail(b, ErrStatus(b->h_ctrl[0].err), "non-finite state or dt, or a wait that gave up, during advance");
  return FV_OK;
}

// Conserved totals of problem i (compensated sums on the host, in the
// reference's field order).
int batch_totals(fv_batch* b, int i, double out[5]) {
  if (!b->state_set[i]) return Fail(b, FV_ERR_STATE, "no state set");
  const Grid& G = b->G[i];
  Fields S;
  for (int k = 0; k < 5; ++k) S.f[k] = b->scratch + (size_t)k * G.fstride;
  cudaError_t e = b->precision == FV_PREC_FP64
                      ? cudaSuccess
                      : fv::launch_double_from_pairs(G, Current(b, i), S, b->stream);
  if (e != cudaSuccess) return Fail(b, FV_ERR_CUDA, "totals: %s", cudaGetErrorString(e));
  const Fields& src = b->precision == FV_PREC_FP64 ? Current(b, i) : S;
  int slot_of[5];
  StorageOrder(G.plane, slot_of);
  std::vector<double> h((size_t)G.na * G.rows);
  for (int k = 0; k < 5; ++k) {
    const int v = slot_of[k];
    if (v == 3 && !b->wact[i]) {
      out[k] = 0.0;
      continue;
    }
    BCUDA(b, cudaMemcpy2DAsync(h.data(), (size_t)G.na * sizeof(double), src.f[v], (size_t)G.pitch * sizeof(double),
                               (size_t)G.na * sizeof(double), G.rows, cudaMemcpyDeviceToHost, b->stream));
    BCUDA(b, cudaStreamSynchronize(b->stream));
    double sum = 0.0, comp = 0.0;
    for (double x : h) {
      const double t = sum + x;
      comp += std::fabs(sum) >= std::fabs(x) ? (sum - t) + x : (x - t) + sum;
      sum = t;
    }
    out[k] = sum + comp;
  }
  return FV_OK;
}

cudaStream_t batch_stream(const fv_batch* b) { return b->stream; }

}  // namespace fv
