// fv3d_main.cpp -- command-line driver, the counterpart of the reference's
// main.cpp (main.cpp:12-89) on the GB300 path.
//
//   fv3d settings.ini [--ic state.bin] [--out prefix] [--device-loop]
//                     [--write-ic state.bin] [--restart] [--format h5|raw]
//
// Reads the same .ini file (readInifile semantics), sets the initial state,
// and runs the reference's time loop: while (t + epsilon < tend) { dt =
// computeDt; log every log_frequency steps; save when due; update; t += dt }.
// Every problem generator of Init.h runs on the GPU (sod_x, sod_y, sod_z,
// blast, diffusion, rayleigh-taylor, H84, C91: fvgpu_init_problem, the
// state written in place as init.init(Q); primToCons(Q, U) do).  H84 and C91
// draw their perturbations from Kokkos' XorShift64 pool in the reference,
// whose sequence depends on the thread schedule; here each cell draws from a
// counter-based splitmix64 stream of [misc] seed instead (the same stream as
// fv3d_gb300.problems.uniform), so the runs are reproducible but not
// bit-identical to a reference run.  Any other initial state is read with --ic
// from a raw file of 5 float64 arrays (rho, u, v, w, p), each Nz*Ny*Nx in C
// order; --write-ic writes the generated state in that format (generated
// into host arrays with fvgpu_generate, then set with fvgpu_set_prim: the
// same state).  Snapshots go, as the reference's IOManager writes them, to
// <prefix>.h5 (fv_h5_save: group ite_<n> per save) with an XDMF index
// <prefix>.xdmf naming its datasets; --format raw writes them as the raw
// format above instead (<prefix>_<ite>.bin, vertex coordinates in
// <prefix>_grid.bin) with the XDMF index pointing into those files.
//
// --device-loop runs the steps between two saves with fvgpu_advance (dt stays
// on the GPU) instead of one compute_dt/step round trip per step.
//
// Checkpoint / restart: every save also writes <prefix>_restart.bin (the
// conserved state, so a restarted run continues bit for bit; primitives in
// the FP32-mixed form, which keeps no FP64 conserved state) and
// <prefix>_restart.txt (time, next save time, counters, the snapshot list).
// --restart resumes the run of the same prefix from its last save: the same
// steps follow, the snapshots continue their numbering and the XDMF index
// keeps the earlier ones.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "fv3d_gb300.h"

namespace {

struct Fields {
  std::vector<double> f[5];
};

bool ReadRaw(const std::string& path, size_t n, Fields& q) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  bool ok = true;
  for (auto& a : q.f) {
    a.resize(n);
    ok = ok && std::fread(a.data(), sizeof(double), n, f) == n;
  }
  std::fclose(f);
  return ok;
}

bool WriteRaw(const std::string& path, const Fields& q) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = true;
  for (const auto& a : q.f) ok = ok && std::fwrite(a.data(), sizeof(double), a.size(), f) == a.size();
  std::fclose(f);
  return ok;
}

std::string BaseName(const std::string& path) {
  const size_t k = path.find_last_of('/');
  return k == std::string::npos ? path : path.substr(k + 1);
}

// Vertex coordinates as IOManager.h:115-124 writes them ((i - ibeg) * dx,
// ...; no xmin offset), three arrays of (Nz+1)(Ny+1)(Nx+1) doubles.
bool WriteGrid(const std::string& path, const fv_params& p) {
  Fields g;
  const size_t nv = (size_t)(p.Nx + 1) * (p.Ny + 1) * (p.Nz + 1);
  for (int a = 0; a < 3; ++a) g.f[a].reserve(nv);
  for (int k = 0; k <= p.Nz; ++k)
    for (int j = 0; j <= p.Ny; ++j)
      for (int i = 0; i <= p.Nx; ++i) {
        g.f[0].push_back(i * p.dx);
        g.f[1].push_back(j * p.dy);
        g.f[2].push_back(k * p.dz);
      }
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  bool ok = true;
  for (int a = 0; a < 3; ++a) ok = ok && std::fwrite(g.f[a].data(), sizeof(double), nv, f) == nv;
  std::fclose(f);
  return ok;
}

// The XDMF index of the snapshots, laid out like the reference's
// (IOManager.h:16-77: a temporal collection over one 3DSMesh / X_Y_Z
// geometry; per save rho, a velocity vector joined from u, v, w, and prs).
// Its data items name the HDF5 datasets of `h5` (Format="HDF",
// file:/ite_<n>/rho, as the reference's) or, with `h5` empty, point into the
// raw files (Format="Binary", Seek = byte offset of the field; `grid` holds
// the vertex coordinates).
bool WriteXdmf(const std::string& path, const fv_params& p, const std::string& grid, const std::string& h5,
               const std::vector<std::pair<std::string, double>>& snaps) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  const int nx = p.Nx, ny = p.Ny, nz = p.Nz;
  const size_t nv = (size_t)(nx + 1) * (ny + 1) * (nz + 1), nc = (size_t)nx * ny * nz;
  static const char* kField[5] = {"rho", "u", "v", "w", "prs"};
  // field v (0-4: rho, u, v, w, prs of save n; 5-7: x, y, z) with extents a x b x c
  auto item = [&](size_t n, int v, int a, int b, int c) {
    if (!h5.empty()) {
      const std::string ds = v >= 5 ? std::string(1, "xyz"[v - 5]) : "ite_" + std::to_string(n) + "/" + kField[v];
      std::fprintf(f, "<DataItem Dimensions=\"%d %d %d\" NumberType=\"Float\" Precision=\"8\" Format=\"HDF\">%s:/%s"
                      "</DataItem>", a, b, c, h5.c_str(), ds.c_str());
      return;
    }
    const std::string& file = v >= 5 ? grid : snaps[n].first;
    const size_t seek = v >= 5 ? (size_t)(v - 5) * nv * sizeof(double) : (size_t)v * nc * sizeof(double);
    std::fprintf(f,
                 "<DataItem Dimensions=\"%d %d %d\" NumberType=\"Float\" Precision=\"8\" Format=\"Binary\" "
                 "Endian=\"Little\" Seek=\"%zu\">%s</DataItem>",
                 a, b, c, seek, file.c_str());
  };
  std::fprintf(f, "<?xml version=\"1.0\" ?>\n<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n<Xdmf Version=\"2.0\">\n"
                  "<Domain CollectionType=\"Temporal\">\n"
                  "  <Grid Name=\"MainTimeSeries\" GridType=\"Collection\" CollectionType=\"Temporal\">\n"
                  "    <Topology Name=\"Main Topology\" TopologyType=\"3DSMesh\" NumberOfElements=\"%d %d %d\"/>\n"
                  "    <Geometry Name=\"Main Geometry\" GeometryType=\"X_Y_Z\">\n",
               nz + 1, ny + 1, nx + 1);
  for (int a = 0; a < 3; ++a) {
    std::fprintf(f, "      ");
    item(0, 5 + a, nz + 1, ny + 1, nx + 1);
    std::fprintf(f, "\n");
  }
  std::fprintf(f, "    </Geometry>\n");
  for (size_t n = 0; n < snaps.size(); ++n) {
    const auto& sn = snaps[n];
    std::fprintf(f,
                 "    <Grid Name=\"Cells\" GridType=\"Uniform\">\n      <Time TimeType=\"Single\" Value=\"%.17g\" />\n"
                 "      <Topology Reference=\"//Topology[@Name='Main Topology']\" />\n"
                 "      <Geometry Reference=\"//Geometry[@Name='Main Geometry']\" />\n",
                 sn.second);
    std::fprintf(f, "      <Attribute Name=\"rho\" AttributeType=\"Scalar\" Center=\"Cell\">\n        ");
    item(n, 0, nz, ny, nx);
    std::fprintf(f, "\n      </Attribute>\n");
    std::fprintf(f, "      <Attribute Name=\"velocity\" AttributeType=\"Vector\" Center=\"Cell\">\n"
                    "        <DataItem Dimensions=\"%d %d %d 3\" ItemType=\"Function\" Function=\"JOIN($0, $1, $2)\">\n",
                 nz, ny, nx);
    for (int v = 1; v <= 3; ++v) {
      std::fprintf(f, "          ");
      item(n, v, nz, ny, nx);
      std::fprintf(f, "\n");
    }
    std::fprintf(f, "        </DataItem>\n      </Attribute>\n");
    std::fprintf(f, "      <Attribute Name=\"prs\" AttributeType=\"Scalar\" Center=\"Cell\">\n        ");
    item(n, 4, nz, ny, nx);
    std::fprintf(f, "\n      </Attribute>\n    </Grid>\n");
  }
  std::fprintf(f, "  </Grid>\n</Domain>\n</Xdmf>\n");
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok;
}

// The loop's position at a save, enough to resume it exactly.
struct Checkpoint {
  double t = 0.0, next_save = 0.0;
  int ite = 0, next_log = 0, conserved = 1;
  long steps = 0;
  std::vector<std::pair<std::string, double>> snaps;
};

bool WriteCheckpoint(const std::string& prefix, const Checkpoint& c, const Fields& state) {
  if (!WriteRaw(prefix + "_restart.bin", state)) return false;
  FILE* f = std::fopen((prefix + "_restart.txt").c_str(), "w");
  if (!f) return false;
  std::fprintf(f, "fv3d-restart 1\nt %.17g\nnext_save %.17g\nite %d\nnext_log %d\nsteps %ld\nconserved %d\n", c.t,
               c.next_save, c.ite, c.next_log, c.steps, c.conserved);
  for (const auto& sn : c.snaps) std::fprintf(f, "snap %.17g %s\n", sn.second, sn.first.c_str());
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok;
}

bool ReadCheckpoint(const std::string& prefix, size_t n, Checkpoint& c, Fields& state) {
  FILE* f = std::fopen((prefix + "_restart.txt").c_str(), "r");
  if (!f) return false;
  char key[64], name[1024];
  int version = 0;
  bool ok = std::fscanf(f, "%63s %d", key, &version) == 2 && !std::strcmp(key, "fv3d-restart") && version == 1 &&
            std::fscanf(f, " t %lg next_save %lg ite %d next_log %d steps %ld conserved %d", &c.t, &c.next_save,
                        &c.ite, &c.next_log, &c.steps, &c.conserved) == 6;
  double ts;
  while (ok && std::fscanf(f, " snap %lg %1023s", &ts, name) == 2) c.snaps.emplace_back(name, ts);
  std::fclose(f);
  return ok && ReadRaw(prefix + "_restart.bin", n, state);
}

int Check(fv_sim* s, int rc, const char* what) {
  if (rc != FV_OK) std::fprintf(stderr, "%s: %s (%s)\n", what, fv_status_string(rc), fvgpu_last_error(s));
  return rc;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr,
                 "usage: fv3d settings.ini [--ic state.bin] [--out prefix] [--device-loop] [--write-ic state.bin] "
                 "[--restart] [--format h5|raw]\n");
    return 2;
  }
  std::string ini = argv[1], ic, out, write_ic;
  bool device_loop = false, restart = false, raw = false;
  for (int a = 2; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--ic") && a + 1 < argc) ic = argv[++a];
    else if (!std::strcmp(argv[a], "--restart")) restart = true;
    else if (!std::strcmp(argv[a], "--out") && a + 1 < argc) out = argv[++a];
    else if (!std::strcmp(argv[a], "--device-loop")) device_loop = true;
    else if (!std::strcmp(argv[a], "--write-ic") && a + 1 < argc) write_ic = argv[++a];
    else if (!std::strcmp(argv[a], "--format") && a + 1 < argc && (!std::strcmp(argv[a + 1], "h5") ||
                                                                   !std::strcmp(argv[a + 1], "raw")))
      raw = !std::strcmp(argv[++a], "raw");
    else {
      std::fprintf(stderr, "unknown argument %s\n", argv[a]);
      return 2;
    }
  }
  fv_params p;
  fv_read_ini(ini.c_str(), &p);
  if (out.empty()) out = p.filename_out;
  const size_t n = (size_t)p.Nx * p.Ny * p.Nz;
  Fields q;
  Checkpoint ck;
  if (restart) {
    if (!ReadCheckpoint(out, n, ck, q)) {
      std::fprintf(stderr, "cannot read the checkpoint %s_restart.txt / .bin\n", out.c_str());
      return 1;
    }
  } else if (!ic.empty()) {
    if (!ReadRaw(ic, n, q)) {
      std::fprintf(stderr, "cannot read %zu cells from %s\n", n, ic.c_str());
      return 1;
    }
  } else if (!write_ic.empty()) {  // generated on the GPU into host arrays, written, then set
    for (auto& a : q.f) a.resize(n);
    if (fvgpu_generate(&p, q.f[0].data(), q.f[1].data(), q.f[2].data(), q.f[3].data(), q.f[4].data()) != FV_OK) {
      std::fprintf(stderr, "Error unknown problem %s (give --ic)\n", p.problem);
      return 1;
    }
  }
  const bool on_device = !restart && ic.empty() && write_ic.empty();  // fvgpu_init_problem
  if (!write_ic.empty() && !WriteRaw(write_ic, q)) {
    std::fprintf(stderr, "cannot write %s\n", write_ic.c_str());
    return 1;
  }
  fv_sim* s = nullptr;
  if (Check(s, fvgpu_create(&p, &s), "fvgpu_create")) return 1;
  const double* qs[5] = {q.f[0].data(), q.f[1].data(), q.f[2].data(), q.f[3].data(), q.f[4].data()};
  if (on_device) {
    if (Check(s, fvgpu_init_problem(s), "init_problem")) return 1;
  } else if (restart && ck.conserved) {
    if (Check(s, fvgpu_set_cons(s, qs[0], qs[1], qs[2], qs[3], qs[4]), "set_cons")) return 1;
  } else if (Check(s, fvgpu_set_prim(s, qs[0], qs[1], qs[2], qs[3], qs[4]), "set_prim")) {
    return 1;
  }
  const bool fp64 = p.precision == FV_PREC_FP64;
  for (auto& a : q.f) a.resize(n);  // host copy of the state for the saves (empty after an on-device start)

  double t = ck.t, dt = 0.0, next_save = ck.next_save;
  int ite = ck.ite, next_log = ck.next_log;
  long steps = ck.steps;
  // the loop announces its saves (main.cpp:64); the final one is silent (main.cpp:76)
  std::vector<std::pair<std::string, double>> snaps = ck.snaps;
  const std::string grid = out + "_grid.bin";
  Fields cons;
  auto save = [&](double tt, bool announce, double next) {
    fvgpu_get_prim(s, q.f[0].data(), q.f[1].data(), q.f[2].data(), q.f[3].data(), q.f[4].data());
    char name[512];
    std::snprintf(name, sizeof(name), "%s_%04d.bin", out.c_str(), ite);
    if (announce) std::printf(" - Saving at time %g\n", tt);
    snaps.emplace_back(BaseName(name), tt);
    if (raw) {
      if (snaps.size() == 1) WriteGrid(grid, p);
      WriteRaw(name, q);
      WriteXdmf(out + ".xdmf", p, BaseName(grid), "", snaps);
    } else {  // IOManager::saveSolution: <out>.h5, group ite_<n>
      const int rc = fv_h5_save(&p, (out + ".h5").c_str(), ite, tt, q.f[0].data(), q.f[1].data(), q.f[2].data(),
                                q.f[3].data(), q.f[4].data());
      if (rc != FV_OK) std::fprintf(stderr, "cannot write %s.h5 (%s)\n", out.c_str(), fv_status_string(rc));
      WriteXdmf(out + ".xdmf", p, "", BaseName(out) + ".h5", snaps);
    }
    ++ite;
    Checkpoint c;
    c.t = tt;
    c.next_save = next;
    c.ite = ite;
    c.next_log = next_log;
    c.steps = steps;
    c.conserved = fp64 ? 1 : 0;
    c.snaps = snaps;
    if (fp64) {
      for (auto& v : cons.f) v.resize(n);
      fvgpu_get_cons(s, cons.f[0].data(), cons.f[1].data(), cons.f[2].data(), cons.f[3].data(), cons.f[4].data());
    }
    if (!WriteCheckpoint(out, c, fp64 ? cons : q))
      std::fprintf(stderr, "cannot write the checkpoint of %s\n", out.c_str());
  };
  while (t + p.epsilon < p.tend) {
    const bool save_needed = (t + p.epsilon > next_save);
    double inv[3];
    if (Check(s, fvgpu_compute_dt(s, &dt, inv), "compute_dt")) return 1;
    if (next_log == 0) {
      std::printf("Computing dts at (t=%g) : dt_hyp=%g; dt_TC=%g; dt_visc=%g\n", t, 1.0 / inv[0], 1.0 / inv[1],
                  1.0 / inv[2]);
      next_log = p.log_frequency;
    } else {
      next_log--;
    }
    if (save_needed) {
      save(t, true, next_save + p.save_freq);
      next_save += p.save_freq;
    }
    if (device_loop) {
      // run on the device up to the next save time (or tend)
      long k = 0;
      const double bound = std::fmin(p.tend, next_save);
      if (Check(s, fvgpu_advance(s, bound, 0, &t, &k), "advance")) return 1;
      steps += k;
      if (k == 0) {  // next_save within epsilon: take one ordinary step
        if (Check(s, fvgpu_step(s, dt), "step")) return 1;
        t += dt;
        ++steps;
      }
    } else {
      if (Check(s, fvgpu_step(s, dt), "step")) return 1;
      t += dt;
      ++steps;
    }
  }
  save(t, false, next_save);
  std::printf("done: %ld steps, t = %.17g\n", steps, t);
  fvgpu_destroy(s);
  return 0;
}
