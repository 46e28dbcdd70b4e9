// fv_batch.cpp -- extern "C" entry points for batches of independent problems.
//
// Placeholder until the persistent batched kernel lands: every call reports
// FV_ERR_UNSUPPORTED with a message.
#include <string>

#include "fv3d_gb300.h"

struct fv_batch {
  std::string err;
};

namespace {
int Unsupported(fv_batch* b) {
  if (b) b->err = "batched problems are not built yet";
  return FV_ERR_UNSUPPORTED;
}
}  // namespace

extern "C" {

int fvgpu_batch_create(const fv_params* params, int n, fv_batch** out) {
  (void)params;
  (void)n;
  if (!out) return FV_ERR_PARAM;
  *out = new fv_batch();
  return Unsupported(*out);
}
int fvgpu_batch_destroy(fv_batch* b) {
  delete b;
  return FV_OK;
}
const char* fvgpu_batch_last_error(const fv_batch* b) { return b ? b->err.c_str() : "null handle"; }
int fvgpu_batch_set_prim(fv_batch* b, int, const double*, const double*, const double*, const double*,
                         const double*) {
  return Unsupported(b);
}
int fvgpu_batch_get_prim(fv_batch* b, int, double*, double*, double*, double*, double*) { return Unsupported(b); }
int fvgpu_batch_run(fv_batch* b, long) { return Unsupported(b); }
int fvgpu_batch_times(fv_batch* b, double*) { return Unsupported(b); }
int fvgpu_batch_set_stream(fv_batch* b, void*) { return Unsupported(b); }
int fvgpu_batch_synchronize(fv_batch* b) { return Unsupported(b); }
int fvgpu_batch_launch_count(const fv_batch* b, long* c) {
  (void)b;
  if (c) *c = 0;
  return FV_OK;
}

}  // extern "C"
