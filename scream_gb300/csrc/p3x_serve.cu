/* Serving loop of libp3x (continuous batching of P3 steps). */
#include "p3x.h"

extern "C" {

int p3x_server_create(p3x_context*, const p3x_runtime*, int64_t, int32_t, p3x_server** out) {
  if (out) *out = nullptr;
  return P3X_EINVAL;
}
int p3x_server_destroy(p3x_server*) { return P3X_EINVAL; }
int p3x_server_submit(p3x_server*, int64_t, int32_t, int32_t, int32_t, int32_t, uint64_t, double, double) {
  return P3X_EINVAL;
}
int p3x_server_run_poisson(p3x_server*, double, int32_t, int32_t, uint64_t, p3x_serve_stats*) {
  return P3X_EINVAL;
}
int p3x_server_read_field(p3x_server*, int64_t, int32_t, double*, int64_t) { return P3X_EINVAL; }
int p3x_server_drain(p3x_server*, p3x_serve_stats*) { return P3X_EINVAL; }

}  // extern "C"
