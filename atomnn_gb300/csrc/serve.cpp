// serve.cpp - placeholder until the serving loop lands.
#include "context.h"

namespace nnpgpu {
struct Serving::Impl {};
Serving::Serving(nnpgpu_ctx*, const nnpgpu_serve_opts&) : impl_(new Impl) {}
Serving::~Serving() { delete impl_; }
int Serving::submit(int, const double*, const int*, const double*, long long, long long*) { return NNPGPU_ERR_UNSUPPORTED; }
int Serving::poll(long long, double*, double*, double*) { return NNPGPU_ERR_UNSUPPORTED; }
}  // namespace nnpgpu

extern "C" int nnpgpu_serve_start(nnpgpu_ctx* c, const nnpgpu_serve_opts*) {
  return nnpgpu::set_error(c, NNPGPU_ERR_UNSUPPORTED, "serving not built yet");
}
extern "C" int nnpgpu_submit(nnpgpu_ctx* c, int, const double*, const int*, const double*, long long, long long*) {
  return nnpgpu::set_error(c, NNPGPU_ERR_UNSUPPORTED, "serving not built yet");
}
extern "C" int nnpgpu_poll(nnpgpu_ctx* c, long long, double*, double*, double*) {
  return nnpgpu::set_error(c, NNPGPU_ERR_UNSUPPORTED, "serving not built yet");
}
extern "C" int nnpgpu_serve_stop(nnpgpu_ctx* c) { return nnpgpu::set_error(c, NNPGPU_ERR_UNSUPPORTED, "serving not built yet"); }
