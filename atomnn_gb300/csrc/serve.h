// serve.h - continuous-batching request loop behind nnpgpu_serve_* (include/nnpgpu.h).
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/nnpgpu.h"

struct nnpgpu_ctx;

namespace nnpgpu {

class Serving {
 public:
  Serving(nnpgpu_ctx* c, const nnpgpu_serve_opts& o);
  ~Serving();
  int submit(int natoms, const double* posn, const int* species, const double* cell, long long key, long long* id);
  int poll(long long id, double* energy, double* force, double* latency);

 private:
  struct Impl;
  Impl* impl_;
};

}  // namespace nnpgpu
