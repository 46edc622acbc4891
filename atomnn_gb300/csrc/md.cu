// md.cu - molecular dynamics with the engine as the force field, on resident device state.
//
// The reference's MD job (src/torch/torch.cpp:267-275) steps a structure with an integrator
// (Verlet::compute, src/torch/integrator.cpp:170-193) whose forces come from Engine::compute
// (src/torch/engine.cpp:107-118) and the NNP potential PotNNPE::compute
// (src/torch/pot_nnpe.cpp:175-295): energy with the species vacuum energies, forces with the
// minimum-image rule of NNP::force.  Here positions, velocities, forces and masses stay on the
// GPU for the whole run; a step is two integrator kernels around the engine's batched launch
// sequence (replayed from its CUDA graph).
//
// Neighbour lists: the reference rebuilds a list at the potential cutoff every `stride` steps
// and misses pairs that enter the cutoff in between.  Here a list at rc + skin is kept
// resident and every step refreshes it exactly at rc (neighbour mode 3), so each step's forces
// equal those of a fresh list; the resident list is rebuilt when some atom has moved more than
// skin/2 since it was built.  Structures with more than one image of an atom within rc (image
// shells) get a fresh list every step.
//
// Positions are not wrapped into the cell between steps (the wrapped fractional coordinates
// the neighbour build uses are computed per step anyway); nnpgpu_md_state returns them wrapped
// as Cell::returnToCell does (src/struc/cell.cpp:84-94).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

namespace nnpgpu {

// v += (dt/2) F / m ; x += v dt  (FP64, no contraction: the oracle's rounding)
__global__ void md_kick_drift_kernel(int n, double hdt, double dt, const double* __restrict__ mass, const double* __restrict__ F,
                                     double* __restrict__ v, double* __restrict__ x) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 3 * n) return;
  const double m = mass[k / 3];
  const double vk = __dadd_rn(v[k], __ddiv_rn(__dmul_rn(hdt, F[k]), m));
  v[k] = vk;
  x[k] = __dadd_rn(x[k], __dmul_rn(vk, dt));
}

// v += (dt/2) F / m, and per-block partial sums of m |v|^2 (fixed order within the block)
__global__ void __launch_bounds__(256) md_kick_kernel(int n, double hdt, const double* __restrict__ mass, const double* __restrict__ F,
                                                      double* __restrict__ v, double* __restrict__ part) {
  __shared__ double red[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0;
  if (i < n) {
    const double m = mass[i];
    double s = 0.0;
    for (int x = 0; x < 3; ++x) {
      const double vk = __dadd_rn(v[3 * i + x], __ddiv_rn(__dmul_rn(hdt, F[3 * i + x]), m));
      v[3 * i + x] = vk;
      s = __dadd_rn(s, __dmul_rn(vk, vk));
    }
    ke = __dmul_rn(m, s);
  }
  red[threadIdx.x] = ke;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out[0] = 0.5 * sum of the block partials, in block order
__global__ void md_sum_kernel(int nb, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s = __dadd_rn(s, part[b]);
  out[0] = __dmul_rn(0.5, s);
}

// largest |x' - x0|^2 over the atoms (as float bits: non-negative floats order as ints), where
// x' are the positions the next md_kick_drift_kernel will write: the same FP64 operations on the
// same v, F and x, so the skin test of the next step is known when this step's energies are read
__global__ void md_disp_next_kernel(int n, double hdt, double dt, const double* __restrict__ mass, const double* __restrict__ F,
                                    const double* __restrict__ v, const double* __restrict__ x, const double* __restrict__ x0,
                                    unsigned* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float d2 = 0.f;
  if (i < n) {
    const double m = mass[i];
    double s = 0.0;
    for (int k = 3 * i; k < 3 * i + 3; ++k) {
      const double vk = __dadd_rn(v[k], __ddiv_rn(__dmul_rn(hdt, F[k]), m));
      const double a = __dsub_rn(__dadd_rn(x[k], __dmul_rn(vk, dt)), x0[k]);
      s = __dadd_rn(s, __dmul_rn(a, a));
    }
    d2 = (float)s;
  }
  for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_xor_sync(0xffffffffu, d2, o));
  if ((threadIdx.x & 31) == 0 && d2 > 0.f) atomicMax(out, __float_as_uint(d2));
}

}  // namespace nnpgpu

using namespace nnpgpu;

struct nnpgpu_md {
  nnpgpu_ctx* c = nullptr;
  int natoms = 0;
  double cell[9] = {};
  double dt = 0.0, skin = 0.0;
  int flags = 0;
  long long step = 0;
  int rebuilds = 0;
  bool use_skin = false;
  // device state
  double *x = nullptr, *v = nullptr, *F = nullptr, *m = nullptr, *x0 = nullptr, *pe = nullptr, *part = nullptr, *ke = nullptr;
  int* type = nullptr;
  unsigned* disp = nullptr;
  // resident neighbour list at rc + skin
  int *sj = nullptr, *scode = nullptr, *scnt = nullptr;
  float4* sr = nullptr;
  int scap = 0;
  double* h = nullptr;  // pinned: pe, ke, displacement word
};

namespace {

int md_fail(nnpgpu_ctx* c, cudaError_t e, const char* where) {
  return set_error(c, NNPGPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

void md_free(nnpgpu_md* s) {
  void* dev[] = {s->x, s->v, s->F, s->m, s->x0, s->pe, s->part, s->ke, s->type, s->disp, s->sj, s->scode, s->scnt, s->sr};
  for (void* p : dev)
    if (p) cudaFree(p);
  if (s->h) cudaFreeHost(s->h);
}

// (re)builds the resident list from the current positions
int md_build(nnpgpu_md* s) {
  nnpgpu_ctx* c = s->c;
  const double rcs = c->pot.rc + s->skin;
  for (int attempt = 0; attempt < 4; ++attempt) {
    if (!s->sj) {
      const size_t slots = (size_t)s->natoms * s->scap;
      if (cudaMalloc(&s->sj, slots * 4) != cudaSuccess || cudaMalloc(&s->scode, slots * 4) != cudaSuccess ||
          cudaMalloc(&s->sr, slots * 16) != cudaSuccess || cudaMalloc(&s->scnt, (size_t)s->natoms * 4) != cudaSuccess) {
        cudaGetLastError();
        return set_error(c, NNPGPU_ERR_OOM, "md: resident neighbour list allocation failed");
      }
    }
    int maxc = 0;
    const int rc = build_skin(c, s->natoms, s->x, s->cell, rcs, s->scap, s->sj, s->scode, s->scnt, s->sr, &maxc, true);
    if (rc == NNPGPU_OK) {
      cudaMemcpyAsync(s->x0, s->x, sizeof(double) * 3 * s->natoms, cudaMemcpyDeviceToDevice, c->stream);
      ++s->rebuilds;
      return NNPGPU_OK;
    }
    if (rc != NNPGPU_ERR_CAPACITY || maxc > 1024) return rc;
    cudaFree(s->sj); cudaFree(s->scode); cudaFree(s->sr); cudaFree(s->scnt);
    s->sj = s->scode = s->scnt = nullptr;
    s->sr = nullptr;
    s->scap = (maxc + 31) / 32 * 32;
  }
  return set_error(c, NNPGPU_ERR_CAPACITY, "md: resident neighbour list capacity retries exhausted");
}

// forces and potential energy at the current positions
int md_forces(nnpgpu_md* s) {
  SkinRef ref;
  if (s->use_skin) {
    ref.j = s->sj;
    ref.code = s->scode;
    ref.cnt = s->scnt;
    ref.cap = s->scap;
  }
  return compute_device_skins(s->c, 1, &s->natoms, s->x, s->type, s->cell, NNPGPU_ENERGY | NNPGPU_FORCE | NNPGPU_BATCHED | s->flags, s->pe,
                              s->F, s->c->stream, s->use_skin ? &ref : nullptr);
}

}  // namespace

extern "C" int nnpgpu_md_create(nnpgpu_ctx* c, int natoms, const double* posn, const double* vel, const int* species, const double* mass,
                                const double* cell, double dt, double skin, int flags, nnpgpu_md** out) {
  if (!out) return NNPGPU_ERR_INVALID;
  *out = nullptr;
  if (!c) return NNPGPU_ERR_INVALID;
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  if (natoms <= 0 || !posn || !species || !mass || !cell) return set_error(c, NNPGPU_ERR_INVALID, "md: invalid arguments");
  if (!(dt > 0) || !(skin >= 0) || !std::isfinite(dt) || !std::isfinite(skin)) return set_error(c, NNPGPU_ERR_INVALID, "md: invalid time step or skin");
  for (int a = 0; a < natoms; ++a) {
    if (species[a] < 0 || species[a] >= c->pot.ntypes) return set_error(c, NNPGPU_ERR_INVALID, "md: species index out of range");
    if (!(mass[a] > 0) || !std::isfinite(mass[a])) return set_error(c, NNPGPU_ERR_INVALID, "md: masses must be positive");
  }
  cudaSetDevice(c->device);
  nnpgpu_md* s = new nnpgpu_md();
  s->c = c;
  s->natoms = natoms;
  std::copy(cell, cell + 9, s->cell);
  s->dt = dt;
  s->skin = skin;
  s->flags = flags & (NNPGPU_BF16);
  // a resident list pays only where a single image of each atom lies within rc (modes 2/4)
  {
    StrucMeta m;
    std::vector<ImgEntry> imgs;
    try {
      make_meta(cell, 0, natoms, c->pot.rc, m, imgs);
    } catch (PotError& e) {
      delete s;
      return set_error(c, e.code, e.what());
    }
    s->use_skin = skin > 0 && (m.mode == 2 || m.mode == 4);
    double vol = std::fabs(cell[0] * (cell[4] * cell[8] - cell[7] * cell[5]) - cell[3] * (cell[1] * cell[8] - cell[7] * cell[2]) +
                           cell[6] * (cell[1] * cell[5] - cell[4] * cell[2]));
    const double rcs = c->pot.rc + skin;
    const double nb = vol > 0 ? natoms / vol * 4.0 / 3.0 * M_PI * std::pow(rcs + 0.5, 3) * 1.25 + 16 : natoms;
    s->scap = std::min(1024, (int)std::ceil(nb / 32.0) * 32);
  }
  const size_t n3 = 3 * (size_t)natoms;
  const int nb = (natoms + 255) / 256;
  bool ok = cudaMalloc(&s->x, n3 * 8) == cudaSuccess && cudaMalloc(&s->v, n3 * 8) == cudaSuccess && cudaMalloc(&s->F, n3 * 8) == cudaSuccess &&
            cudaMalloc(&s->x0, n3 * 8) == cudaSuccess && cudaMalloc(&s->m, (size_t)natoms * 8) == cudaSuccess &&
            cudaMalloc(&s->type, (size_t)natoms * 4) == cudaSuccess && cudaMalloc(&s->pe, 8) == cudaSuccess &&
            cudaMalloc(&s->ke, 8) == cudaSuccess && cudaMalloc(&s->part, (size_t)nb * 8) == cudaSuccess &&
            cudaMalloc(&s->disp, 4) == cudaSuccess && cudaMallocHost(&s->h, 64) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    md_free(s);
    delete s;
    return set_error(c, NNPGPU_ERR_OOM, "md: device allocation failed");
  }
  cudaStream_t st = c->stream;
  cudaMemcpyAsync(s->x, posn, n3 * 8, cudaMemcpyHostToDevice, st);
  if (vel) cudaMemcpyAsync(s->v, vel, n3 * 8, cudaMemcpyHostToDevice, st);
  else cudaMemsetAsync(s->v, 0, n3 * 8, st);
  // the reference's MD job enters its first step with zero forces (torch.cpp:267-275)
  cudaMemsetAsync(s->F, 0, n3 * 8, st);
  cudaMemcpyAsync(s->m, mass, (size_t)natoms * 8, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(s->type, species, (size_t)natoms * 4, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(s->pe, 0, 8, st);
  cudaMemsetAsync(s->ke, 0, 8, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    md_free(s);
    delete s;
    return md_fail(c, e, "md set-up");
  }
  if (s->use_skin) {
    const int rc = md_build(s);
    if (rc != NNPGPU_OK) {
      md_free(s);
      delete s;
      return rc;
    }
  }
  *out = s;
  return NNPGPU_OK;
}

extern "C" int nnpgpu_md_forces(nnpgpu_md* s, double* pe) {
  if (!s) return NNPGPU_ERR_INVALID;
  cudaSetDevice(s->c->device);
  const int rc = md_forces(s);
  if (rc != NNPGPU_OK) return rc;
  if (pe) {
    const cudaError_t e = cudaMemcpy(pe, s->pe, 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return md_fail(s->c, e, "md forces");
  }
  return NNPGPU_OK;
}

extern "C" int nnpgpu_md_run(nnpgpu_md* s, int nsteps, double* pe, double* ke) {
  if (!s || nsteps < 0) return NNPGPU_ERR_INVALID;
  nnpgpu_ctx* c = s->c;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  const int n = s->natoms;
  const int nb = (n + 255) / 256;
  const double hdt = 0.5 * s->dt;
  const float half_skin2 = (float)(0.25 * s->skin * s->skin * (1.0 - 1e-4));  // FP32 test, conservative
  // the displacement the first step's drift will give (later steps read theirs with the
  // previous step's energies)
  auto enqueue_disp_next = [&]() {
    cudaMemsetAsync(s->disp, 0, 4, st);
    md_disp_next_kernel<<<nb, 256, 0, st>>>(n, hdt, s->dt, s->m, s->F, s->v, s->x, s->x0, s->disp);
    cudaMemcpyAsync(s->h + 2, s->disp, 4, cudaMemcpyDeviceToHost, st);
  };
  if (s->use_skin && nsteps > 0) {
    enqueue_disp_next();
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return md_fail(c, e, "md step");
  }
  for (int t = 0; t < nsteps; ++t) {
    bool rebuild = false;
    if (s->use_skin) {
      unsigned bits;
      std::memcpy(&bits, s->h + 2, 4);
      float d2;
      std::memcpy(&d2, &bits, 4);
      rebuild = d2 > half_skin2;
    }
    // first half-step (Verlet::compute, integrator.cpp:172-177)
    md_kick_drift_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(n, hdt, s->dt, s->m, s->F, s->v, s->x);
    if (rebuild) {
      const int rc = md_build(s);
      if (rc != NNPGPU_OK) return rc;
    }
    // forces (Engine::compute -> PotNNPE::compute)
    const int rc = md_forces(s);
    if (rc != NNPGPU_OK) return rc;
    // second half-step and kinetic energy (integrator.cpp:181-189)
    md_kick_kernel<<<nb, 256, 0, st>>>(n, hdt, s->m, s->F, s->v, s->part);
    md_sum_kernel<<<1, 32, 0, st>>>(nb, s->part, s->ke);
    if (s->use_skin && t + 1 < nsteps) enqueue_disp_next();
    cudaMemcpyAsync(s->h, s->pe, 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(s->h + 1, s->ke, 8, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return md_fail(c, e, "md step");
    if (pe) pe[t] = s->h[0];
    if (ke) ke[t] = s->h[1];
    ++s->step;
  }
  return NNPGPU_OK;
}

extern "C" int nnpgpu_md_state(nnpgpu_md* s, double* posn, double* vel, double* force, int* rebuilds) {
  if (!s) return NNPGPU_ERR_INVALID;
  nnpgpu_ctx* c = s->c;
  cudaSetDevice(c->device);
  const size_t n3 = 3 * (size_t)s->natoms;
  if (vel) cudaMemcpyAsync(vel, s->v, n3 * 8, cudaMemcpyDeviceToHost, c->stream);
  if (force) cudaMemcpyAsync(force, s->F, n3 * 8, cudaMemcpyDeviceToHost, c->stream);
  std::vector<double> x(posn ? n3 : 0);
  if (posn) cudaMemcpyAsync(x.data(), s->x, n3 * 8, cudaMemcpyDeviceToHost, c->stream);
  const cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return md_fail(c, e, "md state");
  if (posn) {
    // Cell::returnToCell: fractional coordinates mod (0, 1), back to Cartesian
    StrucMeta m;
    std::vector<ImgEntry> imgs;
    make_meta(s->cell, 0, s->natoms, c->pot.rc, m, imgs);
    const bool periodic = m.mode != 0;
    for (int a = 0; a < s->natoms; ++a) {
      const double* p = &x[3 * (size_t)a];
      if (!periodic) {
        for (int k = 0; k < 3; ++k) posn[3 * (size_t)a + k] = p[k];
        continue;
      }
      double f[3];
      for (int r = 0; r < 3; ++r) f[r] = m.RInv[r] * p[0] + m.RInv[3 + r] * p[1] + m.RInv[6 + r] * p[2];
      for (int r = 0; r < 3; ++r) {
        const double a1 = f[r] - std::trunc(f[r]);
        const double b = a1 + 1.0;
        f[r] = b - std::trunc(b);
      }
      for (int r = 0; r < 3; ++r) posn[3 * (size_t)a + r] = m.R[r] * f[0] + m.R[3 + r] * f[1] + m.R[6 + r] * f[2];
    }
  }
  if (rebuilds) *rebuilds = s->rebuilds;
  return NNPGPU_OK;
}

extern "C" void nnpgpu_md_destroy(nnpgpu_md* s) {
  if (!s) return;
  cudaSetDevice(s->c->device);
  cudaStreamSynchronize(s->c->stream);
  md_free(s);
  delete s;
}
