// gather.cu - forces and per-structure energy.
//
// NNP::force (src/nnp/nnp.cpp:416-482) adds each neighbour-slot contribution W to the centre
// atom and subtracts it from the neighbour only when the slot is the neighbour's minimum image.
// The chain-rule kernel does both adds itself, in 64-bit fixed point (FORCE_FRAC_BITS fractional
// bits, common.cuh): every slot's FP32 vector is rounded once to that grid and the integer sums
// are exact, so F does not depend on the order in which the warps' adds land and no transposed
// index of the lists is needed.  Here the sums become FP64.
#include "common.cuh"
#include "kernels.h"

namespace nnpgpu {

__global__ void __launch_bounds__(256) force_fixed_kernel(int n3, const long long* __restrict__ facc, double* __restrict__ force) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) force[k] = ldexp((double)facc[k], -FORCE_FRAC_BITS);
}

// One CTA per structure: E = sum_i NN_i (+ vacuum energy of each atom's species), FP64.
__global__ void __launch_bounds__(256) energy_kernel(int s0, int ntypes, const StrucMeta* __restrict__ meta, const int* __restrict__ type,
                                                     const float* __restrict__ eatom, const __grid_constant__ NetsP N,
                                                     int add_vacuum, double* __restrict__ energy) {
  __shared__ double red[8];
  const StrucMeta& S = meta[s0 + blockIdx.x];
  double e = 0;
  for (int a = threadIdx.x; a < S.natoms; a += blockDim.x) {
    const int i = S.atom0 + a;
    e += (double)eatom[i];
    if (add_vacuum) e += N.net[clamp_type(type[i], ntypes)].evac;
  }
  e = warp_sum_d(e);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    energy[s0 + blockIdx.x] = t;
  }
}

void launch_gather(const BatchDev& B, const NetsP& N, bool add_vacuum, bool want_force, cudaStream_t st) {
  if (B.natoms == 0) return;
  if (want_force) {
    const int n3 = 3 * B.natoms;
    force_fixed_kernel<<<(n3 + 255) / 256, 256, 0, st>>>(n3, B.facc + 3 * (size_t)B.a0, B.force + 3 * (size_t)B.a0);
  }
  energy_kernel<<<B.nstruc, 256, 0, st>>>(B.s0, B.ntypes, B.meta, B.type, B.eatom, N, add_vacuum ? 1 : 0, B.energy);
}

}  // namespace nnpgpu
