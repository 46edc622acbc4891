// gather.cu - force assembly and per-structure energy.
//
// NNP::force (src/nnp/nnp.cpp:416-482) adds each neighbour-slot contribution W to the centre
// atom and subtracts it from the neighbour only when the slot is the neighbour's minimum image.
// Here F_j = sum_{s in list(j)} W[j,s] - sum_{s in list(j), min} W[rev(j,s)], where rev is the
// transposed slot built by reverse_kernel: a gather over the atom's own list, no atomics.
// Each lane sums its few slots without rounding loss as an unevaluated pair hi + lo of floats
// (TwoSum, Knuth; the pair carries about 48 bits), the lanes' pairs are added pairwise the same
// way across the warp, and only the final pair becomes FP64: GB300's FP64 pipe (1/64 of the
// FP32 rate) sees a handful of operations per atom instead of a warp-wide FP64 reduction.
#include "common.cuh"
#include "kernels.h"

namespace nnpgpu {

// s + e == a + b exactly (TwoSum; correctly rounded adds, no contraction)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
struct PairSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  // adds another pair: TwoSum of the high parts, the low parts and the rounding error summed
  __device__ __forceinline__ void add_pair(float h, float l) {
    float s, e;
    two_sum(hi, h, s, e);
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, l), e);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
// pairwise across the warp; lane 0 ends with the total pair
__device__ __forceinline__ void warp_pair_sum(PairSum& p) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_down_sync(0xffffffffu, p.hi, o);
    const float l = __shfl_down_sync(0xffffffffu, p.lo, o);
    p.add_pair(h, l);
  }
}

__global__ void __launch_bounds__(128) gather_kernel(int a0, int natoms, int cap, const int* __restrict__ nb_code,
                                                     const int* __restrict__ nb_cnt, const int* __restrict__ nb_rev,
                                                     const float4* __restrict__ W, double* __restrict__ force) {
  const int lane = threadIdx.x & 31;
  const int j = a0 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= a0 + natoms) return;
  const int n = min(nb_cnt[j], cap);
  PairSum sx, sy, sz;
  for (int s = lane; s < n; s += 32) {
    const size_t g = (size_t)j * cap + s;
    const float4 w = W[g];
    sx.add(w.x);
    sy.add(w.y);
    sz.add(w.z);
    if (code_min(nb_code[g])) {
      const int r = nb_rev[g];
      if (r >= 0) {
        const float4 v = W[r];
        sx.add(-v.x);
        sy.add(-v.y);
        sz.add(-v.z);
      }
    }
  }
  warp_pair_sum(sx);
  warp_pair_sum(sy);
  warp_pair_sum(sz);
  // lane k < 3 turns component k's pair into FP64: three FP64 instructions per atom, not nine
  const float hy = __shfl_sync(0xffffffffu, sy.hi, 0), ly = __shfl_sync(0xffffffffu, sy.lo, 0);
  const float hz = __shfl_sync(0xffffffffu, sz.hi, 0), lz = __shfl_sync(0xffffffffu, sz.lo, 0);
  const float hx = __shfl_sync(0xffffffffu, sx.hi, 0), lx = __shfl_sync(0xffffffffu, sx.lo, 0);
  if (lane < 3) {
    const float h = lane == 0 ? hx : (lane == 1 ? hy : hz), l = lane == 0 ? lx : (lane == 1 ? ly : lz);
    force[3 * (size_t)j + lane] = (double)h + (double)l;
  }
}

// Sources whose transposed slot could not be matched: subtract serially (deterministic order).
__global__ void orphan_kernel(int cap, const int* __restrict__ nb_j, const float4* __restrict__ W, const int* __restrict__ orphans,
                              int* __restrict__ status, int orphan_cap, double* __restrict__ force) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int n = min(status[ST_ORPHANS], orphan_cap);
  if (n > 4096) {  // far more than rounding ties can produce: report instead of a long serial pass
    atomicOr(&status[ST_ERROR], ERR_ORPHANS);
    return;
  }
  // insertion order from atomics is arbitrary: apply in increasing slot order
  int last = -1;
  for (int k = 0; k < n; ++k) {
    int best = 0x7fffffff;
    for (int q = 0; q < n; ++q)
      if (orphans[q] > last && orphans[q] < best) best = orphans[q];
    last = best;
    const int j = nb_j[best];
    const float4 v = W[best];
    force[3 * (size_t)j] -= v.x;
    force[3 * (size_t)j + 1] -= v.y;
    force[3 * (size_t)j + 2] -= v.z;
  }
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
    gather_kernel<<<(B.natoms + 3) / 4, 128, 0, st>>>(B.a0, B.natoms, B.cap, B.nb_code, B.nb_cnt, B.nb_rev, B.W, B.force);
    orphan_kernel<<<1, 32, 0, st>>>(B.cap, B.nb_j, B.W, B.orphans, B.status, B.orphan_cap, B.force);
  }
  energy_kernel<<<B.nstruc, 256, 0, st>>>(B.s0, B.ntypes, B.meta, B.type, B.eatom, N, add_vacuum ? 1 : 0, B.energy);
}

}  // namespace nnpgpu
