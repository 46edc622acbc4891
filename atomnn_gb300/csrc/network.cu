// network.cu - atomic networks, plain FP32 path: forward pass and back-propagation to dE/dG
// for tiles of atoms of one species (ANN::fpbp + DODZ::grad, src/ml/nn.cpp:1215-1233,1620-1628;
// NNH::energy, src/nnp/nnh.cpp:127-130).
//
// Atoms are grouped by species first (type_sort), so each CTA runs one network over a tile of
// TILE atoms (16, 32 or 64, chosen by the autotuner): every layer is an (atoms x in) x (in x out)
// product with activations staged transposed in shared memory and weights streamed from L2.
#include "common.cuh"
#include "kernels.h"

namespace nnpgpu {

// One atomic per warp and species (ballot + popc) instead of one per atom: a batch has a
// handful of species, so per-atom atomics would all hit the same few counters.
__global__ void type_count_kernel(int a0, int natoms, int ntypes, const int* __restrict__ type, int* __restrict__ tc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int t = i < natoms ? clamp_type(type[a0 + i], ntypes) : -1;
  for (int tt = 0; tt < ntypes; ++tt) {
    const unsigned m = __ballot_sync(0xffffffffu, t == tt);
    if (lane == 0 && m) atomicAdd(&tc[tt], __popc(m));
  }
}
// tc[0..NT) counts -> exclusive offsets in tc[NT_MAX+1 .. 2*NT_MAX+1], cursors in tc[2*NT_MAX+2 ..]
__global__ void type_offsets_kernel(int ntypes, int* __restrict__ tc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int acc = 0;
    for (int t = 0; t < ntypes; ++t) {
      tc[NT_MAX + 1 + t] = acc;
      tc[2 * NT_MAX + 2 + t] = acc;
      acc += tc[t];
    }
    tc[NT_MAX + 1 + ntypes] = acc;
  }
}
__global__ void type_scatter_kernel(int a0, int natoms, int ntypes, const int* __restrict__ type, int* __restrict__ tc, int* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int t = i < natoms ? clamp_type(type[a0 + i], ntypes) : -1;
  for (int tt = 0; tt < ntypes; ++tt) {
    const unsigned m = __ballot_sync(0xffffffffu, t == tt);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(&tc[2 * NT_MAX + 2 + tt], __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (t == tt) perm[base + __popc(m & ((1u << lane) - 1u))] = a0 + i;
  }
}

void launch_type_sort(const BatchDev& B, int ntypes, cudaStream_t st) {
  if (B.natoms == 0) return;
  cudaMemsetAsync(B.type_count, 0, sizeof(int) * (3 * NT_MAX + 3), st);
  type_count_kernel<<<(B.natoms + 255) / 256, 256, 0, st>>>(B.a0, B.natoms, ntypes, B.type, B.type_count);
  type_offsets_kernel<<<1, 32, 0, st>>>(ntypes, B.type_count);
  type_scatter_kernel<<<(B.natoms + 255) / 256, 256, 0, st>>>(B.a0, B.natoms, ntypes, B.type, B.type_count, B.perm);
}

__device__ __forceinline__ void act_fd(int act, float z, float& a, float& d) {
  if (act == ACT_TANH) {
    const float t = tanhf(z);
    a = t;
    d = 1.0f - t * t;
  } else if (act == ACT_SIGMOID) {
    if (z >= 0.f) { const float e = expf(-z), f = 1.0f / (1.0f + e); a = f; d = e * f * f; }
    else { const float e = expf(z), f = 1.0f / (1.0f + e); a = e * f; d = e * f * f; }
  } else {
    a = z;
    d = 1.0f;
  }
}

// out[n][t] = sum_k inT[k][t] * B[k*ldb + n] for t < TILE, n < N; inT is [K][TILE] in smem.
// Each thread owns one output column n and 16 atoms.
template <int TILE>
__device__ __forceinline__ void tile_gemm(const float* __restrict__ inT, int K, const float* __restrict__ Bm, int ldb, int N,
                                          float* __restrict__ outT, const float* __restrict__ bias) {
  for (int w = threadIdx.x; w < N * (TILE / 16); w += blockDim.x) {
    const int n = w % N, h = w / N;
    float acc[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) acc[t] = bias ? bias[n] : 0.f;
    for (int k = 0; k < K; ++k) {
      const float bv = __ldg(Bm + (size_t)k * ldb + n);
      const float4* row = reinterpret_cast<const float4*>(inT + k * TILE + h * 16);
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const float4 x = row[v];
        acc[4 * v + 0] = fmaf(x.x, bv, acc[4 * v + 0]);
        acc[4 * v + 1] = fmaf(x.y, bv, acc[4 * v + 1]);
        acc[4 * v + 2] = fmaf(x.z, bv, acc[4 * v + 2]);
        acc[4 * v + 3] = fmaf(x.w, bv, acc[4 * v + 3]);
      }
    }
    float4* o = reinterpret_cast<float4*>(outT + n * TILE + h * 16);
#pragma unroll
    for (int v = 0; v < 4; ++v) o[v] = make_float4(acc[4 * v], acc[4 * v + 1], acc[4 * v + 2], acc[4 * v + 3]);
  }
}

template <int TILE>
__global__ void __launch_bounds__(128) network_fp32_kernel(const __grid_constant__ NetsP N, int ntypes, const int* __restrict__ tc,
                                                           const int* __restrict__ perm, const float* __restrict__ G, int gstride,
                                                           float* __restrict__ eatom, float* __restrict__ dEdG, int want_grad) {
  extern __shared__ float sm[];
  // locate (type, tile) of this CTA
  int t = -1, start = 0, cnt = 0, rem = blockIdx.x;
  for (int ty = 0; ty < ntypes; ++ty) {
    const int c = tc[ty];
    const int nt = (c + TILE - 1) / TILE;
    if (rem < nt) { t = ty; start = tc[NT_MAX + 1 + ty] + rem * TILE; cnt = min(TILE, c - rem * TILE); break; }
    rem -= nt;
  }
  if (t < 0) return;
  const NetP& net = N.net[t];
  const int L = net.nlayer;
  const int K0 = net.nin;
  // smem: XT [K0][TILE], A[l] [nodes[l]][TILE] for hidden layers, two gradient buffers
  float* XT = sm;
  float* A[NLAYER_MAX];
  float* p = XT + K0 * TILE;
  int maxn = K0;
  for (int l = 0; l < L - 1; ++l) { A[l] = p; p += net.nodes[l] * TILE; maxn = max(maxn, net.nodes[l]); }
  float* G0 = p;
  float* G1 = p + maxn * TILE;
  __shared__ float outs[TILE];

  // scaled inputs ins = inpw * (G + inpb) (ANN::fp, nn.cpp:1194)
  for (int w = threadIdx.x; w < K0 * TILE; w += blockDim.x) {
    const int k = w / TILE, a = w % TILE;
    float v = 0.f;
    if (a < cnt) v = net.inpw[k] * (G[(size_t)perm[start + a] * gstride + k] + net.inpb[k]);
    XT[w] = v;
  }
  __syncthreads();
  // hidden layers
  const float* in = XT;
  int Kl = K0;
  for (int l = 0; l < L - 1; ++l) {
    tile_gemm<TILE>(in, Kl, net.wt[l], net.nodes[l], net.nodes[l], A[l], net.b[l]);
    __syncthreads();
    for (int w = threadIdx.x; w < net.nodes[l] * TILE; w += blockDim.x) {
      float a, d;
      act_fd(net.act, A[l][w], a, d);
      A[l][w] = a;
    }
    __syncthreads();
    in = A[l];
    Kl = net.nodes[l];
  }
  // linear output layer (one node): out = outb + outw * (b + w . a)
  const float* wl = net.w[L - 1];
  for (int a = threadIdx.x; a < TILE; a += blockDim.x) {
    float z = net.b[L - 1][0];
    for (int k = 0; k < Kl; ++k) z = fmaf(in[k * TILE + a], wl[k], z);
    outs[a] = net.outb + net.outw * z;
  }
  __syncthreads();
  for (int a = threadIdx.x; a < cnt; a += blockDim.x) eatom[perm[start + a]] = outs[a];
  if (!want_grad) return;
  // back-propagation (DODZ::grad): g_{L-1} = outw * w_L .* a'_{L-1}
  float* gcur = G0;
  float* gnext = G1;
  {
    const int l = L - 2;
    for (int w = threadIdx.x; w < Kl * TILE; w += blockDim.x) {
      const int k = w / TILE;
      const float a = A[l][w];
      const float d = (net.act == ACT_TANH) ? 1.0f - a * a : (net.act == ACT_SIGMOID) ? a * (1.0f - a) : 1.0f;
      gcur[w] = net.outw * wl[k] * d;
    }
    __syncthreads();
  }
  for (int l = L - 2; l >= 1; --l) {
    // gnext[c][t] = sum_r gcur[r][t] W_l[r][c]
    tile_gemm<TILE>(gcur, net.nodes[l], net.w[l], net.nodes[l - 1], net.nodes[l - 1], gnext, nullptr);
    __syncthreads();
    for (int w = threadIdx.x; w < net.nodes[l - 1] * TILE; w += blockDim.x) {
      const float a = A[l - 1][w];
      const float d = (net.act == ACT_TANH) ? 1.0f - a * a : (net.act == ACT_SIGMOID) ? a * (1.0f - a) : 1.0f;
      gnext[w] *= d;
    }
    __syncthreads();
    float* tmp = gcur; gcur = gnext; gnext = tmp;
  }
  // dodi = (g_0 W_0) .* inpw -> dE/dG
  tile_gemm<TILE>(gcur, net.nodes[0], net.w[0], K0, K0, gnext, nullptr);
  __syncthreads();
  for (int w = threadIdx.x; w < K0 * TILE; w += blockDim.x) {
    const int k = w / TILE, a = w % TILE;
    if (a < cnt) dEdG[(size_t)perm[start + a] * gstride + k] = gnext[w] * net.inpw[k];
  }
}

template <int TILE>
static void launch_network_fp32_t(const BatchDev& B, const NetsP& N, int ntypes, cudaStream_t st) {
  size_t floats = 0;
  for (int t = 0; t < ntypes; ++t) {
    const NetP& n = N.net[t];
    size_t f = (size_t)n.nin * TILE;
    int maxn = n.nin;
    for (int l = 0; l < n.nlayer - 1; ++l) { f += (size_t)n.nodes[l] * TILE; maxn = max(maxn, n.nodes[l]); }
    f += 2 * (size_t)maxn * TILE;
    floats = max(floats, f);
  }
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(network_fp32_kernel<TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  const int tiles = (B.natoms + TILE - 1) / TILE + ntypes;
  network_fp32_kernel<TILE><<<tiles, 128, floats * sizeof(float), st>>>(N, ntypes, B.type_count, B.perm, B.G, B.gstride, B.eatom,
                                                                         B.dEdG, 1);
}

void launch_network_fp32(const BatchDev& B, const NetsP& N, int ntypes, int tile, cudaStream_t st) {
  if (B.natoms == 0) return;
  if (tile <= 16) launch_network_fp32_t<16>(B, N, ntypes, st);
  else if (tile <= 32) launch_network_fp32_t<32>(B, N, ntypes, st);
  else launch_network_fp32_t<64>(B, N, ntypes, st);
}

}  // namespace nnpgpu
