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

// Species sort without atomics, so the order is the same on every call: atoms of one species
// stay in index order.  type_count_kernel counts per block of 256 atoms (warp ballots), the
// type_offsets_kernel scans the block counts, type_scatter_kernel places each atom
// at its species offset + its block's offset + its rank within the block.  (The scan runs one
// warp per species over contiguous runs of block counts per lane.)
// Layout of tc: [0, NT) counts, [NT_MAX+1, ...) species offsets, [TC_BLK + b*NT_MAX + t) per-block
// counts (then per-block offsets).
constexpr int TC_BLK = 3 * NT_MAX + 3;

__device__ __forceinline__ void block_type_ranks(int t, int ntypes, int* wcnt /* [8][NT_MAX] */, unsigned* mask_out) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int tt = 0; tt < NT_MAX; ++tt) {
    const unsigned m = __ballot_sync(0xffffffffu, t == tt && tt < ntypes);
    if (lane == 0) wcnt[w * NT_MAX + tt] = __popc(m);
    if (t == tt) *mask_out = m;
  }
}

__global__ void __launch_bounds__(256) type_count_kernel(int a0, int natoms, int ntypes, const int* __restrict__ type, int* __restrict__ tc) {
  __shared__ int wcnt[8 * NT_MAX];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = i < natoms ? clamp_type(type[a0 + i], ntypes) : -1;
  unsigned m = 0;
  block_type_ranks(t, ntypes, wcnt, &m);
  __syncthreads();
  if (threadIdx.x < NT_MAX) {
    int c = 0;
    for (int w = 0; w < 8; ++w) c += wcnt[w * NT_MAX + threadIdx.x];
    tc[TC_BLK + blockIdx.x * NT_MAX + threadIdx.x] = c;
  }
}
// one warp per species: each lane owns a contiguous run of block counts (its loads independent of
// one another), the runs' totals are scanned across the warp, and after the species totals are
// known each lane writes its run's offsets with its species' base folded in
__global__ void type_offsets_kernel(int ntypes, int nblocks, int* __restrict__ tc) {
  __shared__ int total[NT_MAX];
  const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
  const int* cnt = tc + TC_BLK;
  int* off = tc + TC_BLK + nblocks * NT_MAX;
  const int per = (nblocks + 31) / 32, b0 = min(lane * per, nblocks), b1 = min(b0 + per, nblocks);
  int seg = 0, incl = 0;
  if (t < ntypes) {
    for (int b = b0; b < b1; ++b) seg += cnt[b * NT_MAX + t];
    incl = seg;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int x = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += x;
    }
  }
  if (t < NT_MAX) {
    const int run = __shfl_sync(0xffffffffu, incl, 31);
    if (lane == 0) total[t] = t < ntypes ? run : 0;
  }
  __syncthreads();
  if (t < ntypes) {
    int acc = incl - seg;
    for (int u = 0; u < t; ++u) acc += total[u];
    for (int b = b0; b < b1; ++b) {
      const int v = cnt[b * NT_MAX + t];
      off[b * NT_MAX + t] = acc;
      acc += v;
    }
  }
  if (threadIdx.x < NT_MAX) {
    int acc = 0;
    for (int u = 0; u < (int)threadIdx.x; ++u) acc += total[u];
    tc[threadIdx.x] = total[threadIdx.x];
    if ((int)threadIdx.x < ntypes) tc[NT_MAX + 1 + threadIdx.x] = acc;
  }
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int u = 0; u < ntypes; ++u) acc += total[u];
    tc[NT_MAX + 1 + ntypes] = acc;
  }
}

__global__ void __launch_bounds__(256) type_scatter_kernel(int a0, int natoms, int ntypes, int nblocks, const int* __restrict__ type,
                                                           const int* __restrict__ tc, int* __restrict__ perm) {
  __shared__ int wcnt[8 * NT_MAX];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int t = i < natoms ? clamp_type(type[a0 + i], ntypes) : -1;
  unsigned m = 0;
  block_type_ranks(t, ntypes, wcnt, &m);
  __syncthreads();
  if (t >= 0) {
    int pos = tc[TC_BLK + nblocks * NT_MAX + blockIdx.x * NT_MAX + t];
    for (int v = 0; v < w; ++v) pos += wcnt[v * NT_MAX + t];
    perm[pos + __popc(m & ((1u << lane) - 1u))] = a0 + i;
  }
}

// Stored descriptors (FP64 rows of sstride values) into the FP32 input rows of the networks:
// atom i keeps its type's nin values, the rest of the row is zero.  Species outside the
// potential are flagged in the status word.
struct NinP {
  int nin[NT_MAX];
};
__global__ void symm_load_kernel(int natoms, int ntypes, const NinP n, const int* __restrict__ type, const double* __restrict__ src,
                                 int sstride, float* __restrict__ G, int gstride, int* __restrict__ status) {
  const size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= (size_t)natoms * gstride) return;
  const int i = (int)(w / gstride), k = (int)(w % gstride);
  const int t = type[i];
  if (t < 0 || t >= ntypes) {
    if (k == 0) atomicOr(&status[ST_ERROR], ERR_BAD_TYPE);
    G[w] = 0.f;
    return;
  }
  G[w] = k < n.nin[t] ? (float)src[(size_t)i * sstride + k] : 0.f;
}

void launch_symm_load(const BatchDev& B, const int* nin, int ntypes, const double* src, int sstride, cudaStream_t st) {
  if (B.natoms == 0) return;
  NinP n{};
  for (int t = 0; t < ntypes && t < NT_MAX; ++t) n.nin[t] = nin[t];
  const size_t total = (size_t)B.natoms * B.gstride;
  symm_load_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(B.natoms, ntypes, n, B.type + B.a0, src, sstride, B.G + (size_t)B.a0 * B.gstride,
                                                                     B.gstride, B.status);
}

size_t type_sort_ints(int natoms) { return TC_BLK + 2 * (size_t)((natoms + 255) / 256) * NT_MAX; }

void launch_type_sort(const BatchDev& B, int ntypes, cudaStream_t st) {
  if (B.natoms == 0) return;
  const int nblocks = (B.natoms + 255) / 256;
  type_count_kernel<<<nblocks, 256, 0, st>>>(B.a0, B.natoms, ntypes, B.type, B.type_count);
  type_offsets_kernel<<<1, 32 * NT_MAX, 0, st>>>(ntypes, nblocks, B.type_count);
  type_scatter_kernel<<<nblocks, 256, 0, st>>>(B.a0, B.natoms, ntypes, nblocks, B.type, B.type_count, B.perm);
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

// ------------------------------------------------------------------------------- training
// The energy trainer's per-batch error and parameter gradient (NNPTE::error,
// src/nnp/nnpte.cpp:870-921, with Cost::grad, src/ml/nn.cpp:1554-1589).  Descriptors and
// atomic energies come from the regular batched pass; then
//   train_loss_kernel   per structure dE = (E - E_ref)/N, the loss, dc/dout = dloss/d(dE) / N;
//   train_grad_kernel   per tile of TILE atoms of one species: forward pass, back-propagation of
//                       dc/dout, and the tile's parameter gradient (biases, then weights with the
//                       input index outer) into its own row of `partial`;
//   train_reduce_kernel the rows of each species summed in tile order in FP64.
// No atomics: the result does not depend on scheduling.
namespace nnpgpu {

__global__ void __launch_bounds__(256) train_loss_kernel(int nstruc, int s0, const StrucMeta* __restrict__ meta,
                                                         const double* __restrict__ energy, const double* __restrict__ eref, int loss,
                                                         double delta, double* __restrict__ dcdo, double* __restrict__ err) {
  __shared__ double r0[256], r1[256];
  double l0 = 0.0, l1 = 0.0;
  for (int s = threadIdx.x; s < nstruc; s += blockDim.x) {
    const int n = meta[s0 + s].natoms;
    const double norm = n > 0 ? 1.0 / n : 0.0;
    const double dE = (energy[s] - eref[s]) * norm;
    double g = norm;
    if (loss == 0) {
      l0 += 0.5 * dE * dE;
      g *= dE;
    } else if (loss == 1) {
      l0 += fabs(dE);
      g *= (dE > 0.0) ? 1.0 : ((dE < 0.0) ? -1.0 : 0.0);
    } else if (loss == 2) {
      const double arg = dE / delta, sq = sqrt(1.0 + arg * arg);
      l0 += delta * delta * (sq - 1.0);
      g *= dE / sq;
    } else {
      const double arg = dE / delta, sq = sqrt(1.0 + arg * arg), lg = log(arg + sq);
      l0 += delta * delta * (1.0 - sq + arg * lg);
      g *= lg * delta;
    }
    l1 += dE * dE;
    dcdo[s] = g;
  }
  r0[threadIdx.x] = l0;
  r1[threadIdx.x] = l1;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      r0[threadIdx.x] += r0[threadIdx.x + o];
      r1[threadIdx.x] += r1[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    err[0] = r0[0];
    err[1] = r1[0];
  }
}

// parameters of one network (ANN::size, src/ml/nn.cpp:899-905)
__host__ __device__ inline int net_params(const NetP& n) {
  int s = 0;
  for (int l = 0; l < n.nlayer; ++l) s += n.nodes[l] * (1 + (l == 0 ? n.nin : n.nodes[l - 1]));
  return s;
}

template <int TILE>
__global__ void __launch_bounds__(128) train_grad_kernel(const __grid_constant__ NetsP N, int ntypes, const int* __restrict__ tc,
                                                         const int* __restrict__ perm, const float* __restrict__ G, int gstride,
                                                         const int* __restrict__ atom_struc, int s0, const double* __restrict__ dcdo,
                                                         float* __restrict__ partial, int pstride) {
  extern __shared__ float sm[];
  int t = -1, start = 0, cnt = 0, rem = blockIdx.x;
  for (int ty = 0; ty < ntypes; ++ty) {
    const int c = tc[ty];
    const int nt = (c + TILE - 1) / TILE;
    if (rem < nt) { t = ty; start = tc[NT_MAX + 1 + ty] + rem * TILE; cnt = min(TILE, c - rem * TILE); break; }
    rem -= nt;
  }
  if (t < 0) return;
  const NetP& net = N.net[t];
  const int L = net.nlayer, K0 = net.nin;
  // smem: X0 = scaled inputs [K0][TILE], A[l] activations of hidden layer l, D[l] dc/dz of layer l
  float* X0 = sm;
  float* A[NLAYER_MAX];
  float* D[NLAYER_MAX];
  float* p = X0 + K0 * TILE;
  for (int l = 0; l < L - 1; ++l) { A[l] = p; p += net.nodes[l] * TILE; }
  for (int l = 0; l < L; ++l) { D[l] = p; p += net.nodes[l] * TILE; }
  for (int w = threadIdx.x; w < K0 * TILE; w += blockDim.x) {
    const int k = w / TILE, a = w % TILE;
    X0[w] = a < cnt ? net.inpw[k] * (G[(size_t)perm[start + a] * gstride + k] + net.inpb[k]) : 0.f;
  }
  __syncthreads();
  const float* in = X0;
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
  // output layer (one linear node): dc/dz = dc/dout * outw
  for (int a = threadIdx.x; a < TILE; a += blockDim.x)
    D[L - 1][a] = a < cnt ? (float)dcdo[atom_struc[perm[start + a]] - s0] * net.outw : 0.f;
  __syncthreads();
  // dc/dz_{l-1} = (W_l^T dc/dz_l) .* a'_{l-1}
  for (int l = L - 1; l > 0; --l) {
    tile_gemm<TILE>(D[l], net.nodes[l], net.w[l], net.nodes[l - 1], net.nodes[l - 1], D[l - 1], nullptr);
    __syncthreads();
    for (int w = threadIdx.x; w < net.nodes[l - 1] * TILE; w += blockDim.x) {
      const float a = A[l - 1][w];
      const float d = (net.act == ACT_TANH) ? 1.0f - a * a : (net.act == ACT_SIGMOID) ? a * (1.0f - a) : 1.0f;
      D[l - 1][w] *= d;
    }
    __syncthreads();
  }
  // the tile's gradient: bias(l, n) = sum_a D[l][n][a]; weight(l, n, m) = sum_a D[l][n][a] X_l[m][a]
  float* out = partial + (size_t)blockIdx.x * pstride;
  int nb = 0;
  for (int l = 0; l < L; ++l) nb += net.nodes[l];
  const int np = net_params(net);
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    int l = 0, r = q, n, m = -1;
    if (r < nb) {
      while (r >= net.nodes[l]) { r -= net.nodes[l]; ++l; }
      n = r;
    } else {
      r -= nb;
      while (r >= net.nodes[l] * (l == 0 ? K0 : net.nodes[l - 1])) { r -= net.nodes[l] * (l == 0 ? K0 : net.nodes[l - 1]); ++l; }
      m = r / net.nodes[l];
      n = r % net.nodes[l];
    }
    const float4* d4 = reinterpret_cast<const float4*>(D[l] + n * TILE);
    // rows are TILE floats apart, so neighbouring threads (consecutive n, or consecutive m in
    // the output layer) start at a rotated float4: a quarter-warp then reads 8 distinct bank groups
    static_assert(((TILE / 4) & (TILE / 4 - 1)) == 0, "the rotation wraps with a mask");
    const int rot = n + (m > 0 ? m : 0);
    float s = 0.f;
    if (m < 0) {
#pragma unroll 4
      for (int v = 0; v < TILE / 4; ++v) {
        const float4 x = d4[(v + rot) & (TILE / 4 - 1)];
        s += (x.x + x.y) + (x.z + x.w);
      }
    } else {
      const float4* x4 = reinterpret_cast<const float4*>((l == 0 ? X0 : A[l - 1]) + m * TILE);
#pragma unroll 4
      for (int v = 0; v < TILE / 4; ++v) {
        const int u = (v + rot) & (TILE / 4 - 1);
        const float4 x = d4[u], y = x4[u];
        s = fmaf(x.x, y.x, fmaf(x.y, y.y, fmaf(x.z, y.z, fmaf(x.w, y.w, s))));
      }
    }
    out[q] = s;
  }
}

// grad[goff[t] + q] (+)= sum over the tiles of species t, in tile order, of partial[tile][q]
__global__ void train_reduce_kernel(const __grid_constant__ NetsP N, int ntypes, int tile, const int* __restrict__ tc,
                                    const float* __restrict__ partial, int pstride, double* __restrict__ grad, int accumulate) {
  int t = blockIdx.y, first = 0, goff = 0;
  if (t >= ntypes) return;
  for (int ty = 0; ty < t; ++ty) {
    first += (tc[ty] + tile - 1) / tile;
    goff += net_params(N.net[ty]);
  }
  const int ntiles = (tc[t] + tile - 1) / tile;
  const int np = net_params(N.net[t]);
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np) return;
  // 16 rows are loaded before they are added (in tile order): the loads overlap, the sum does not
  // change
  constexpr int R = 16;
  const float* col = partial + (size_t)first * pstride + q;
  double s = 0.0;
  int k = 0;
  for (; k + R <= ntiles; k += R) {
    float v[R];
#pragma unroll
    for (int u = 0; u < R; ++u) v[u] = col[(size_t)(k + u) * pstride];
#pragma unroll
    for (int u = 0; u < R; ++u) s += (double)v[u];
  }
  for (; k < ntiles; ++k) s += (double)col[(size_t)k * pstride];
  grad[goff + q] = accumulate ? grad[goff + q] + s : s;
}

constexpr int TRAIN_REDUCE_THREADS = 64;

constexpr int TRAIN_TILE = 64;

size_t train_smem_bytes(const NetsP& N, int ntypes) {
  size_t floats = 0;
  for (int t = 0; t < ntypes; ++t) {
    const NetP& n = N.net[t];
    size_t f = (size_t)n.nin * TRAIN_TILE;
    for (int l = 0; l < n.nlayer; ++l) f += (size_t)n.nodes[l] * TRAIN_TILE * (l < n.nlayer - 1 ? 2 : 1);
    floats = floats > f ? floats : f;
  }
  return floats * sizeof(float);
}

int train_tiles(int natoms, int ntypes) { return (natoms + TRAIN_TILE - 1) / TRAIN_TILE + ntypes; }

int launch_train(const BatchDev& B, const NetsP& N, int ntypes, const double* eref, int loss, double delta, double* dcdo, double* err,
                 float* partial, int pstride, double* grad, int max_params, cudaStream_t st) {
  train_loss_kernel<<<1, 256, 0, st>>>(B.nstruc, B.s0, B.meta, B.energy, eref, loss, delta, dcdo, err);
  const size_t smem = train_smem_bytes(N, ntypes);
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(train_grad_kernel<TRAIN_TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  if (smem > 200 * 1024) return -1;
  train_grad_kernel<TRAIN_TILE><<<train_tiles(B.natoms, ntypes), 128, smem, st>>>(N, ntypes, B.type_count, B.perm, B.G, B.gstride,
                                                                                    B.atom_struc, B.s0, dcdo, partial, pstride);
  train_reduce_kernel<<<dim3((max_params + TRAIN_REDUCE_THREADS - 1) / TRAIN_REDUCE_THREADS, ntypes), TRAIN_REDUCE_THREADS, 0, st>>>(
      N, ntypes, TRAIN_TILE, B.type_count, partial, pstride, grad, 0);
  return 0;
}

// ------------------------------------------------------------------------- force training
// Per atom: fdiff = (F - F_ref)/N (nnptef.cpp:1163-1166), t = beta fdiff / N (dloss/dF),
// fatom = |fdiff|^2.
__global__ void train_force_diff_kernel(int a0, int natoms, int s0, const int* __restrict__ atom_struc, const StrucMeta* __restrict__ meta,
                                        const double* __restrict__ force, const double* __restrict__ fref, double beta,
                                        float4* __restrict__ tvec, double* __restrict__ fatom) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= natoms) return;
  const int i = a0 + k;
  const double norm = 1.0 / meta[atom_struc[i]].natoms;
  double f2 = 0.0, t[3];
  for (int x = 0; x < 3; ++x) {
    const double fd = (force[3 * (size_t)i + x] - fref[3 * (size_t)i + x]) * norm;
    f2 += fd * fd;
    t[x] = beta * fd * norm;
  }
  tvec[i] = make_float4((float)t[0], (float)t[1], (float)t[2], 0.f);
  fatom[i] = f2;
}

// one CTA per structure: fstruc[s] = sum of fatom over its atoms (fixed order)
__global__ void __launch_bounds__(256) train_force_struc_kernel(int s0, const StrucMeta* __restrict__ meta, const double* __restrict__ fatom,
                                                                double* __restrict__ fstruc) {
  __shared__ double red[8];
  const StrucMeta& S = meta[s0 + blockIdx.x];
  double v = 0.0;
  for (int a = threadIdx.x; a < S.natoms; a += blockDim.x) v += fatom[S.atom0 + a];
  v = warp_sum_d(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    fstruc[blockIdx.x] = t;
  }
}

// err[0] += 0.5 beta sum_s fstruc, err[2] = sum_s fstruc (tree order fixed)
__global__ void train_force_err_kernel(int nstruc, const double* __restrict__ fstruc, double beta, double* __restrict__ err) {
  __shared__ double r[256];
  double v = 0.0;
  for (int s = threadIdx.x; s < nstruc; s += blockDim.x) v += fstruc[s];
  r[threadIdx.x] = v;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) r[threadIdx.x] += r[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    err[0] += 0.5 * beta * r[0];
    err[2] = r[0];
  }
}

void launch_train_force_loss(const BatchDev& B, const double* fref, double beta, float4* tvec, double* fatom, double* fstruc, double* err,
                             cudaStream_t st) {
  if (B.natoms == 0) return;
  train_force_diff_kernel<<<(B.natoms + 255) / 256, 256, 0, st>>>(B.a0, B.natoms, B.s0, B.atom_struc, B.meta, B.force, fref, beta, tvec, fatom);
  train_force_struc_kernel<<<B.nstruc, 256, 0, st>>>(B.s0, B.meta, fatom, fstruc);
  train_force_err_kernel<<<1, 256, 0, st>>>(B.nstruc, fstruc, beta, err);
}

// activation derivatives from the activation value a: first and second
__device__ __forceinline__ void act_d12(int act, float a, float& d1, float& d2) {
  if (act == ACT_TANH) {
    d1 = 1.0f - a * a;
    d2 = -2.0f * a * d1;
  } else if (act == ACT_SIGMOID) {
    d1 = a * (1.0f - a);
    d2 = d1 * (1.0f - 2.0f * a);
  } else {
    d1 = 1.0f;
    d2 = 0.f;
  }
}

// Parameter gradient of sum_atoms u . d out/d G for one tile of TILE atoms of one species: the
// networks' mixed second derivative (D2ODZDI, src/ml/nn.cpp:1789-1890) contracted with u, by a
// forward tangent inpw .* u through the layers and a reverse pass over the primal and tangent
// chains.  smem per hidden layer l: A (activation), TA (tangent activation), TZ (tangent
// pre-activation), DP and DT (adjoints of the pre-activation and of its tangent); X0/TX0 the
// scaled inputs and their tangents.  The output layer is linear with one node: its tangent
// adjoint is outw and its primal adjoint zero.  The first-layer weight term keeps inpw
// (D2ODZDI::grad, nn.cpp:1854-1862, leaves it out).
template <int TILE>
__global__ void __launch_bounds__(128) train_force_kernel(const __grid_constant__ NetsP N, int ntypes, const int* __restrict__ tc,
                                                          const int* __restrict__ perm, const float* __restrict__ G,
                                                          const float* __restrict__ U, int gstride, float* __restrict__ partial, int pstride) {
  extern __shared__ float sm[];
  int t = -1, start = 0, cnt = 0, rem = blockIdx.x;
  for (int ty = 0; ty < ntypes; ++ty) {
    const int c = tc[ty];
    const int nt = (c + TILE - 1) / TILE;
    if (rem < nt) { t = ty; start = tc[NT_MAX + 1 + ty] + rem * TILE; cnt = min(TILE, c - rem * TILE); break; }
    rem -= nt;
  }
  if (t < 0) return;
  const NetP& net = N.net[t];
  const int L = net.nlayer, K0 = net.nin, H = L - 1;  // H hidden layers
  float* X0 = sm;
  float* TX0 = X0 + K0 * TILE;
  float *A[NLAYER_MAX], *TA[NLAYER_MAX], *TZ[NLAYER_MAX], *DP[NLAYER_MAX], *DT[NLAYER_MAX];
  float* p = TX0 + K0 * TILE;
  for (int l = 0; l < H; ++l) {
    const int sz = net.nodes[l] * TILE;
    A[l] = p; TA[l] = p + sz; TZ[l] = p + 2 * sz; DP[l] = p + 3 * sz; DT[l] = p + 4 * sz;
    p += 5 * sz;
  }
  for (int w = threadIdx.x; w < K0 * TILE; w += blockDim.x) {
    const int k = w / TILE, a = w % TILE;
    const bool on = a < cnt;
    const size_t row = on ? (size_t)perm[start + a] * gstride : 0;
    X0[w] = on ? net.inpw[k] * (G[row + k] + net.inpb[k]) : 0.f;
    TX0[w] = on ? net.inpw[k] * U[row + k] : 0.f;
  }
  __syncthreads();
  // forward: primal and tangent
  const float* in = X0;
  const float* tin = TX0;
  int Kl = K0;
  for (int l = 0; l < H; ++l) {
    tile_gemm<TILE>(in, Kl, net.wt[l], net.nodes[l], net.nodes[l], A[l], net.b[l]);
    tile_gemm<TILE>(tin, Kl, net.wt[l], net.nodes[l], net.nodes[l], TZ[l], nullptr);
    __syncthreads();
    for (int w = threadIdx.x; w < net.nodes[l] * TILE; w += blockDim.x) {
      float a, d;
      act_fd(net.act, A[l][w], a, d);
      A[l][w] = a;
      TA[l][w] = d * TZ[l][w];
    }
    __syncthreads();
    in = A[l];
    tin = TA[l];
    Kl = net.nodes[l];
  }
  // top hidden layer: adjoint of its tangent activation = outw * w_out; of its activation 0
  {
    const int l = H - 1;
    const float* wout = net.w[L - 1];
    for (int w = threadIdx.x; w < net.nodes[l] * TILE; w += blockDim.x) {
      const int c = w / TILE;
      float d1, d2;
      act_d12(net.act, A[l][w], d1, d2);
      const float g = net.outw * wout[c];
      DT[l][w] = d1 * g;
      DP[l][w] = d2 * TZ[l][w] * g;
    }
    __syncthreads();
  }
  for (int l = H - 1; l > 0; --l) {
    tile_gemm<TILE>(DT[l], net.nodes[l], net.w[l], net.nodes[l - 1], net.nodes[l - 1], DT[l - 1], nullptr);
    tile_gemm<TILE>(DP[l], net.nodes[l], net.w[l], net.nodes[l - 1], net.nodes[l - 1], DP[l - 1], nullptr);
    __syncthreads();
    for (int w = threadIdx.x; w < net.nodes[l - 1] * TILE; w += blockDim.x) {
      float d1, d2;
      act_d12(net.act, A[l - 1][w], d1, d2);
      const float st = DT[l - 1][w];
      DT[l - 1][w] = d1 * st;
      DP[l - 1][w] = d1 * DP[l - 1][w] + d2 * TZ[l - 1][w] * st;
    }
    __syncthreads();
  }
  // the tile's gradient: bias(l, n) = sum_a DP[l][n][a]; weight(l, n, m) = sum_a DT[l][n][a] TX_l[m][a] +
  // DP[l][n][a] X_l[m][a]; the output layer: bias 0, weight(m) = outw sum_a TA[H-1][m][a]
  float* out = partial + (size_t)blockIdx.x * pstride;
  int nb = 0;
  for (int l = 0; l < L; ++l) nb += net.nodes[l];
  const int np = net_params(net);
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    int l = 0, r = q, n, m = -1;
    if (r < nb) {
      while (r >= net.nodes[l]) { r -= net.nodes[l]; ++l; }
      n = r;
    } else {
      r -= nb;
      while (r >= net.nodes[l] * (l == 0 ? K0 : net.nodes[l - 1])) { r -= net.nodes[l] * (l == 0 ? K0 : net.nodes[l - 1]); ++l; }
      m = r / net.nodes[l];
      n = r % net.nodes[l];
    }
    // rotated start per thread: conflict-free reads of rows TILE floats apart (as above)
    static_assert(((TILE / 4) & (TILE / 4 - 1)) == 0, "the rotation wraps with a mask");
    const int rot = n + (m > 0 ? m : 0);
    float s = 0.f;
    if (l == L - 1) {
      if (m >= 0) {
        const float4* x4 = reinterpret_cast<const float4*>(TA[H - 1] + m * TILE);
#pragma unroll 4
        for (int v = 0; v < TILE / 4; ++v) {
          const float4 x = x4[(v + rot) & (TILE / 4 - 1)];
          s += (x.x + x.y) + (x.z + x.w);
        }
        s *= net.outw;
      }
    } else if (m < 0) {
      const float4* d4 = reinterpret_cast<const float4*>(DP[l] + n * TILE);
#pragma unroll 4
      for (int v = 0; v < TILE / 4; ++v) {
        const float4 x = d4[(v + rot) & (TILE / 4 - 1)];
        s += (x.x + x.y) + (x.z + x.w);
      }
    } else {
      const float4* dp4 = reinterpret_cast<const float4*>(DP[l] + n * TILE);
      const float4* dt4 = reinterpret_cast<const float4*>(DT[l] + n * TILE);
      const float4* x4 = reinterpret_cast<const float4*>((l == 0 ? X0 : A[l - 1]) + m * TILE);
      const float4* tx4 = reinterpret_cast<const float4*>((l == 0 ? TX0 : TA[l - 1]) + m * TILE);
#pragma unroll 4
      for (int v = 0; v < TILE / 4; ++v) {
        const int u = (v + rot) & (TILE / 4 - 1);
        const float4 a = dp4[u], b = x4[u], c = dt4[u], d = tx4[u];
        s = fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, fmaf(a.w, b.w, s))));
        s = fmaf(c.x, d.x, fmaf(c.y, d.y, fmaf(c.z, d.z, fmaf(c.w, d.w, s))));
      }
    }
    out[q] = s;
  }
}

constexpr int TRAIN_FORCE_TILE = 32;

static size_t train_force_smem_bytes(const NetsP& N, int ntypes) {
  size_t floats = 0;
  for (int t = 0; t < ntypes; ++t) {
    const NetP& n = N.net[t];
    size_t f = (size_t)2 * n.nin * TRAIN_FORCE_TILE;
    for (int l = 0; l < n.nlayer - 1; ++l) f += (size_t)5 * n.nodes[l] * TRAIN_FORCE_TILE;
    floats = floats > f ? floats : f;
  }
  return floats * sizeof(float);
}

int train_force_tiles(int natoms, int ntypes) { return (natoms + TRAIN_FORCE_TILE - 1) / TRAIN_FORCE_TILE + ntypes; }

int launch_train_force(const BatchDev& B, const NetsP& N, int ntypes, const float* U, float* partial, int pstride, double* grad,
                       int max_params, cudaStream_t st) {
  const size_t smem = train_force_smem_bytes(N, ntypes);
  if (smem > 200 * 1024) return -1;
  for (int t = 0; t < ntypes; ++t)
    if (N.net[t].nlayer < 2) return -1;
  static bool attr = false;
  if (!attr)
    attr = cudaFuncSetAttribute(train_force_kernel<TRAIN_FORCE_TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  train_force_kernel<TRAIN_FORCE_TILE><<<train_force_tiles(B.natoms, ntypes), 128, smem, st>>>(N, ntypes, B.type_count, B.perm, B.G, U,
                                                                                              B.gstride, partial, pstride);
  train_reduce_kernel<<<dim3((max_params + TRAIN_REDUCE_THREADS - 1) / TRAIN_REDUCE_THREADS, ntypes), TRAIN_REDUCE_THREADS, 0, st>>>(
      N, ntypes, TRAIN_FORCE_TILE, B.type_count, partial, pstride, grad, 1);
  return 0;
}

}  // namespace nnpgpu
