// network_tc.cu - atomic networks as BF16 tensor-core GEMMs (tcgen05, TMEM accumulators, FP32
// accumulation): forward pass and back-propagation to dE/dG for tiles of 128 atoms of one
// species (ANN::fpbp + DODZ::grad, src/ml/nn.cpp:1215-1233,1620-1628).
//
// Per tile (one CTA, 4 warps; thread t owns atom row t = TMEM lane t):
//   X  = bf16(inpw .* (G + inpb))                      -> smem (A operand)
//   Z_l = A_{l-1} W_l^T                                 (tcgen05.mma, D in TMEM)
//   A_l = tanh(Z_l + b_l): bf16 -> smem; A_l' = 1 - A_l^2 parked in TMEM (tcgen05.st)
//   out = outb + outw (b_L + w_L . A_{L-1})             (CUDA cores, FP32)
//   g_{L-1} = outw w_L .* A_{L-1}'; g_{l-1} = (g_l W_l) .* A_{l-1}'   (tcgen05.mma with W_l^T)
//   dE/dG = (g_0 W_0) .* inpw                           (tcgen05.mma with W_0^T), FP32 out
// Every operand is split into two BF16 values, x = hi + lo with hi = bf16(x), lo = bf16(x - hi),
// and each product is formed as A_hi B_hi + A_lo B_hi + A_hi B_lo: three tcgen05.mma into one
// FP32 TMEM accumulator, which keeps the networks within FP32-level error of the FP64 reference
// (plain BF16 operands give force errors of a few 1e-3 eV/A on the mixed workload).
// Operands use the no-swizzle K-major canonical layout: 8x8 bf16 core matrices of 128 bytes,
// consecutive along K (leading byte offset 128), 8-row groups SBO = K*16 bytes apart.  The
// weights of each species are packed once on the host in that layout, one hi/lo block per GEMM;
// each GEMM's block is brought into shared memory by a 1-D TMA bulk copy (cp.async.bulk) into
// one buffer, requested as soon as the previous GEMM's MMAs have completed, so that it loads while
// that GEMM's epilogue runs.  One buffer (not two) keeps a CTA at 48 KB of shared memory on
// 64-wide networks, so that four CTAs share an SM, as many as their TMEM columns allow.
//
// Every mbarrier wait is bounded (wait_limit polls, a kernel argument); on timeout the kernel
// records ERR_TIMEOUT and stops issuing work.  Before it frees its TMEM and leaves, thread 0 waits
// for every weight copy and MMA commit it issued and has not seen complete, bounded by
// TC_DRAIN_LIMIT; if such a drain wait also runs out it records ERR_DRAIN.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "context.h"

namespace nnpgpu {

constexpr int TC_M = 128;        // atoms per tile (MMA M)
constexpr int TC_HMAX = 128;     // widest layer / padded input supported
constexpr int TC_LMAX = 4;       // layers (hidden + output)

constexpr int TC_GMAX = 2 * (TC_LMAX - 1);  // GEMMs per tile
constexpr int TC_DRAIN_LIMIT = 1 << 22;     // polls of a drain wait (about half a second)
// Per-species packed weights: GEMM g's B operand block [hi | lo] at blob offset off[g] with
// bytes[g] bytes; g = 0..L-2 are the forward W_l (N=H_l, K=K_l), g = L-1.. the backward W_l^T
// (N=K_l, K=H_l) for l = L-2 down to 0.
struct TcNetP {
  const uint8_t* blob;
  int nlayer;        // hidden + output
  int nin, k0p;      // inputs, padded to a multiple of 16
  int dims[TC_LMAX + 1];  // k0p, H_0, ..., H_{L-2}, 1
  int off[TC_GMAX];
  int bytes[TC_GMAX];
  int maxblock;      // largest GEMM block
  const float* b[TC_LMAX];
  const float* wout;     // last layer weights [H_{L-2}]
  float bout, outw, outb;
  const float* inpw;
  const float* inpb;
  int act;
};
struct TcNetsP {
  TcNetP net[NT_MAX];
};

// byte offset of element (r, k) of a [rows x K] bf16 operand in the canonical layout
__host__ __device__ __forceinline__ uint32_t core_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, int K) {
  const uint64_t lbo = 128, sbo = (uint64_t)K * 16;
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= ((lbo >> 4) & 0x3FFF) << 16;
  d |= ((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; base offset 0, no swizzle
  return d;
}
// instruction descriptor, kind::f16: D F32, A/B BF16, both K-major, N>>3 at bit 17, M>>4 at bit 24
__device__ __forceinline__ uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait of at most limit polls: false on timeout (at once for limit 0)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit) {
  for (int it = 0; it < limit; ++it) {
    if (mbar_try(bar, parity)) return true;
    if (it > 64) __nanosleep(128);
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 32 consecutive TMEM columns of this thread's lane -> registers
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,"
      "%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
        "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float* v) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,"
      "%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};\n" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
      "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])),
      "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])), "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])),
      "r"(__float_as_uint(v[20])), "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
      "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])), "r"(__float_as_uint(v[27])),
      "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])), "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
// write 8*ng values of row r, columns [c0, c0+8*ng), into the hi and lo [128 x K] operands
__device__ __forceinline__ void store_row_split(uint8_t* hi, uint8_t* lo, int r, int c0, int K, const float* v, int ng) {
  for (int g = 0; g < ng; ++g) {
    float h[8], l[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      h[q] = bf16_round(v[8 * g + q]);
      l[q] = v[8 * g + q] - h[q];
    }
    uint4 wh, wl;
    wh.x = pack_bf16(h[0], h[1]); wh.y = pack_bf16(h[2], h[3]); wh.z = pack_bf16(h[4], h[5]); wh.w = pack_bf16(h[6], h[7]);
    wl.x = pack_bf16(l[0], l[1]); wl.y = pack_bf16(l[2], l[3]); wl.z = pack_bf16(l[4], l[5]); wl.w = pack_bf16(l[6], l[7]);
    *reinterpret_cast<uint4*>(hi + core_off(r, c0 + 8 * g, K)) = wh;
    *reinterpret_cast<uint4*>(lo + core_off(r, c0 + 8 * g, K)) = wl;
  }
}

__device__ __forceinline__ float act_a(int act, float z) {
  if (act == ACT_TANH) return tanhf(z);
  if (act == ACT_SIGMOID) {
    if (z >= 0.f) return 1.0f / (1.0f + expf(-z));
    const float e = expf(z);
    return e / (1.0f + e);
  }
  return z;
}
__device__ __forceinline__ float act_d(int act, float a) {
  return (act == ACT_TANH) ? 1.0f - a * a : (act == ACT_SIGMOID) ? a * (1.0f - a) : 1.0f;
}

__global__ void __launch_bounds__(128, 4) network_tc_kernel(const __grid_constant__ TcNetsP N, int ntypes, const int* __restrict__ tc,
                                                            const int* __restrict__ perm, const float* __restrict__ G, int gstride,
                                                            float* __restrict__ eatom, float* __restrict__ dEdG, int want_grad,
                                                            uint32_t tmem_cols, int opk, int pcols, int wait_limit,
                                                            int* __restrict__ status) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ uint64_t bar_w, bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_err;
  const int tid = threadIdx.x, warp = tid >> 5;
  // locate (type, tile) of this CTA from the device-side type counts
  int t = -1, start = 0, cnt = 0, rem = blockIdx.x;
  for (int ty = 0; ty < ntypes; ++ty) {
    const int c = tc[ty];
    const int nt = (c + TC_M - 1) / TC_M;
    if (rem < nt) { t = ty; start = tc[NT_MAX + 1 + ty] + rem * TC_M; cnt = min(TC_M, c - rem * TC_M); break; }
    rem -= nt;
  }
  if (t < 0) return;
  const TcNetP& net = N.net[t];
  const int L = net.nlayer;
  const int ngemm = want_grad ? 2 * (L - 1) : (L - 1);
  const int opbytes = TC_M * opk * 2;  // opk: the widest K of any GEMM of the batch's networks
  uint8_t* a_hi = smem_raw;                       // activation operand hi [128 x K]
  uint8_t* a_lo = smem_raw + opbytes;             // activation operand lo
  uint8_t* const wbuf = smem_raw + 2 * opbytes;  // the current GEMM's weight block

  if (tid == 0) {
    mbar_init(&bar_w, 1);
    mbar_init(&bar_mma, 1);
    s_err = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)), "r"(tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const uint32_t t_acc = tmem;                      // accumulator columns [0, pcols)
  const uint32_t t_park = tmem + (uint32_t)pcols;   // parked derivatives, pcols columns per hidden layer

  // thread 0's record of the asynchronous work it issued: a weight copy per buffer and the MMA
  // commit, each with the barrier parity of its completion
  bool w_pending = false, mma_pending = false;
  uint32_t w_par = 0, mma_par = 0;
  // weights of GEMM g -> the weight buffer by one 1-D TMA bulk copy, completion on bar_w
  auto load_w = [&](int g) {
    if (g < ngemm) {
      w_pending = true;
      uint64_t* bar = &bar_w;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(net.bytes[g]) : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(wbuf)),
                   "l"(net.blob + net.off[g]), "r"(net.bytes[g]), "r"(smem_u32(bar))
                   : "memory");
    }
  };
  if (tid == 0) load_w(0);
  // scaled inputs of this thread's atom -> split bf16 operand (zero rows past the tile end)
  {
    const int r = tid;
    // the row in 16-byte loads: rows are gstride floats (a multiple of 16) apart and the padded
    // width k0p <= gstride, so whole float4 of the row are read
    const float4* g4 = (r < cnt) ? reinterpret_cast<const float4*>(G + (size_t)perm[start + r] * gstride) : nullptr;
    for (int c0 = 0; c0 < net.k0p; c0 += 32) {
      float v[32];
#pragma unroll
      for (int k4 = 0; k4 < 8; ++k4) {
        const int c = c0 + 4 * k4;
        const float4 x = (g4 && c < net.k0p) ? g4[c >> 2] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) v[4 * k4 + q] = (c + q < net.nin) ? net.inpw[c + q] * (xs[q] + net.inpb[c + q]) : 0.f;
      }
      store_row_split(a_hi, a_lo, r, c0, net.k0p, v, min(4, (net.k0p - c0) / 8));
    }
  }
  fence_async_smem();
  __syncthreads();

  // GEMM g: D[128 x n] = A[128 x k] * B[n x k]^T with split operands; all threads return after
  // the MMAs completed (or a timeout was recorded); then the next-but-one weights are requested.
  auto gemm = [&](int g, int n, int k) {
    if (s_err == 0 && tid == 0) {
      if (mbar_wait(&bar_w, w_par, wait_limit)) {
        w_pending = false;
        w_par ^= 1u;
      } else {
        s_err = 1;
      }
      tc_fence_after();
      if (s_err == 0) {
        const uint32_t idesc = umma_idesc(TC_M, n);
        const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo);
        const uint32_t bh = smem_u32(wbuf), bl = bh + (uint32_t)(n * k * 2);
        for (int kk = 0; kk < k; kk += 16) {
          // advance by two core matrices (16 k) = 256 bytes along K
          const uint32_t o = (uint32_t)(kk * 16);
          tc_mma(t_acc, umma_desc(ah + o, k), umma_desc(bh + o, k), idesc, kk > 0 ? 1u : 0u);
          tc_mma(t_acc, umma_desc(al + o, k), umma_desc(bh + o, k), idesc, 1u);
          tc_mma(t_acc, umma_desc(ah + o, k), umma_desc(bl + o, k), idesc, 1u);
        }
        tc_commit(&bar_mma);
        mma_pending = true;
        if (mbar_wait(&bar_mma, mma_par, wait_limit)) {
          mma_pending = false;
          mma_par ^= 1u;
        } else {
          s_err = 1;
        }
      }
      if (s_err == 0) load_w(g + 1);  // the buffer is free again
    }
    __syncthreads();
    tc_fence_after();
  };

  const int r = tid;
  const bool live = r < cnt;
  float out_acc = 0.f;
  int g = 0;
  // ---- forward through hidden layers
  for (int l = 0; l < L - 1; ++l, ++g) {
    const int k = net.dims[l], n = net.dims[l + 1];
    gemm(g, n, k);
    if (s_err) break;
    for (int c0 = 0; c0 < n; c0 += 32) {
      float v[32];
      tmem_ld32(t_acc + lane_base + c0, v);
      float d[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const float a = act_a(net.act, v[q] + net.b[l][c0 + q]);
        v[q] = a;
        d[q] = act_d(net.act, a);
      }
      if (l < L - 2) {
        tmem_st32(t_park + (uint32_t)(l * pcols) + lane_base + c0, d);
        store_row_split(a_hi, a_lo, r, c0, n, v, 4);  // next layer's A operand
      } else {
        // last hidden layer: output node and the first back-propagated gradient
        float gr[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
          out_acc = fmaf(net.wout[c0 + q], v[q], out_acc);
          gr[q] = net.outw * net.wout[c0 + q] * d[q];
        }
        store_row_split(a_hi, a_lo, r, c0, n, gr, 4);
      }
    }
    tc_fence_before();
    fence_async_smem();
    __syncthreads();
  }
  if (!s_err && live) eatom[perm[start + r]] = net.outb + net.outw * (net.bout + out_acc);
  // ---- back-propagation: g_{l-1} = (g_l W_l) .* A'_{l-1}, then dE/dG = (g_0 W_0) .* inpw
  if (want_grad && !s_err) {
    for (int l = L - 2; l >= 0; --l, ++g) {
      const int n = net.dims[l], k = net.dims[l + 1];  // output width of the transposed product
      gemm(g, n, k);
      if (s_err) break;
      for (int c0 = 0; c0 < n; c0 += 32) {
        float v[32];
        tmem_ld32(t_acc + lane_base + c0, v);
        if (l > 0) {
          float d[32];
          tmem_ld32(t_park + (uint32_t)((l - 1) * pcols) + lane_base + c0, d);
#pragma unroll
          for (int q = 0; q < 32; ++q) v[q] *= d[q];
          store_row_split(a_hi, a_lo, r, c0, n, v, 4);
        } else if (live) {
          // 16-byte stores; columns from nin up to the padded width k0p (<= gstride) get zeros
          float4* o4 = reinterpret_cast<float4*>(dEdG + (size_t)perm[start + r] * gstride);
#pragma unroll
          for (int k4 = 0; k4 < 8; ++k4) {
            const int c = c0 + 4 * k4;
            if (c < net.k0p) {
              float4 w;
              w.x = (c < net.nin) ? v[4 * k4] * net.inpw[c] : 0.f;
              w.y = (c + 1 < net.nin) ? v[4 * k4 + 1] * net.inpw[c + 1] : 0.f;
              w.z = (c + 2 < net.nin) ? v[4 * k4 + 2] * net.inpw[c + 2] : 0.f;
              w.w = (c + 3 < net.nin) ? v[4 * k4 + 3] * net.inpw[c + 3] : 0.f;
              o4[c >> 2] = w;
            }
          }
        }
      }
      tc_fence_before();
      fence_async_smem();
      __syncthreads();
    }
  }
  // every copy and MMA this CTA issued lands before its shared memory and TMEM are released
  if (tid == 0) {
    bool drained = true;
    if (w_pending) drained = mbar_wait(&bar_w, w_par, TC_DRAIN_LIMIT) && drained;
    if (mma_pending) drained = mbar_wait(&bar_mma, mma_par, TC_DRAIN_LIMIT) && drained;
    if (s_err) atomicOr(&status[ST_ERROR], ERR_TIMEOUT);
    if (!drained) atomicOr(&status[ST_ERROR], ERR_DRAIN);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols));
  }
}
#endif  // __CUDACC__

// ------------------------------------------------------------------------------------ host
// Packs m (row-major [rows][cols]) as a [rows x K] operand (zero padded) in hi and lo parts.
static void pack_split(std::vector<uint8_t>& blob, int off, const std::vector<double>& m, int rows, int cols, int K) {
  const int lo_off = off + rows * K * 2;
  for (int r = 0; r < rows; ++r)
    for (int k = 0; k < K; ++k) {
      const float v = k < cols ? (float)m[(size_t)r * cols + k] : 0.f;
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
      std::memcpy(&blob[off + core_off(r, k, K)], &h, 2);
      std::memcpy(&blob[lo_off + core_off(r, k, K)], &l, 2);
    }
}

int prepare_tc_weights(nnpgpu_ctx* c) {
  c->tcbuf = nullptr;
  const HPot& pot = c->pot;
  std::vector<std::vector<uint8_t>> blobs(pot.ntypes);
  TcNetsP host{};
  size_t total = 0;
  for (int t = 0; t < pot.ntypes; ++t) {
    const HNet& n = pot.nets[t];
    const int L = (int)n.nodes.size();
    if (L < 2 || L > TC_LMAX) return -1;
    TcNetP& p = host.net[t];
    p.nlayer = L;
    p.nin = n.nin;
    p.k0p = (n.nin + 15) / 16 * 16;
    if (p.k0p > TC_HMAX) return -1;
    p.dims[0] = p.k0p;
    for (int l = 0; l < L - 1; ++l) {
      if (n.nodes[l] % 32 != 0 || n.nodes[l] > TC_HMAX) return -1;  // epilogue works in 32-column chunks
      p.dims[l + 1] = n.nodes[l];
    }
    // GEMM blocks: forward W_l [H_l x K_l], then backward W_l^T [K_l x H_l] for l = L-2 .. 0
    std::vector<uint8_t>& blob = blobs[t];
    int off = 0, g = 0;
    p.maxblock = 0;
    auto add = [&](int rows, int K) {
      p.off[g] = off;
      p.bytes[g] = 2 * rows * K * 2;
      p.maxblock = std::max(p.maxblock, p.bytes[g]);
      off += p.bytes[g];
      ++g;
    };
    for (int l = 0; l < L - 1; ++l) add(p.dims[l + 1], p.dims[l]);
    for (int l = L - 2; l >= 0; --l) add(p.dims[l], p.dims[l + 1]);
    blob.assign(off, 0);
    g = 0;
    for (int l = 0; l < L - 1; ++l, ++g) {
      const int cols = (l == 0) ? n.nin : p.dims[l];
      pack_split(blob, p.off[g], n.w[l], p.dims[l + 1], cols, p.dims[l]);
    }
    for (int l = L - 2; l >= 0; --l, ++g) {
      const int cols = (l == 0) ? n.nin : p.dims[l];
      const int h = p.dims[l + 1];
      std::vector<double> wt((size_t)cols * h);  // [cols][h]
      for (int rr = 0; rr < h; ++rr)
        for (int q = 0; q < cols; ++q) wt[(size_t)q * h + rr] = n.w[l][(size_t)rr * cols + q];
      // rows beyond cols (input padding) stay zero
      std::vector<double> wtp((size_t)p.dims[l] * h, 0.0);
      std::copy(wt.begin(), wt.end(), wtp.begin());
      pack_split(blob, p.off[g], wtp, p.dims[l], h, h);
    }
    total += (size_t)off;
    // shared memory: two activation operands + two weight buffers
    if (2 * TC_M * TC_HMAX * 2 + 2 * ((p.maxblock + 1023) & ~1023) > 225 * 1024) return -1;
  }
  void* d = nullptr;
  if (cudaMalloc(&d, total + 64) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  size_t o = 0;
  for (int t = 0; t < pot.ntypes; ++t) {
    cudaMemcpy((uint8_t*)d + o, blobs[t].data(), blobs[t].size(), cudaMemcpyHostToDevice);
    host.net[t].blob = (const uint8_t*)d + o;
    o += blobs[t].size();
    const NetP& f = c->nets.net[t];
    for (int l = 0; l < host.net[t].nlayer - 1; ++l) host.net[t].b[l] = f.b[l];
    host.net[t].wout = f.w[host.net[t].nlayer - 1];
    host.net[t].bout = (float)pot.nets[t].b.back()[0];
    host.net[t].outw = f.outw;
    host.net[t].outb = f.outb;
    host.net[t].inpw = f.inpw;
    host.net[t].inpb = f.inpb;
    host.net[t].act = f.act;
  }
  c->tcbuf = d;
  c->tcbytes = total;
  c->used += total;
  static_assert(sizeof(TcNetsP) < 4096, "kernel parameter size");
  c->tcnets = std::make_shared<std::vector<uint8_t>>(sizeof(TcNetsP));
  std::memcpy(c->tcnets->data(), &host, sizeof(TcNetsP));
  return 0;
}

int launch_network_bf16(const BatchDev& B, const NetsP&, const void* tc, int ntypes, cudaStream_t st, const void* tcnets_host,
                        int want_grad, int wait_limit) {
  if (!tc || !tcnets_host) return -1;
  if (B.natoms == 0) return 0;
  const TcNetsP& N = *reinterpret_cast<const TcNetsP*>(tcnets_host);
  // operand K stride and TMEM column block: the widest GEMM input / output of any network
  int kmax = 16, maxl = 2, wblock = 0;
  for (int t = 0; t < ntypes; ++t) {
    const TcNetP& n = N.net[t];
    for (int l = 0; l < n.nlayer; ++l) kmax = std::max(kmax, n.dims[l]);
    maxl = std::max(maxl, n.nlayer);
    wblock = std::max(wblock, (n.maxblock + 1023) & ~1023);
  }
  const int opk = (kmax + 15) / 16 * 16;
  const int pcols = (kmax + 31) / 32 * 32;
  int smem = 2 * TC_M * opk * 2 + wblock;
  // accumulator + one parked derivative block per hidden layer but the last
  const int need = pcols * (1 + (maxl - 2));
  uint32_t cols = 32;
  while ((int)cols < need) cols <<= 1;
  // TMEM has 512 columns per SM and tcgen05.alloc waits while they are taken: the shared-memory
  // request bounds the CTAs per SM (228 KB of shared memory) so that their columns always fit.
  const int fit = 512 / (int)cols;
  smem = std::max(smem, 228 * 1024 / (fit + 1) + 1024);
  static int attr_bytes = 0;
  if (smem > attr_bytes) {
    if (cudaFuncSetAttribute(network_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return -2;
    attr_bytes = smem;
  }
  const int tiles = (B.natoms + TC_M - 1) / TC_M + ntypes;
  network_tc_kernel<<<tiles, 128, smem, st>>>(N, ntypes, B.type_count, B.perm, B.G, B.gstride, B.eatom, B.dEdG, want_grad, cols,
                                             opk, pcols, wait_limit, B.status);
  return 0;
}

}  // namespace nnpgpu
