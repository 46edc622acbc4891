// descriptor.cu - G2/G4 symmetry functions (NNP::symm, src/nnp/nnp.cpp:334-381) and their
// chain rule into per-neighbour force contributions (NNP::force, src/nnp/nnp.cpp:416-482).
//
// One warp per centre atom.  The atom's neighbour slots are staged in shared memory, grouped
// by neighbour type (stable), with per-pair unit vectors, distances and cutoff values.  The
// pair sets of each angular block (J,K) are walked with a circulant schedule: in round d lane
// x pairs owner x with partner (x+d) mod m.  Within a round every partner index is distinct,
// so the partner-side force contribution is a conflict-free shared-memory update, and the
// owner-side one stays in registers; no atomics are used.
//
// Angular functions (GAUSS, basis_angular.cpp:406-446,456-640) are evaluated on a grid of
// (distinct eta) x (lambda) x (zeta = 2^m):  exp(-(r_ij^a + r_ik^a)/eta^a) factorises into
// per-pair terms, ((1+lambda cos)/2)^(2^m) is a chain of squarings, and the force pass needs
// only three scalars per triplet (d/dcos, d/dr_ij, d/dr_ik of sum_f dE/dG_f G_f).
#include "common.cuh"
#include "kernels.h"

namespace nnpgpu {

constexpr int QMAX = 8;  // owner chunks of 32 per block -> at most 256 neighbours

struct WarpSmem {
  float *ux, *uy, *uz, *d, *inv, *fc, *gc, *dpa, *ex, *wx, *wy, *wz, *scratch;
  int *orig, *toff;
};

__host__ __device__ inline size_t warp_smem_floats(int cap, int ne) { return (size_t)(12 + ne) * cap + 64 + 8; }

__device__ inline WarpSmem carve(float* base, int cap, int ne) {
  WarpSmem s;
  s.ux = base; s.uy = base + cap; s.uz = base + 2 * cap; s.d = base + 3 * cap; s.inv = base + 4 * cap;
  s.fc = base + 5 * cap; s.gc = base + 6 * cap; s.dpa = base + 7 * cap; s.ex = base + 8 * cap;
  s.wx = base + (8 + ne) * cap; s.wy = base + (9 + ne) * cap; s.wz = base + (10 + ne) * cap;
  s.orig = reinterpret_cast<int*>(base + (11 + ne) * cap);
  s.scratch = base + (12 + ne) * cap;
  s.toff = reinterpret_cast<int*>(s.scratch + 64);
  return s;
}

__device__ __forceinline__ float powi(float x, int a) {
  float y = 1.f;
  for (int k = 0; k < a; ++k) y *= x;
  return y;
}

// Stage the neighbour slots of atom i in shared memory, grouped by neighbour type.
// Returns the number of staged slots; toff[t]..toff[t+1] is the range of type t.
__device__ int stage_neighbors(const WarpSmem& S, int i, int cap, int ntypes, const int* __restrict__ type,
                               const int* __restrict__ nb_j, const float4* __restrict__ nb_r, const int* __restrict__ nb_cnt) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int n = min(nb_cnt[i], cap);
  int cnt[NT_MAX];
#pragma unroll
  for (int t = 0; t < NT_MAX; ++t) cnt[t] = 0;
  for (int c = 0; c < n; c += 32) {
    const int s = c + lane;
    const int t = (s < n) ? clamp_type(type[nb_j[(size_t)i * cap + s]], ntypes) : -1;
#pragma unroll
    for (int tt = 0; tt < NT_MAX; ++tt) cnt[tt] += __popc(__ballot_sync(0xffffffffu, t == tt));
  }
  int run[NT_MAX];
  int acc = 0;
#pragma unroll
  for (int t = 0; t < NT_MAX; ++t) {
    run[t] = acc;
    if (lane == t) S.toff[t] = acc;
    acc += (t < ntypes) ? cnt[t] : 0;
  }
  if (lane == 0) S.toff[NT_MAX] = acc;
  for (int c = 0; c < n; c += 32) {
    const int s = c + lane;
    const size_t g = (size_t)i * cap + s;
    const int t = (s < n) ? clamp_type(type[nb_j[g]], ntypes) : -1;
    int pos = 0;
#pragma unroll
    for (int tt = 0; tt < NT_MAX; ++tt) {
      const unsigned m = __ballot_sync(0xffffffffu, t == tt);
      if (t == tt) pos = run[tt] + __popc(m & lt);
      run[tt] += __popc(m);
    }
    if (s < n) {
      const float4 r = nb_r[g];
      const float inv = 1.0f / r.w;
      S.ux[pos] = r.x * inv;
      S.uy[pos] = r.y * inv;
      S.uz[pos] = r.z * inv;
      S.d[pos] = r.w;
      S.inv[pos] = inv;
      S.orig[pos] = s;
    }
  }
  __syncwarp();
  return n;
}

// Per-pair factors of angular block A for slots [lo,hi): ex[e] = exp(-ietap_e d^alpha)
// (times the cutoff when with_fc), cutoff value/gradient and alpha d^(alpha-1) fc.
__device__ void block_pair_factors(const WarpSmem& S, const AngP& A, int lo, int hi, int cap, bool with_fc) {
  const int lane = threadIdx.x & 31;
  for (int p = lo + lane; p < hi; p += 32) {
    const float d = S.d[p];
    float f, g;
    cutoff_fg(A.cut, d, A.rc, A.pirc, A.rci, f, g);
    const float da = powi(d, A.alpha);
    for (int e = 0; e < A.ne; ++e) {
      const float x = expf(-A.ietap[e] * da);
      S.ex[e * cap + p] = with_fc ? x * f : x;
    }
    S.fc[p] = f;
    S.gc[p] = g;
    S.dpa[p] = (float)A.alpha * powi(d, A.alpha - 1) * f;
  }
}

// ------------------------------------------------------------------------------------ blocks
// Geometry of the circulant schedule of one angular block.
struct Sched {
  int xb, nown, yb, mod, d0, d1, nJ;
  bool tri;
};
__device__ __forceinline__ Sched make_sched(int J, int K, int j0, int nJ, int k0, int nK) {
  Sched s;
  s.tri = (J == K);
  s.nJ = nJ;
  if (s.tri) { s.xb = j0; s.yb = j0; s.nown = nJ; s.mod = nJ; s.d0 = 1; s.d1 = nJ / 2; }
  else if (nJ <= nK) { s.xb = j0; s.nown = nJ; s.yb = k0; s.mod = nK; s.d0 = 0; s.d1 = nK - 1; }
  else { s.xb = k0; s.nown = nK; s.yb = j0; s.mod = nJ; s.d0 = 0; s.d1 = nJ - 1; }
  if (s.nown == 0 || (s.tri && nJ < 2)) s.d1 = s.d0 - 1;
  return s;
}

// G4 sums of one block on the (eta) x (lambda) x (zeta = 2^m) grid, NE x NL x NZ, written to
// scratch[(e*NL+l)*NZ_MAX+m] (BasisA::symm, basis_angular.cpp:406-421; NNP::symm, nnp.cpp:359-377).
template <int NE, int NZ>
__device__ __forceinline__ void symm_block(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  const int lane = threadIdx.x & 31;
  float acc[NE][NL][NZ];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NZ; ++m) acc[e][l][m] = 0.f;
  const float lam0 = A.lam[0], lam1 = A.lam[1];
  const float* __restrict__ ux = S.ux;
  const float* __restrict__ uy = S.uy;
  const float* __restrict__ uz = S.uz;
  const float* __restrict__ ex = S.ex;
  for (int q = 0; q * 32 < sc.nown; ++q) {
    const int x = q * 32 + lane;
    const int a = sc.xb + min(x, sc.nown - 1);
    const float uax = ux[a], uay = uy[a], uaz = uz[a];
    float exa[NE];
#pragma unroll
    for (int e = 0; e < NE; ++e) exa[e] = ex[e * cap + a];
    // two rounds per iteration: independent dependency chains for latency hiding
    for (int dd = sc.d0; dd <= sc.d1; dd += 2) {
      const int nx1 = (sc.tri && 2 * dd == sc.nJ) ? (sc.nJ >> 1) : sc.nown;
      const int nx2 = (dd + 1 > sc.d1) ? 0 : ((sc.tri && 2 * (dd + 1) == sc.nJ) ? (sc.nJ >> 1) : sc.nown);
      const bool v1 = x < nx1, v2 = x < nx2;
      int y1 = x + dd, y2 = x + dd + 1;
      if (y1 >= sc.mod) y1 -= sc.mod;
      if (y2 >= sc.mod) y2 -= sc.mod;
      const int b1 = sc.yb + (v1 ? y1 : 0), b2 = sc.yb + (v2 ? y2 : 0);
      const float w1 = v1 ? 1.0f : 0.0f, w2 = v2 ? 1.0f : 0.0f;
      const float cs1 = uax * ux[b1] + uay * uy[b1] + uaz * uz[b1];
      const float cs2 = uax * ux[b2] + uay * uy[b2] + uaz * uz[b2];
      float p1[NL][NZ], p2[NL][NZ];
      p1[0][0] = fabsf(0.5f * (1.0f + lam0 * cs1));
      p1[1][0] = fabsf(0.5f * (1.0f + lam1 * cs1));
      p2[0][0] = fabsf(0.5f * (1.0f + lam0 * cs2));
      p2[1][0] = fabsf(0.5f * (1.0f + lam1 * cs2));
#pragma unroll
      for (int l = 0; l < NL; ++l)
#pragma unroll
        for (int m = 1; m < NZ; ++m) {
          p1[l][m] = p1[l][m - 1] * p1[l][m - 1];
          p2[l][m] = p2[l][m - 1] * p2[l][m - 1];
        }
#pragma unroll
      for (int e = 0; e < NE; ++e) {
        const float E1 = w1 * exa[e] * ex[e * cap + b1];
        const float E2 = w2 * exa[e] * ex[e * cap + b2];
#pragma unroll
        for (int l = 0; l < NL; ++l)
#pragma unroll
          for (int m = 0; m < NZ; ++m) acc[e][l][m] = fmaf(p2[l][m], E2, fmaf(p1[l][m], E1, acc[e][l][m]));
      }
    }
  }
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NZ; ++m) {
        const float v = warp_sum(acc[e][l][m]);
        if (lane == 0) S.scratch[(e * NL + l) * NZ_MAX + m] = v;
      }
}

// Chain rule of one block: per triplet phi = dE/dcos and eta0/eta1 = dE/dr_ij, dE/dr_ik
// summed over the block's functions (BasisA::force, basis_angular.cpp:456-507), turned into the
// neighbour-slot vectors of NNP::force (nnp.cpp:466-478).  The owner's vector accumulates in
// registers; the partner's goes to shared memory (distinct partners within a round).
// One triplet of the chain rule for owner a (registers) and partner b: returns the owner-side
// vector in (oa*) and the partner-side vector in (ob*).
template <int NE, int NZ>
__device__ __forceinline__ void chain_triplet(float uax, float uay, float uaz, float fa, float ga, float pa, float ia, const float* exa,
                                              float ubx, float uby, float ubz, float fb, float gb, float pb, float ib, const float* exb,
                                              const float (&sg)[NE][NL][NZ], const float* ie, float lam0, float lam1, float hn, float nn,
                                              float& oa0, float& oa1, float& oa2, float& ob0, float& ob1, float& ob2) {
  const float cs = uax * ubx + uay * uby + uaz * ubz;
  float p[NL][NZ], qd[NL][NZ];
  p[0][0] = fabsf(0.5f * (1.0f + lam0 * cs));
  p[1][0] = fabsf(0.5f * (1.0f + lam1 * cs));
#pragma unroll
  for (int l = 0; l < NL; ++l) {
    qd[l][0] = 1.0f;
#pragma unroll
    for (int m = 1; m < NZ; ++m) {
      qd[l][m] = 2.0f * qd[l][m - 1] * p[l][m - 1];
      p[l][m] = p[l][m - 1] * p[l][m - 1];
    }
  }
  float Q = 0.f, Q2 = 0.f, Pp = 0.f;
#pragma unroll
  for (int e = 0; e < NE; ++e) {
    const float E = exa[e] * exb[e];
    float q0 = 0.f, q1 = 0.f, r0 = 0.f, r1 = 0.f;
#pragma unroll
    for (int m = 0; m < NZ; ++m) {
      q0 = fmaf(sg[e][0][m], p[0][m], q0);
      q1 = fmaf(sg[e][1][m], p[1][m], q1);
      r0 = fmaf(sg[e][0][m], qd[0][m], r0);
      r1 = fmaf(sg[e][1][m], qd[1][m], r1);
    }
    const float qe = q0 + q1;
    const float pe = lam0 * r0 + lam1 * r1;
    Q = fmaf(E, qe, Q);
    Q2 = fmaf(E * ie[e], qe, Q2);
    Pp = fmaf(E, pe, Pp);
  }
  const float phi = hn * fa * fb * Pp;
  const float eta0 = nn * fb * (ga * Q - pa * Q2);
  const float eta1 = nn * fa * (gb * Q - pb * Q2);
  const float Aa = -phi * cs * ia + eta0, Ba = phi * ia;
  const float Ab = -phi * cs * ib + eta1, Bb = phi * ib;
  oa0 = Aa * uax + Ba * ubx;
  oa1 = Aa * uay + Ba * uby;
  oa2 = Aa * uaz + Ba * ubz;
  ob0 = Ab * ubx + Bb * uax;
  ob1 = Ab * uby + Bb * uay;
  ob2 = Ab * ubz + Bb * uaz;
}

// Chain rule of one block: per triplet phi = dE/dcos and eta0/eta1 = dE/dr_ij, dE/dr_ik
// summed over the block's functions (BasisA::force, basis_angular.cpp:456-507), turned into the
// neighbour-slot vectors of NNP::force (nnp.cpp:466-478).  The owner's vector accumulates in
// registers; the partner's goes to shared memory (distinct partners within a round).
template <int NE, int NZ>
__device__ __forceinline__ void force_block(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  const int lane = threadIdx.x & 31;
  float sg[NE][NL][NZ];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NZ; ++m) sg[e][l][m] = S.scratch[(e * NL + l) * NZ_MAX + m];
  float ie[NE];
#pragma unroll
  for (int e = 0; e < NE; ++e) ie[e] = A.ietap[e];
  const float lam0 = A.lam[0], lam1 = A.lam[1];
  const float hn = -0.5f * A.norm, nn = -A.norm;
  const float* __restrict__ ux = S.ux;
  const float* __restrict__ uy = S.uy;
  const float* __restrict__ uz = S.uz;
  const float* __restrict__ ex = S.ex;
  const float* __restrict__ fc = S.fc;
  const float* __restrict__ gc = S.gc;
  const float* __restrict__ dpa = S.dpa;
  const float* __restrict__ inv = S.inv;
  float* __restrict__ wx = S.wx;
  float* __restrict__ wy = S.wy;
  float* __restrict__ wz = S.wz;
  for (int q = 0; q * 32 < sc.nown; ++q) {
    const int x = q * 32 + lane;
    const int a = sc.xb + min(x, sc.nown - 1);
    const float uax = ux[a], uay = uy[a], uaz = uz[a];
    const float fa = fc[a], ga = gc[a], pa = dpa[a], ia = inv[a];
    float exa[NE];
#pragma unroll
    for (int e = 0; e < NE; ++e) exa[e] = ex[e * cap + a];
    float w0 = 0.f, w1 = 0.f, w2 = 0.f;
    for (int dd = sc.d0; dd <= sc.d1; ++dd) {
      const int nx = (sc.tri && 2 * dd == sc.nJ) ? (sc.nJ >> 1) : sc.nown;
      if (x < nx) {
        int y = x + dd;
        if (y >= sc.mod) y -= sc.mod;
        const int b = sc.yb + y;
        float exb[NE];
#pragma unroll
        for (int e = 0; e < NE; ++e) exb[e] = ex[e * cap + b];
        float a0, a1, a2, c0, c1, c2;
        chain_triplet<NE, NZ>(uax, uay, uaz, fa, ga, pa, ia, exa, ux[b], uy[b], uz[b], fc[b], gc[b], dpa[b], inv[b], exb, sg, ie, lam0,
                              lam1, hn, nn, a0, a1, a2, c0, c1, c2);
        w0 += a0; w1 += a1; w2 += a2;
        wx[b] += c0; wy[b] += c1; wz[b] += c2;
      }
      __syncwarp();
    }
    if (x < sc.nown) {
      wx[sc.xb + x] += w0;
      wy[sc.xb + x] += w1;
      wz[sc.xb + x] += w2;
    }
    __syncwarp();
  }
}

// Dispatch on the block's grid size: eta count 1..NEK, zeta chain length rounded up to 3, 5 or 6
// (at most NZK).  Only instances within the kernel's bounds are linked, which keeps the
// kernel's register allocation to what its potential needs.
template <bool FORCE, int NEK, int NZK>
__device__ void run_block(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  const int z = A.nz <= 3 ? 3 : (A.nz <= 5 ? 5 : 6);
  const int key = A.ne * 8 + z;
#define NNP_CASE(NE_, NZ_)                                   \
  case NE_ * 8 + NZ_:                                        \
    if constexpr (NE_ <= NEK && NZ_ <= NZK) {                \
      if (FORCE) force_block<NE_, NZ_>(S, A, sc, cap);       \
      else symm_block<NE_, NZ_>(S, A, sc, cap);              \
    }                                                        \
    break;
  switch (key) {
    NNP_CASE(1, 3) NNP_CASE(1, 5) NNP_CASE(1, 6)
    NNP_CASE(2, 3) NNP_CASE(2, 5) NNP_CASE(2, 6)
    NNP_CASE(3, 3) NNP_CASE(3, 5) NNP_CASE(3, 6)
    NNP_CASE(4, 3) NNP_CASE(4, 5) NNP_CASE(4, 6)
    default: break;
  }
#undef NNP_CASE
}

// ------------------------------------------------------------------------------------ symm
template <int NEK, int NZK>
__global__ void __launch_bounds__(128) symm_kernel(const __grid_constant__ PotParams P, int a0, int natoms, int cap,
                                                   const int* __restrict__ type, const int* __restrict__ nb_j,
                                                   const float4* __restrict__ nb_r, const int* __restrict__ nb_cnt,
                                                   float* __restrict__ G, int gstride) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = a0 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= a0 + natoms) return;
  const WarpSmem S = carve(smem + warp * warp_smem_floats(cap, NEK), cap, NEK);
  const int I = clamp_type(type[i], P.ntypes);
  stage_neighbors(S, i, cap, P.ntypes, type, nb_j, nb_r, nb_cnt);
  float* Gi = G + (size_t)i * gstride;
  for (int k = P.nin[I] + lane; k < gstride; k += 32) Gi[k] = 0.f;

  // ---- radial: G2 of neighbour type J (BasisR::symm, basis_radial.cpp:302-310)
  for (int J = 0; J < P.ntypes; ++J) {
    const RadialP& R = P.rad[I][J];
    float acc[NR_MAX];
#pragma unroll
    for (int f = 0; f < NR_MAX; ++f) acc[f] = 0.f;
    for (int p = S.toff[J] + lane; p < S.toff[J + 1]; p += 32) {
      const float d = S.d[p];
      float fc, gc;
      cutoff_fg(R.cut, d, R.rc, R.pirc, R.rci, fc, gc);
#pragma unroll
      for (int f = 0; f < NR_MAX; ++f)
        if (f < R.n) {
          const float x = d - R.rs[f];
          acc[f] += expf(-R.eta[f] * x * x) * fc;
        }
    }
#pragma unroll
    for (int f = 0; f < NR_MAX; ++f)
      if (f < R.n) {
        const float v = warp_sum(acc[f]);
        if (lane == f) Gi[R.off + f] = v * R.norm;
      }
  }

  // ---- angular blocks (J <= K): G4
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0) continue;
      const int j0 = S.toff[J], nJ = S.toff[J + 1] - j0;
      const int k0 = S.toff[K], nK = S.toff[K + 1] - k0;
      block_pair_factors(S, A, j0, j0 + nJ, cap, true);
      if (K != J) block_pair_factors(S, A, k0, k0 + nK, cap, true);
      __syncwarp();
      run_block<false, NEK, NZK>(S, A, make_sched(J, K, j0, nJ, k0, nK), cap);
      __syncwarp();
      for (int f = lane; f < A.n; f += 32) Gi[A.off + f] = A.norm * S.scratch[A.gidx[f]];
      __syncwarp();
    }
}

// ------------------------------------------------------------------------------------ force
template <int NEK, int NZK>
__global__ void __launch_bounds__(128) force_kernel(const __grid_constant__ PotParams P, int a0, int natoms, int cap,
                                                    const int* __restrict__ type, const int* __restrict__ nb_j,
                                                    const float4* __restrict__ nb_r, const int* __restrict__ nb_cnt,
                                                    const float* __restrict__ dEdG, int gstride, float4* __restrict__ W) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = a0 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= a0 + natoms) return;
  const WarpSmem S = carve(smem + warp * warp_smem_floats(cap, NEK), cap, NEK);
  const int I = clamp_type(type[i], P.ntypes);
  const int n = stage_neighbors(S, i, cap, P.ntypes, type, nb_j, nb_r, nb_cnt);
  const float* gi = dEdG + (size_t)i * gstride;

  // ---- radial chain rule: W_p = BasisR::force(d) * u_p (basis_radial.cpp:371-380, nnp.cpp:441-446)
  for (int J = 0; J < P.ntypes; ++J) {
    const RadialP& R = P.rad[I][J];
    float s[NR_MAX];
#pragma unroll
    for (int f = 0; f < NR_MAX; ++f) s[f] = (f < R.n) ? gi[R.off + f] : 0.f;
    for (int p = S.toff[J] + lane; p < S.toff[J + 1]; p += 32) {
      const float d = S.d[p];
      float fc, gc;
      cutoff_fg(R.cut, d, R.rc, R.pirc, R.rci, fc, gc);
      float amp = 0.f;
#pragma unroll
      for (int f = 0; f < NR_MAX; ++f)
        if (f < R.n) {
          const float x = d - R.rs[f];
          amp -= s[f] * expf(-R.eta[f] * x * x) * (-2.0f * R.eta[f] * x * fc + gc);
        }
      amp *= R.norm;
      S.wx[p] = amp * S.ux[p];
      S.wy[p] = amp * S.uy[p];
      S.wz[p] = amp * S.uz[p];
    }
  }
  __syncwarp();

  // ---- angular chain rule
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0) continue;
      const int j0 = S.toff[J], nJ = S.toff[J + 1] - j0;
      const int k0 = S.toff[K], nK = S.toff[K + 1] - k0;
      if (nJ == 0 || nK == 0 || (J == K && nJ < 2)) continue;
      block_pair_factors(S, A, j0, j0 + nJ, cap, false);
      if (K != J) block_pair_factors(S, A, k0, k0 + nK, cap, false);
      // dE/dG on the function grid (duplicates of a grid cell add up)
      if (lane == 0) {
        for (int c = 0; c < NE_MAX * NL * NZ_MAX; ++c) S.scratch[c] = 0.f;
        for (int f = 0; f < A.n; ++f) S.scratch[A.gidx[f]] += gi[A.off + f];
      }
      __syncwarp();
      run_block<true, NEK, NZK>(S, A, make_sched(J, K, j0, nJ, k0, nK), cap);
      __syncwarp();
    }

  // write the per-slot contributions in the list's own slot order
  float4* Wi = W + (size_t)i * cap;
  for (int p = lane; p < n; p += 32) Wi[S.orig[p]] = make_float4(S.wx[p], S.wy[p], S.wz[p], 0.f);
}

size_t symm_smem_bytes(int cap, int ne, int warps) { return sizeof(float) * warp_smem_floats(cap, ne) * warps; }
size_t force_smem_bytes(int cap, int ne, int warps) { return sizeof(float) * warp_smem_floats(cap, ne) * warps; }

template <int NEK, int NZK>
static void launch_symm_t(const BatchDev& B, const PotParams& P, int warps, cudaStream_t st) {
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(symm_kernel<NEK, NZK>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  symm_kernel<NEK, NZK><<<(B.natoms + warps - 1) / warps, 32 * warps, symm_smem_bytes(B.cap, NEK, warps), st>>>(
      P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_r, B.nb_cnt, B.G, B.gstride);
}
template <int NEK, int NZK>
static void launch_force_t(const BatchDev& B, const PotParams& P, int warps, cudaStream_t st) {
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(force_kernel<NEK, NZK>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  force_kernel<NEK, NZK><<<(B.natoms + warps - 1) / warps, 32 * warps, force_smem_bytes(B.cap, NEK, warps), st>>>(
      P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_r, B.nb_cnt, B.dEdG, B.gstride, B.W);
}

// Kernel instance covering the potential's largest block grid: (ne, nz) within (2,5), (4,5) or (4,6).
int launch_symm(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st) {
  if (B.natoms == 0) return 0;
  if (ne <= 2 && nz <= 5) launch_symm_t<2, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 5) launch_symm_t<4, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 6) launch_symm_t<4, 6>(B, P, warps, st);
  else return -1;
  return 0;
}
int launch_force(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st) {
  if (B.natoms == 0) return 0;
  if (ne <= 2 && nz <= 5) launch_force_t<2, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 5) launch_force_t<4, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 6) launch_force_t<4, 6>(B, P, warps, st);
  else return -1;
  return 0;
}

}  // namespace nnpgpu
