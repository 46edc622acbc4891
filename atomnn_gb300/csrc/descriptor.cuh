// descriptor.cuh - G2/G4 symmetry functions (NNP::symm, src/nnp/nnp.cpp:334-381) and their
// chain rule into per-neighbour force contributions (NNP::force, src/nnp/nnp.cpp:416-482).
//
// One warp per centre atom.  The atom's neighbour slots are staged in shared memory, grouped
// by neighbour type (stable), with per-pair unit vectors, distances and cutoff values.  The
// pair sets of each angular block (J,K) are walked with a circulant schedule: in round d lane
// x pairs owner x with partner (x+d) mod m.  Within a round every partner index is distinct,
// so the partner-side force contribution is a conflict-free shared-memory update, and the
// owner-side one stays in registers; no atomics are used.
//
// Exponentials and the cosine cutoff use the hardware approximations (__expf, __sincosf: a few
// ulp, below the FP32 rounding of the sums they enter).
//
// Angular functions (basis_angular.cpp:406-446,456-640) are evaluated on a grid of
// (distinct eta) x (lambda) x (zeta = 2^m):  the GAUSS factor exp(-(r_ij^a + r_ik^a)/eta^a)
// (and the IPOWP and SECHP ones) factorise into per-pair terms, ((1+lambda cos)/2)^(2^m) is a
// chain of squarings, and the force pass needs only three scalars per triplet (d/dcos, d/dr_ij,
// d/dr_ik of sum_f dE/dG_f G_f).  The sum families IPOWS and SECHS evaluate their factor per
// triplet.
//
// Device code only; the kernel instances and their launchers live in descriptor_symm.cu,
// descriptor_force.cu, descriptor_force_gen.cu and descriptor_tangent.cu, which compile in parallel.
#pragma once
#include "common.cuh"
#include "kernels.h"

namespace nnpgpu {

constexpr int QMAX = 8;  // owner chunks of 32 per block -> at most 256 neighbours

struct WarpSmem {
  float *ux, *uy, *uz, *d, *inv, *fc, *gc, *dpa, *ex, *kx, *wx, *wy, *wz, *scratch, *gi;
  int *orig, *toff;
};

// The per-width region ex is at least MOM_EX floats per width so that a moment block's tensors
// fit there: in the descriptor pass two sets of MOM_C per width plus the diagonal terms, in the
// chain rule two contraction tables of MOM_Q float4 per width.  With kx, a second per-width
// region holds the pair factors' derivative weights (IPOWP and SECHP blocks of the force pass).
// ng floats at the end hold the centre's dE/dG row in the force pass (0 elsewhere).  scratch is 96
// floats: the G4 grid sums, or a moment block's coefficients, or those of up to three blocks plus
// the shared tables' degree-0 terms.
__host__ __device__ inline int ex_stride(int cap) { return cap > MOM_EX ? cap : MOM_EX; }
__host__ __device__ inline size_t warp_smem_floats(int cap, int ne, bool kx, int ng = 0) {
  return (size_t)12 * cap + (size_t)ne * ex_stride(cap) + (kx ? (size_t)ne * cap : 0) + 96 + 8 + ng;
}

__device__ inline WarpSmem carve(float* base, int cap, int ne, bool kx) {
  WarpSmem s;
  s.ux = base; s.uy = base + cap; s.uz = base + 2 * cap; s.d = base + 3 * cap; s.inv = base + 4 * cap;
  s.fc = base + 5 * cap; s.gc = base + 6 * cap; s.dpa = base + 7 * cap; s.ex = base + 8 * cap;
  float* w = s.ex + (size_t)ne * ex_stride(cap);
  s.kx = kx ? w : nullptr;
  if (kx) w += (size_t)ne * cap;
  s.wx = w; s.wy = w + cap; s.wz = w + 2 * cap;
  s.orig = reinterpret_cast<int*>(w + 3 * cap);
  s.scratch = w + 4 * cap;
  s.toff = reinterpret_cast<int*>(s.scratch + 96);
  s.gi = s.scratch + 104;
  return s;
}


__device__ __forceinline__ float powi(float x, int a) {
  float y = 1.f;
  for (int k = 0; k < a; ++k) y *= x;
  return y;
}

// ------------------------------------------------------------------------------- moment tensors
// Blocks whose functions all have zeta <= 4 (and |lambda| <= 1) skip the triplet loop.  The
// angular term ((1 + lambda cos)/2)^zeta is a polynomial of degree <= 4 in cos = u_j . u_k, and
//   sum_{j in J, k in K} w_j w_k (u_j . u_k)^n = <M^J_n, M^K_n>,   M^S_n = sum_{j in S} w_j u_j^(x)n,
// with w = h(r^alpha/eta^alpha) f_c(r), h the pair factor of a product family (exp(-x) for
// GAUSS, 1/(1+x) for IPOWP, sech(x) for SECHP; basis_angular.cpp:406-446).
// The symmetric tensors M_n (n = 0..4) have 35 components in all, so a block costs
// O(neighbours x 35) instead of O(neighbours^2); J == K blocks take half the full double sum
// minus its j == k terms (the reference sums j < k, nnp.cpp:359-377).  The chain rule
// differentiates each neighbour's term against the other species' moments, which the
// descriptor pass leaves in global memory for the force pass.
//
// Component order: degree n ascending; within a degree, exponent a of u_x descending, then b of
// u_y descending (c = n - a - b).
__host__ __device__ constexpr int mom_off(int n) { return n * (n + 1) * (n + 2) / 6; }
__host__ __device__ constexpr int mom_idx(int a, int b, int c) {
  return mom_off(a + b + c) + (b + c) * (b + c + 1) / 2 + c;
}
__host__ __device__ constexpr float mom_fact(int n) {
  float v = 1.0f;
  for (int k = 2; k <= n; ++k) v *= (float)k;
  return v;
}
// multinomial n!/(a! b! c!): the number of index tuples of the symmetric tensor per component
__host__ __device__ constexpr float mom_mult(int a, int b, int c) {
  return mom_fact(a + b + c) / (mom_fact(a) * mom_fact(b) * mom_fact(c));
}
__host__ __device__ constexpr int mom_deg(int r) { return r < 1 ? 0 : (r < 4 ? 1 : (r < 10 ? 2 : (r < 20 ? 3 : 4))); }
// mom_mult per component, and for each component q of degree <= 3 the components q + e_x,
// q + e_y, q + e_z (runtime-indexed copies of the constexpr functions above)
static __device__ const float c_mom_mult[MOM_C] = {1, 1, 1, 1, 1, 2, 2, 1, 2, 1, 1, 3, 3, 3, 6, 3, 1, 3,
                                            3, 1, 1, 4, 4, 6, 12, 6, 4, 12, 12, 4, 1, 4, 6, 4, 1};
static __device__ const signed char c_mom_up[MOM_Q][3] = {{1, 2, 3},    {4, 5, 6},    {5, 7, 8},    {6, 8, 9},    {10, 11, 12},
                                                   {11, 13, 14}, {12, 14, 15}, {13, 16, 17}, {14, 17, 18}, {15, 18, 19},
                                                   {20, 21, 22}, {21, 23, 24}, {22, 24, 25}, {23, 26, 27}, {24, 27, 28},
                                                   {25, 28, 29}, {26, 30, 31}, {27, 31, 32}, {28, 32, 33}, {29, 33, 34}};

// Moments of nsets slot ranges (set 0: [lo0,hi0), set 1: [lo1,hi1)) for every width of the block:
// M[(set*ne + e)*MOM_C + r] = sum over the set's slots of w_e u^(a,b,c).  Each (set, width) pair
// is summed by its own group of L lanes (L = 32 / pairs, rounded down to a power of two), so the
// cross-lane reduction takes log2(L) shuffle levels instead of 5.  With Dg, every set also gives
// Dg[(set*ne + e)*(MOM_N+1) + n] = sum w_e^2 |u|^2n (the j == k terms of a J == K block).
// GAUSS instances evaluate exp(-x) directly; the others go through ang_h.
template <bool GAUSS>
__device__ void build_moments(const WarpSmem& S, const AngP& A, bool cc, int nsets, int lo0, int hi0, int lo1, int hi1,
                              float* __restrict__ M, float* __restrict__ Dg) {
  const int lane = threadIdx.x & 31;
  const int pairs = nsets * A.ne;
  int L = 32;
  while (L * pairs > 32) L >>= 1;
  const int grp = lane / L, sub = lane % L;
  const bool active = grp < pairs;
  const int set = active ? grp / A.ne : 0, e = active ? grp % A.ne : 0;
  const int lo = active ? (set ? lo1 : lo0) : 0, hi = active ? (set ? hi1 : hi0) : 0;
  const bool want_dg = Dg != nullptr;
  float acc[MOM_C], dg[MOM_N + 1];
#pragma unroll
  for (int r = 0; r < MOM_C; ++r) acc[r] = 0.f;
#pragma unroll
  for (int n = 0; n <= MOM_N; ++n) dg[n] = 0.f;
  const float ie = A.ietap[e];
  for (int p = lo + sub; p < hi; p += L) {
    const float d = S.d[p], ux = S.ux[p], uy = S.uy[p], uz = S.uz[p];
    float f, g;
    if (cc) f = S.fc[p];
    else cutoff_fg(A.cut, d, A.rc, A.pirc, A.rci, f, g);
    float kap;
    const float w = (GAUSS ? __expf(-ie * powi(d, A.alpha)) : ang_h(A.phi, ie * powi(d, A.alpha), kap)) * f;
    float wx[MOM_N + 1], py[MOM_N + 1], pz[MOM_N + 1];
    wx[0] = w;
    py[0] = 1.f;
    pz[0] = 1.f;
#pragma unroll
    for (int k = 1; k <= MOM_N; ++k) {
      wx[k] = wx[k - 1] * ux;
      py[k] = py[k - 1] * uy;
      pz[k] = pz[k - 1] * uz;
    }
#pragma unroll
    for (int n = 0; n <= MOM_N; ++n)
#pragma unroll
      for (int a = n; a >= 0; --a)
#pragma unroll
        for (int b = n - a; b >= 0; --b) {
          const int c = n - a - b;
          acc[mom_idx(a, b, c)] = fmaf(wx[a], py[b] * pz[c], acc[mom_idx(a, b, c)]);
        }
    if (want_dg) {
      const float u2 = ux * ux + uy * uy + uz * uz;
      float t = w * w;
#pragma unroll
      for (int n = 0; n <= MOM_N; ++n) {
        dg[n] += t;
        t *= u2;
      }
    }
  }
  for (int o = L >> 1; o > 0; o >>= 1) {
#pragma unroll
    for (int r = 0; r < MOM_C; ++r) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
    if (Dg) {
#pragma unroll
      for (int n = 0; n <= MOM_N; ++n) dg[n] += __shfl_xor_sync(0xffffffffu, dg[n], o);
    }
  }
  if (active && sub == 0) {
#pragma unroll
    for (int r = 0; r < MOM_C; ++r) M[(set * A.ne + e) * MOM_C + r] = acc[r];
    if (want_dg) {
#pragma unroll
      for (int n = 0; n <= MOM_N; ++n) Dg[(set * A.ne + e) * (MOM_N + 1) + n] = dg[n];
    }
  }
}


// G4 of a moment block (BasisA::symm summed as in NNP::symm, nnp.cpp:359-377)
template <bool GEN>
__device__ void symm_mom_block(const WarpSmem& S, const AngP& A, const float* __restrict__ atab, bool cc, bool same, int j0, int nJ, int k0,
                               int nK, float* __restrict__ gmom, float* __restrict__ Gi) {
  const int lane = threadIdx.x & 31;
  const int nec = A.ne * MOM_C;
  float* MJ = S.ex;
  float* MK = same ? S.ex : S.ex + nec;
  float* Dg = S.ex + 2 * nec;
  if (!GEN || A.phi == ANG_GAUSS) build_moments<true>(S, A, cc, same ? 1 : 2, j0, j0 + nJ, k0, k0 + nK, MJ, same ? Dg : nullptr);
  else if constexpr (GEN) build_moments<false>(S, A, cc, same ? 1 : 2, j0, j0 + nJ, k0, k0 + nK, MJ, same ? Dg : nullptr);
  __syncwarp();
  if (gmom) {
    for (int t = lane; t < nec; t += 32) gmom[t] = MJ[t];
    if (!same)
      for (int t = lane; t < nec; t += 32) gmom[nec + t] = MK[t];
  }
  // V[e][n] = <M^J_n, M^K_n> (half the off-diagonal part for J == K)
  float* V = S.scratch;
  if (lane < A.ne * (MOM_N + 1)) {
    const int e = lane / (MOM_N + 1), n = lane % (MOM_N + 1);
    float s = 0.f;
    for (int r = mom_off(n); r < mom_off(n + 1); ++r) s = fmaf(c_mom_mult[r] * MJ[e * MOM_C + r], MK[e * MOM_C + r], s);
    if (same) s = 0.5f * (s - Dg[e * (MOM_N + 1) + n]);
    V[lane] = s;
  }
  __syncwarp();
  // G_f = sum_k M[f][k] V[k] (the block's coefficient matrix, norm included), one width at a time
  const int w = A.ne * (MOM_N + 1);
  const float* __restrict__ M = atab + A.tab + A.n;
  for (int f = lane; f < A.n; f += 32) {
    float v = 0.f;
    for (int e = 0; e < A.ne; ++e) {
      float m[MOM_N + 1];
#pragma unroll
      for (int k = 0; k <= MOM_N; ++k) m[k] = M[f * w + e * (MOM_N + 1) + k];
#pragma unroll
      for (int k = 0; k <= MOM_N; ++k) v = fmaf(m[k], V[e * (MOM_N + 1) + k], v);
    }
    Gi[A.off + f] = v;
  }
  __syncwarp();
}

// W_p -= d/dr_p of w_p(r) sum_n b_n <u_p^(x)n, B_n> for the slots [lo,hi).  With
// S_n = <u^(x)n, B_n> and V_n = <u^(x)(n-1), B_n> (a vector) the gradient is
// w' u sum_n b_n S_n + (w/r) sum_n n b_n (V_n - (u . V_n) u), and sum_n b_n S_n = b_0 B_0 + u . sum_n b_n V_n.
// T3[e*MOM_Q + q] holds b_n times the three components of B_n one degree above component q
// (n = deg q + 1), T0[e] = b_0 B_0; diag adds the j == k term of a J == K block.
template <bool GAUSS>
__device__ void mom_contract(const WarpSmem& S, const AngP& A, bool cc, int lo, int hi, const float4* __restrict__ T3,
                             const float* __restrict__ T0, const float* __restrict__ b, bool diag) {
  const int lane = threadIdx.x & 31;
  for (int p = lo + lane; p < hi; p += 32) {
    const float d = S.d[p], ux = S.ux[p], uy = S.uy[p], uz = S.uz[p], inv = S.inv[p];
    float f, g;
    if (cc) {
      f = S.fc[p];
      g = S.gc[p];
    } else {
      cutoff_fg(A.cut, d, A.rc, A.pirc, A.rci, f, g);
    }
    const float da = powi(d, A.alpha);
    const float dpa = (float)A.alpha * powi(d, A.alpha - 1) * f;
    // mult(q) u^(a,b,c) for the components q of degree <= 3, shared by every width
    float mono[MOM_Q];
    {
      float px[MOM_N], py[MOM_N], pz[MOM_N];
      px[0] = py[0] = pz[0] = 1.f;
#pragma unroll
      for (int k = 1; k < MOM_N; ++k) {
        px[k] = px[k - 1] * ux;
        py[k] = py[k - 1] * uy;
        pz[k] = pz[k - 1] * uz;
      }
#pragma unroll
      for (int n = 0; n < MOM_N; ++n)
#pragma unroll
        for (int a = n; a >= 0; --a)
#pragma unroll
          for (int bb = n - a; bb >= 0; --bb) {
            const int c = n - a - bb;
            mono[mom_idx(a, bb, c)] = mom_mult(a, bb, c) * px[a] * (py[bb] * pz[c]);
          }
    }
    float gx = 0.f, gy = 0.f, gz = 0.f;
    for (int e = 0; e < A.ne; ++e) {
      float kap = 1.0f;
      const float x = GAUSS ? __expf(-A.ietap[e] * da) : ang_h(A.phi, A.ietap[e] * da, kap);
      const float w = x * f;
      const float wd = x * (g - A.ietap[e] * kap * dpa);
      const float4* __restrict__ Te = T3 + e * MOM_Q;
      float vx[MOM_N], vy[MOM_N], vz[MOM_N];  // b_n V_n per degree n = 1..MOM_N
#pragma unroll
      for (int n = 0; n < MOM_N; ++n) vx[n] = vy[n] = vz[n] = 0.f;
#pragma unroll
      for (int n = 1; n <= MOM_N; ++n)
#pragma unroll
        for (int a = n - 1; a >= 0; --a)
#pragma unroll
          for (int bb = n - 1 - a; bb >= 0; --bb) {
            const int c = n - 1 - a - bb;
            const float m = mono[mom_idx(a, bb, c)];
            const float4 t = Te[mom_idx(a, bb, c)];
            vx[n - 1] = fmaf(m, t.x, vx[n - 1]);
            vy[n - 1] = fmaf(m, t.y, vy[n - 1]);
            vz[n - 1] = fmaf(m, t.z, vz[n - 1]);
          }
      float p1x = 0.f, p1y = 0.f, p1z = 0.f, p2x = 0.f, p2y = 0.f, p2z = 0.f;
#pragma unroll
      for (int n = 1; n <= MOM_N; ++n) {
        p1x += vx[n - 1];
        p1y += vy[n - 1];
        p1z += vz[n - 1];
        p2x = fmaf((float)n, vx[n - 1], p2x);
        p2y = fmaf((float)n, vy[n - 1], p2y);
        p2z = fmaf((float)n, vz[n - 1], p2z);
      }
      const float eb = T0[e] + ux * p1x + uy * p1y + uz * p1z;
      const float up2 = ux * p2x + uy * p2y + uz * p2z;
      const float s2 = w * inv;
      float s1 = wd * eb - s2 * up2;
      if (diag) {
        float bs = 0.f;
#pragma unroll
        for (int n = 0; n <= MOM_N; ++n) bs += b[e * (MOM_N + 1) + n];
        s1 -= w * wd * bs;
      }
      gx = fmaf(s1, ux, fmaf(s2, p2x, gx));
      gy = fmaf(s1, uy, fmaf(s2, p2y, gy));
      gz = fmaf(s1, uz, fmaf(s2, p2z, gz));
    }
    S.wx[p] -= gx;
    S.wy[p] -= gy;
    S.wz[p] -= gz;
  }
}

// chain rule of a moment block (BasisA::force summed as in NNP::force, nnp.cpp:466-478)
template <bool GEN>
__device__ void force_mom_block(const WarpSmem& S, const AngP& A, const float* __restrict__ atab, bool cc, bool same, int j0, int nJ, int k0,
                                int nK, const float* __restrict__ gmom, const float* __restrict__ gi) {
  const int lane = threadIdx.x & 31;
  const int nec = A.ne * MOM_C;
  // b[e][n] = norm * sum over the block's functions of width e of dE/dG_f * coef_n(f): the block's
  // coefficient matrix applied to the dE/dG values (lanes over its columns, rows coalesced)
  float* b = S.scratch;
  float* T0 = S.scratch + 32;  // [set][e]
  {
    const int w = A.ne * (MOM_N + 1);
    const float* __restrict__ M = atab + A.tab + A.n;
    if (lane < w) {
      float s0 = 0.f, s1 = 0.f;
      int f = 0;
      for (; f + 1 < A.n; f += 2) {
        s0 = fmaf(gi[A.off + f], M[f * w + lane], s0);
        s1 = fmaf(gi[A.off + f + 1], M[(f + 1) * w + lane], s1);
      }
      if (f < A.n) s0 = fmaf(gi[A.off + f], M[f * w + lane], s0);
      b[lane] = s0 + s1;
    }
  }
  __syncwarp();
  // the contraction tables of each set: b_(deg q + 1) times the three components one degree up
  float4* TJ = reinterpret_cast<float4*>(S.ex);
  float4* TK = same ? TJ : TJ + A.ne * MOM_Q;
  const int nsets = same ? 1 : 2;
  // the stored moments are in shared memory (copied asynchronously at the start of the kernel)
  const float* raw = gmom;
  // lane q builds entry q of every (set, width) table: its three component indices are fixed
  if (lane < MOM_Q) {
    const int u0 = c_mom_up[lane][0], u1 = c_mom_up[lane][1], u2 = c_mom_up[lane][2], dq = mom_deg(lane) + 1;
    for (int se = 0; se < nsets * A.ne; ++se) {
      const int set = se / A.ne, e = se % A.ne;
      const float bn = b[e * (MOM_N + 1) + dq];
      const float* Mg = raw + set * nec + e * MOM_C;
      (set ? TK : TJ)[e * MOM_Q + lane] = make_float4(bn * Mg[u0], bn * Mg[u1], bn * Mg[u2], 0.f);
    }
  }
  if (lane < nsets * A.ne) T0[lane] = b[(lane % A.ne) * (MOM_N + 1)] * raw[(lane / A.ne) * nec + (lane % A.ne) * MOM_C];
  __syncwarp();
  // J's slots against the K moments (J's own for J == K); K's slots against the J moments
  if (!GEN || A.phi == ANG_GAUSS) {
    mom_contract<true>(S, A, cc, j0, j0 + nJ, TK, T0 + (same ? 0 : A.ne), b, same);
    if (!same) mom_contract<true>(S, A, cc, k0, k0 + nK, TJ, T0, b, false);
  } else if constexpr (GEN) {
    mom_contract<false>(S, A, cc, j0, j0 + nJ, TK, T0 + (same ? 0 : A.ne), b, same);
    if (!same) mom_contract<false>(S, A, cc, k0, k0 + nK, TJ, T0, b, false);
  }
  __syncwarp();
}

// ------------------------------------------------------------------ shared moments
// Centre types whose moment blocks share one pair weight (PotParams::msh): the moments of each of
// the (at most two) neighbour species are built once, and every moment block takes its inner
// products from them; the chain rule contracts each neighbour once against the sum of the
// tables of the blocks that contain its species.  The same sums as the per-block path.
__device__ __forceinline__ int mom_set(const PotParams& P, int I, int sp) { return sp == P.msp[I][0] ? 0 : 1; }

// G4 of every moment block of centre type I; gmom (may be null) receives the moments
template <bool GEN>
__device__ void symm_mom_shared(const WarpSmem& S, const PotParams& P, int I, bool cc, float* __restrict__ gmom, float* __restrict__ Gi) {
  const int lane = threadIdx.x & 31;
  const AngP& R = P.ang[I][P.mrep[I]];
  const int ns = P.mns[I], ne = R.ne, nec = ne * MOM_C;
  const int sp0 = P.msp[I][0], sp1 = ns > 1 ? P.msp[I][1] : sp0;
  float* MS = S.ex;               // [set][e][MOM_C]
  float* Dg = S.ex + ns * nec;    // [set][e][MOM_N+1]
  const int lo0 = S.toff[sp0], hi0 = S.toff[sp0 + 1], lo1 = S.toff[sp1], hi1 = S.toff[sp1 + 1];
  if (!GEN || R.phi == ANG_GAUSS) build_moments<true>(S, R, cc, ns, lo0, hi0, lo1, hi1, MS, Dg);
  else if constexpr (GEN) build_moments<false>(S, R, cc, ns, lo0, hi0, lo1, hi1, MS, Dg);
  __syncwarp();
  if (gmom)
    for (int t = lane; t < ns * nec; t += 32) gmom[t] = MS[t];
  // the moment blocks (at most three): species pairs packed 4 bits each, function counts 8 bits
  int pk = 0, nk = 0, nb = 0, nf = 0;
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0 || !A.mom || nb >= 3) continue;
      pk |= (J | (K << 2)) << (4 * nb);
      nk |= A.n << (8 * nb);
      nf += A.n;
      ++nb;
    }
  // inner products V[blk][e][n] of every block at once, lanes over (block, width, degree)
  const int w = ne * (MOM_N + 1);
  float* V = S.scratch;
  for (int t = lane; t < nb * w; t += 32) {
    const int k = t / w, c = t - k * w, e = c / (MOM_N + 1), n = c - e * (MOM_N + 1);
    const int J = (pk >> (4 * k)) & 3, K = (pk >> (4 * k + 2)) & 3;
    const int sJ = mom_set(P, I, J), sK = mom_set(P, I, K);
    const float* MJ = MS + sJ * nec + e * MOM_C;
    const float* MK = MS + sK * nec + e * MOM_C;
    float v0 = 0.f, v1 = 0.f;
    int r = mom_off(n);
    const int r1 = mom_off(n + 1);
    for (; r + 1 < r1; r += 2) {
      v0 = fmaf(c_mom_mult[r] * MJ[r], MK[r], v0);
      v1 = fmaf(c_mom_mult[r + 1] * MJ[r + 1], MK[r + 1], v1);
    }
    if (r < r1) v0 = fmaf(c_mom_mult[r] * MJ[r], MK[r], v0);
    float v = v0 + v1;
    if (J == K) v = 0.5f * (v - Dg[(sJ * ne + e) * (MOM_N + 1) + n]);
    V[t] = v;
  }
  __syncwarp();
  // every block's functions at once, lanes over (block, function): G_f = sum_c M[f][c] V[blk][c]
  for (int t = lane; t < nf; t += 32) {
    int k = 0, f = t;
    while (k + 1 < nb && f >= ((nk >> (8 * k)) & 255)) {
      f -= (nk >> (8 * k)) & 255;
      ++k;
    }
    const AngP& A = P.ang[I][lidx((pk >> (4 * k)) & 3, (pk >> (4 * k + 2)) & 3)];
    const float* __restrict__ M = P.atab + A.tab + A.n + f * w;
    const float* Vk = V + k * w;
    float g = 0.f;
    for (int e = 0; e < ne; ++e) {  // one width (MOM_N + 1 columns) at a time, loads first
      float m[MOM_N + 1];
#pragma unroll
      for (int c = 0; c <= MOM_N; ++c) m[c] = M[e * (MOM_N + 1) + c];
#pragma unroll
      for (int c = 0; c <= MOM_N; ++c) g = fmaf(m[c], Vk[e * (MOM_N + 1) + c], g);
    }
    Gi[A.off + f] = g;
  }
  __syncwarp();
}

// chain rule of every moment block of centre type I from the stored moments gm
template <bool GEN>
__device__ void force_mom_shared(const WarpSmem& S, const PotParams& P, int I, bool cc, const float* __restrict__ gm,
                                 const float* __restrict__ gi) {
  const int lane = threadIdx.x & 31;
  const AngP& R = P.ang[I][P.mrep[I]];
  const int ns = P.mns[I], ne = R.ne, nec = ne * MOM_C, w = ne * (MOM_N + 1);
  // coefficients b[blk][e][n] of each moment block (the coefficient matrix applied to dE/dG);
  // the blocks' species pairs packed 4 bits each (J | K << 2) so that they stay in a register
  int pk = 0, nb = 0;
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0 || !A.mom || nb >= 3) continue;
      pk |= (J | (K << 2)) << (4 * nb);
      ++nb;
    }
  // every block at once, lanes over (block, column)
  for (int t = lane; t < nb * w; t += 32) {
    const int k = t / w, c = t - k * w;
    const AngP& A = P.ang[I][lidx((pk >> (4 * k)) & 3, (pk >> (4 * k + 2)) & 3)];
    const float* __restrict__ M = P.atab + A.tab + A.n + c;
    const float* g = gi + A.off;
    float s0 = 0.f, s1 = 0.f;
    int f = 0;
    for (; f + 1 < A.n; f += 2) {
      s0 = fmaf(g[f], M[f * w], s0);
      s1 = fmaf(g[f + 1], M[(f + 1) * w], s1);
    }
    if (f < A.n) s0 = fmaf(g[f], M[f * w], s0);
    S.scratch[20 * k + c] = s0 + s1;
  }
  __syncwarp();
  // tables of each species set: T_s[e][q] = sum over the blocks containing the species of
  // b_(deg q + 1) times the other species' moments one degree up; T0_s[e] likewise with degree 0
  float4* T = reinterpret_cast<float4*>(S.ex);
  float* T0 = S.scratch + 60;  // [set][e]
  for (int v = lane; v < ns * ne * MOM_Q; v += 32) {
    const int se = v / MOM_Q, q = v - se * MOM_Q;
    const int u0 = c_mom_up[q][0], u1 = c_mom_up[q][1], u2 = c_mom_up[q][2], dq = mom_deg(q) + 1;
    const int set = se / ne, e = se % ne;
    const int spc = P.msp[I][set];
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = 0; k < nb; ++k) {
      const int bJ = (pk >> (4 * k)) & 3, bK = (pk >> (4 * k + 2)) & 3;
      if (bJ != spc && bK != spc) continue;
      const int other = bJ == spc ? bK : bJ;
      const float bn = S.scratch[20 * k + e * (MOM_N + 1) + dq];
      const float* Mg = gm + mom_set(P, I, other) * nec + e * MOM_C;
      t.x = fmaf(bn, Mg[u0], t.x);
      t.y = fmaf(bn, Mg[u1], t.y);
      t.z = fmaf(bn, Mg[u2], t.z);
    }
    T[se * MOM_Q + q] = t;
  }
  if (lane < ns * ne) {
    const int set = lane / ne, e = lane % ne, spc = P.msp[I][set];
    float t0 = 0.f;
    for (int k = 0; k < nb; ++k) {
      const int bJ = (pk >> (4 * k)) & 3, bK = (pk >> (4 * k + 2)) & 3;
      if (bJ != spc && bK != spc) continue;
      const int other = bJ == spc ? bK : bJ;
      t0 = fmaf(S.scratch[20 * k + e * (MOM_N + 1)], gm[mom_set(P, I, other) * nec + e * MOM_C], t0);
    }
    T0[lane] = t0;
  }
  __syncwarp();
  // each species' slots once; a species' own block (J == K) adds its diagonal term
  for (int set = 0; set < ns; ++set) {
    const int spc = P.msp[I][set];
    int kd = -1;
    for (int k = 0; k < nb; ++k)
      if (((pk >> (4 * k)) & 3) == spc && ((pk >> (4 * k + 2)) & 3) == spc) kd = k;
    const float* bd = kd >= 0 ? S.scratch + 20 * kd : S.scratch;
    if (!GEN || R.phi == ANG_GAUSS)
      mom_contract<true>(S, R, cc, S.toff[spc], S.toff[spc + 1], T + set * ne * MOM_Q, T0 + set * ne, bd, kd >= 0);
    else if constexpr (GEN)
      mom_contract<false>(S, R, cc, S.toff[spc], S.toff[spc + 1], T + set * ne * MOM_Q, T0 + set * ne, bd, kd >= 0);
    __syncwarp();
  }
}

// Stage the neighbour slots of atom i in shared memory, grouped by neighbour type.
// Returns the number of staged slots; toff[t]..toff[t+1] is the range of type t.
static __device__ int stage_neighbors(const WarpSmem& S, int i, int cap, int ntypes, const int* __restrict__ type,
                               const int* __restrict__ nb_j, const unsigned char* __restrict__ nb_t, const float4* __restrict__ nb_r,
                               const int* __restrict__ nb_cnt) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int n = min(nb_cnt[i], cap);
  // neighbour types and vectors, one chunk of 32 slots per register (cap <= 32 * QMAX), all
  // loads issued before the first ballot consumes one
  int tq[QMAX];
  float4 rq[QMAX];
#pragma unroll
  for (int q = 0; q < QMAX; ++q) {
    const int s = q * 32 + lane;
    const size_t g = (size_t)i * cap + s;
    const bool on = s < n;
    tq[q] = on ? clamp_type(nb_t ? (int)nb_t[g] : type[nb_j[g]], ntypes) : -1;
    rq[q] = on ? nb_r[g] : make_float4(0.f, 0.f, 0.f, 1.f);
  }
  int cnt[NT_MAX];
#pragma unroll
  for (int t = 0; t < NT_MAX; ++t) cnt[t] = 0;
#pragma unroll
  for (int q = 0; q < QMAX; ++q)
    if (q * 32 < n) {
#pragma unroll
      for (int tt = 0; tt < NT_MAX; ++tt) cnt[tt] += __popc(__ballot_sync(0xffffffffu, tq[q] == tt));
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
#pragma unroll
  for (int q = 0; q < QMAX; ++q) {
    if (q * 32 >= n) break;
    const int s = q * 32 + lane;
    const int t = tq[q];
    int pos = 0;
#pragma unroll
    for (int tt = 0; tt < NT_MAX; ++tt) {
      const unsigned m = __ballot_sync(0xffffffffu, t == tt);
      if (t == tt) pos = run[tt] + __popc(m & lt);
      run[tt] += __popc(m);
    }
    if (s < n) {
      const float4 r = rq[q];
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

// Per-pair factors of angular block A for slots [lo,hi): ex[e] = h(ietap_e d^alpha) (times the
// cutoff when with_fc) and, where the kernel has the region, kx[e] = its derivative weight
// (ang_h); sum families instead keep d^alpha in ex[p].  Also the cutoff value/gradient and
// alpha d^(alpha-1) fc.
template <bool GEN>
__device__ void block_pair_factors(const WarpSmem& S, const AngP& A, int lo, int hi, int cap, bool with_fc) {
  const int lane = threadIdx.x & 31;
  const bool sum = GEN && (ang_sum_family(A.phi) || A.fn);
  for (int p = lo + lane; p < hi; p += 32) {
    const float d = S.d[p];
    float f, g;
    cutoff_fg(A.cut, d, A.rc, A.pirc, A.rci, f, g);
    const float da = powi(d, A.alpha);
    if (sum) S.ex[p] = da;
    else if (!GEN || A.phi == ANG_GAUSS)
      for (int e = 0; e < A.ne; ++e) {
        const float x = __expf(-A.ietap[e] * da);
        S.ex[e * cap + p] = with_fc ? x * f : x;
        if (S.kx) S.kx[e * cap + p] = 1.0f;
      }
    else
      for (int e = 0; e < A.ne; ++e) {
        float kap;
        const float x = GEN ? ang_h(A.phi, A.ietap[e] * da, kap) : 0.f;
        S.ex[e * cap + p] = with_fc ? x * f : x;
        if (S.kx) S.kx[e * cap + p] = kap;
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
// TOP: only the level m = NZ-1 (the triplet part of a split block, AngP::top).
template <int NE, int NZ, bool TOP>
__device__ __forceinline__ void symm_block(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  constexpr int NC = TOP ? 1 : NZ, M0 = TOP ? NZ - 1 : 0;  // accumulated levels M0 .. M0+NC-1
  const int lane = threadIdx.x & 31;
  float acc[NE][NL][NC];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NC; ++m) acc[e][l][m] = 0.f;
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
          for (int m = 0; m < NC; ++m) acc[e][l][m] = fmaf(p2[l][M0 + m], E2, fmaf(p1[l][M0 + m], E1, acc[e][l][m]));
      }
    }
  }
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NC; ++m) {
        const float v = warp_sum(acc[e][l][m]);
        if (lane == 0) S.scratch[(e * NL + l) * NZ_MAX + M0 + m] = v;
      }
}

// Chain rule of one block: per triplet phi = dE/dcos and eta0/eta1 = dE/dr_ij, dE/dr_ik
// summed over the block's functions (BasisA::force, basis_angular.cpp:456-507), turned into the
// neighbour-slot vectors of NNP::force (nnp.cpp:466-478).  The owner's vector accumulates in
// registers; the partner's goes to shared memory (distinct partners within a round).
// One triplet of the chain rule for owner a (registers) and partner b: returns the owner-side
// vector in (oa*) and the partner-side vector in (ob*).
// TOP: only the level m = NZ-1, p^(2^(NZ-1)) and its derivative 2^(NZ-1) p^(2^(NZ-1)-1) from
// the squaring chain and the running product of its terms.
template <int NE, int NZ, bool TOP>
__device__ __forceinline__ void chain_triplet(float uax, float uay, float uaz, float fa, float ga, float pa, float ia, const float* exa,
                                              float ubx, float uby, float ubz, float fb, float gb, float pb, float ib, const float* exb,
                                              const float (&sg)[NE][NL][TOP ? 1 : NZ], const float* ie, float lam0, float lam1, float hn,
                                              float nn, float& oa0, float& oa1, float& oa2, float& ob0, float& ob1, float& ob2) {
  constexpr int NC = TOP ? 1 : NZ;
  const float cs = uax * ubx + uay * uby + uaz * ubz;
  float p[NL][NC], qd[NL][NC];
  const float b0 = fabsf(0.5f * (1.0f + lam0 * cs)), b1 = fabsf(0.5f * (1.0f + lam1 * cs));
  if constexpr (TOP) {
    float x0 = b0, x1 = b1, r0 = 1.0f, r1 = 1.0f;
#pragma unroll
    for (int m = 1; m < NZ; ++m) {
      r0 *= x0; r1 *= x1;
      x0 *= x0; x1 *= x1;
    }
    p[0][0] = x0; p[1][0] = x1;
    qd[0][0] = (float)(1 << (NZ - 1)) * r0;
    qd[1][0] = (float)(1 << (NZ - 1)) * r1;
  } else {
    p[0][0] = b0;
    p[1][0] = b1;
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      qd[l][0] = 1.0f;
#pragma unroll
      for (int m = 1; m < NZ; ++m) {
        qd[l][m] = 2.0f * qd[l][m - 1] * p[l][m - 1];
        p[l][m] = p[l][m - 1] * p[l][m - 1];
      }
    }
  }
  float Q = 0.f, Q2 = 0.f, Pp = 0.f;
#pragma unroll
  for (int e = 0; e < NE; ++e) {
    const float E = exa[e] * exb[e];
    float q0 = 0.f, q1 = 0.f, r0 = 0.f, r1 = 0.f;
#pragma unroll
    for (int m = 0; m < NC; ++m) {
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
template <int NE, int NZ, bool TOP>
__device__ __forceinline__ void force_block(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  constexpr int NC = TOP ? 1 : NZ, M0 = TOP ? NZ - 1 : 0;
  const int lane = threadIdx.x & 31;
  float sg[NE][NL][NC];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NC; ++m) sg[e][l][m] = S.scratch[(e * NL + l) * NZ_MAX + M0 + m];
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
        chain_triplet<NE, NZ, TOP>(uax, uay, uaz, fa, ga, pa, ia, exa, ux[b], uy[b], uz[b], fc[b], gc[b], dpa[b], inv[b], exb, sg, ie,
                                   lam0, lam1, hn, nn, a0, a1, a2, c0, c1, c2);
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

// G4 sums of a sum-family block (IPOWS, SECHS: basis_angular.cpp:427-441) on the triplet path:
// the factor h(ietap (r_ij^alpha + r_ik^alpha)) per triplet from ex[p] = r_p^alpha, times the
// cutoffs in fc.  One instance per kernel (its NE x NZ bounds); widths beyond the block's are
// skipped.
template <int NE, int NZ>
__device__ void symm_block_sum(const WarpSmem& S, const AngP& A, const Sched& sc) {
  const int lane = threadIdx.x & 31;
  float acc[NE][NL][NZ];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NZ; ++m) acc[e][l][m] = 0.f;
  const float lam0 = A.lam[0], lam1 = A.lam[1];
  for (int q = 0; q * 32 < sc.nown; ++q) {
    const int x = q * 32 + lane;
    const int a = sc.xb + min(x, sc.nown - 1);
    const float uax = S.ux[a], uay = S.uy[a], uaz = S.uz[a], daa = S.ex[a], fa = S.fc[a];
    for (int dd = sc.d0; dd <= sc.d1; ++dd) {
      const int nx = (sc.tri && 2 * dd == sc.nJ) ? (sc.nJ >> 1) : sc.nown;
      if (x < nx) {
        int y = x + dd;
        if (y >= sc.mod) y -= sc.mod;
        const int b = sc.yb + y;
        const float cs = uax * S.ux[b] + uay * S.uy[b] + uaz * S.uz[b];
        float p[NL][NZ];
        p[0][0] = fabsf(0.5f * (1.0f + lam0 * cs));
        p[1][0] = fabsf(0.5f * (1.0f + lam1 * cs));
#pragma unroll
        for (int l = 0; l < NL; ++l)
#pragma unroll
          for (int m = 1; m < NZ; ++m) p[l][m] = p[l][m - 1] * p[l][m - 1];
        const float fab = fa * S.fc[b], s = daa + S.ex[b];
#pragma unroll
        for (int e = 0; e < NE; ++e) {
          if (e >= A.ne) break;
          float kap;
          const float E = fab * ang_h(A.phi, A.ietap[e] * s, kap);
#pragma unroll
          for (int l = 0; l < NL; ++l)
#pragma unroll
            for (int m = 0; m < NZ; ++m) acc[e][l][m] = fmaf(p[l][m], E, acc[e][l][m]);
        }
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

// Chain rule of a block of the non-GAUSS families on the triplet path (BasisA::force,
// basis_angular.cpp:508-640).  Per triplet and width, the radial factor R and its derivative
// weights kap_a, kap_b (dR/dr_a = -ietap alpha r_a^(alpha-1) kap_a R): products from the pair
// regions ex and kx, sums from h(ietap (r_ij^alpha + r_ik^alpha)).  Then
//   eta0 = -norm f_b (g_a Q - alpha r_a^(alpha-1) f_a Q2a),  Q = sum R q,  Q2a = sum ietap kap_a R q,
// and likewise eta1; phi as for GAUSS.  One instance per kernel, widths beyond the block's skipped.
template <int NE, int NZ>
__device__ void force_block_gen(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  const int lane = threadIdx.x & 31;
  float sg[NE][NL][NZ];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NZ; ++m) sg[e][l][m] = S.scratch[(e * NL + l) * NZ_MAX + m];
  const bool sum = ang_sum_family(A.phi);
  const float lam0 = A.lam[0], lam1 = A.lam[1];
  const float hn = -0.5f * A.norm, nn = -A.norm;
  for (int q = 0; q * 32 < sc.nown; ++q) {
    const int x = q * 32 + lane;
    const int a = sc.xb + min(x, sc.nown - 1);
    const float uax = S.ux[a], uay = S.uy[a], uaz = S.uz[a];
    const float fa = S.fc[a], ga = S.gc[a], pa = S.dpa[a], ia = S.inv[a];
    float w0 = 0.f, w1 = 0.f, w2 = 0.f;
    for (int dd = sc.d0; dd <= sc.d1; ++dd) {
      const int nx = (sc.tri && 2 * dd == sc.nJ) ? (sc.nJ >> 1) : sc.nown;
      if (x < nx) {
        int y = x + dd;
        if (y >= sc.mod) y -= sc.mod;
        const int b = sc.yb + y;
        const float ubx = S.ux[b], uby = S.uy[b], ubz = S.uz[b];
        const float fb = S.fc[b], gb = S.gc[b], pb = S.dpa[b], ib = S.inv[b];
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
        float Q = 0.f, Q2a = 0.f, Q2b = 0.f, Pp = 0.f;
#pragma unroll
        for (int e = 0; e < NE; ++e) {
          if (e >= A.ne) break;
          float R, ka, kb;
          if (sum) {
            R = ang_h(A.phi, A.ietap[e] * (S.ex[a] + S.ex[b]), ka);
            kb = ka;
          } else {
            R = S.ex[e * cap + a] * S.ex[e * cap + b];
            ka = S.kx[e * cap + a];
            kb = S.kx[e * cap + b];
          }
          float q0 = 0.f, q1 = 0.f, r0 = 0.f, r1 = 0.f;
#pragma unroll
          for (int m = 0; m < NZ; ++m) {
            q0 = fmaf(sg[e][0][m], p[0][m], q0);
            q1 = fmaf(sg[e][1][m], p[1][m], q1);
            r0 = fmaf(sg[e][0][m], qd[0][m], r0);
            r1 = fmaf(sg[e][1][m], qd[1][m], r1);
          }
          const float qe = R * (q0 + q1), ie = A.ietap[e];
          Q += qe;
          Q2a = fmaf(ie * ka, qe, Q2a);
          Q2b = fmaf(ie * kb, qe, Q2b);
          Pp = fmaf(R, lam0 * r0 + lam1 * r1, Pp);
        }
        const float phi = hn * fa * fb * Pp;
        const float eta0 = nn * fb * (ga * Q - pa * Q2a);
        const float eta1 = nn * fa * (gb * Q - pb * Q2b);
        const float Aa = -phi * cs * ia + eta0, Ba = phi * ia;
        const float Ab = -phi * cs * ib + eta1, Bb = phi * ib;
        w0 += Aa * uax + Ba * ubx;
        w1 += Aa * uay + Ba * uby;
        w2 += Aa * uaz + Ba * ubz;
        S.wx[b] += Ab * ubx + Bb * uax;
        S.wy[b] += Ab * uby + Bb * uay;
        S.wz[b] += Ab * ubz + Bb * uaz;
      }
      __syncwarp();
    }
    if (x < sc.nown) {
      S.wx[sc.xb + x] += w0;
      S.wy[sc.xb + x] += w1;
      S.wz[sc.xb + x] += w2;
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ per-function angular blocks
// Blocks that leave the (width) x (lambda) x (2^m) grid (AngP::fn: a real zeta, more than NE_MAX
// widths or NL lambdas) evaluate every function per triplet, as BasisA::symm and BasisA::force do
// (basis_angular.cpp:406-640): pow(|(1 + lambda cos)/2|, zeta) times the family's radial factor
// from ex[p] = r_p^alpha and the cutoffs.  Linked only into the GEN kernel instances.
constexpr int FN_CHUNK = 8;  // functions accumulated per walk over the block's triplets

// radial factor of one function: product families h(ie r_a^alpha) h(ie r_b^alpha), sum families
// and GAUSS functions of ie (r_a^alpha + r_b^alpha); ka, kb the derivative weights of ang_h
__device__ __forceinline__ float fn_radial(int phi, float ie, float da, float db, float& ka, float& kb) {
  if (phi == ANG_IPOWP || phi == ANG_SECHP) {
    const float ha = ang_h(phi, ie * da, ka);
    const float hb = ang_h(phi, ie * db, kb);
    return ha * hb;
  }
  const float h = ang_h(phi, ie * (da + db), ka);
  kb = ka;
  return h;
}

// G4 of a per-function block: FN_CHUNK functions per walk, written to Gi (times the norm).
static __device__ void symm_block_fn(const WarpSmem& S, const AngP& A, const float* __restrict__ ftab, const Sched& sc, float* Gi) {
  const int lane = threadIdx.x & 31;
  for (int f0 = 0; f0 < A.n; f0 += FN_CHUNK) {
    float ie[FN_CHUNK], lam[FN_CHUNK], zeta[FN_CHUNK], acc[FN_CHUNK];
#pragma unroll
    for (int k = 0; k < FN_CHUNK; ++k) {
      const int f = min(f0 + k, A.n - 1);
      ie[k] = ftab[4 * f];
      lam[k] = ftab[4 * f + 1];
      zeta[k] = ftab[4 * f + 2];
      acc[k] = 0.f;
    }
    for (int q = 0; q * 32 < sc.nown; ++q) {
      const int x = q * 32 + lane;
      const int a = sc.xb + min(x, sc.nown - 1);
      const float uax = S.ux[a], uay = S.uy[a], uaz = S.uz[a], da = S.ex[a], fa = S.fc[a];
      for (int dd = sc.d0; dd <= sc.d1; ++dd) {
        const int nx = (sc.tri && 2 * dd == sc.nJ) ? (sc.nJ >> 1) : sc.nown;
        if (x < nx) {
          int y = x + dd;
          if (y >= sc.mod) y -= sc.mod;
          const int b = sc.yb + y;
          const float cs = uax * S.ux[b] + uay * S.uy[b] + uaz * S.uz[b];
          const float fab = fa * S.fc[b], db = S.ex[b];
#pragma unroll
          for (int k = 0; k < FN_CHUNK; ++k) {
            float ka, kb;
            const float R = fn_radial(A.phi, ie[k], da, db, ka, kb);
            acc[k] = fmaf(powf(fabsf(0.5f * (1.0f + lam[k] * cs)), zeta[k]), R * fab, acc[k]);
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < FN_CHUNK; ++k) {
      const float v = warp_sum(acc[k]);
      if (lane == 0 && f0 + k < A.n) Gi[A.off + f0 + k] = A.norm * v;
    }
  }
}

// Chain rule of a per-function block: per triplet the sums over the block's functions of
// BasisA::force (basis_angular.cpp:456-640) with cw = |(1 + lambda cos)/2| and s = dE/dG_f:
//   Q = sum s R cw^zeta,  Q2a/b = sum s ie k_a/b R cw^zeta,  Pp = sum s R lambda zeta cw^(zeta-1),
// then phi, eta0, eta1 and the slot vectors as in force_block_gen.
static __device__ void force_block_fn(const WarpSmem& S, const AngP& A, const float* __restrict__ ftab, const Sched& sc, const float* gi) {
  const int lane = threadIdx.x & 31;
  const float hn = -0.5f * A.norm, nn = -A.norm;
  const float* __restrict__ sf = gi + A.off;
  for (int q = 0; q * 32 < sc.nown; ++q) {
    const int x = q * 32 + lane;
    const int a = sc.xb + min(x, sc.nown - 1);
    const float uax = S.ux[a], uay = S.uy[a], uaz = S.uz[a], da = S.ex[a];
    const float fa = S.fc[a], ga = S.gc[a], pa = S.dpa[a], ia = S.inv[a];
    float w0 = 0.f, w1 = 0.f, w2 = 0.f;
    for (int dd = sc.d0; dd <= sc.d1; ++dd) {
      const int nx = (sc.tri && 2 * dd == sc.nJ) ? (sc.nJ >> 1) : sc.nown;
      if (x < nx) {
        int y = x + dd;
        if (y >= sc.mod) y -= sc.mod;
        const int b = sc.yb + y;
        const float ubx = S.ux[b], uby = S.uy[b], ubz = S.uz[b], db = S.ex[b];
        const float fb = S.fc[b], gb = S.gc[b], pb = S.dpa[b], ib = S.inv[b];
        const float cs = uax * ubx + uay * uby + uaz * ubz;
        float Q = 0.f, Q2a = 0.f, Q2b = 0.f, Pp = 0.f;
#pragma unroll 2
        for (int f = 0; f < A.n; ++f) {
          const float ie = ftab[4 * f], lam = ftab[4 * f + 1], zeta = ftab[4 * f + 2];
          float ka, kb;
          const float R = fn_radial(A.phi, ie, da, db, ka, kb);
          const float cw = fabsf(0.5f * (1.0f + lam * cs));
          const float cz1 = powf(cw, zeta - 1.0f);
          const float sR = sf[f] * R;
          const float qe = sR * cw * cz1;
          Q += qe;
          Q2a = fmaf(ie * ka, qe, Q2a);
          Q2b = fmaf(ie * kb, qe, Q2b);
          Pp = fmaf(sR, lam * zeta * cz1, Pp);
        }
        const float phi = hn * fa * fb * Pp;
        const float eta0 = nn * fb * (ga * Q - pa * Q2a);
        const float eta1 = nn * fa * (gb * Q - pb * Q2b);
        const float Aa = -phi * cs * ia + eta0, Ba = phi * ia;
        const float Ab = -phi * cs * ib + eta1, Bb = phi * ib;
        w0 += Aa * uax + Ba * ubx;
        w1 += Aa * uay + Ba * uby;
        w2 += Aa * uaz + Ba * ubz;
        S.wx[b] += Ab * ubx + Bb * uax;
        S.wy[b] += Ab * uby + Bb * uay;
        S.wz[b] += Ab * ubz + Bb * uaz;
      }
      __syncwarp();
    }
    if (x < sc.nown) {
      S.wx[sc.xb + x] += w0;
      S.wy[sc.xb + x] += w1;
      S.wz[sc.xb + x] += w2;
    }
    __syncwarp();
  }
}

// Dispatch on the block's grid size: eta count 1..NEK, zeta chain length rounded up to 3, 5 or 6
// (at most NZK).  Only instances within the kernel's bounds are linked, which keeps the
// kernel's register allocation to what its potential needs.
// The non-GAUSS families take the one generic instance at the kernel's bounds (their G4 sums
// for the product families are the GAUSS ones on other pair factors).  Their code is linked
// only into the GEN kernel instances, launched for potentials that have such blocks: the
// GAUSS-only instances keep the code size and register allocation of the GAUSS code alone.
template <bool FORCE, int NEK, int NZK, bool GEN>
__device__ void run_block(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  if constexpr (GEN) {
    if (FORCE && A.phi != ANG_GAUSS) {
      force_block_gen<NEK, NZK>(S, A, sc, cap);
      return;
    }
    if (!FORCE && ang_sum_family(A.phi)) {
      symm_block_sum<NEK, NZK>(S, A, sc);
      return;
    }
  }
  if (A.top) {  // the top level of a split block: exact nz
#define NNP_TOP(NE_, NZ_)                                         \
  case NE_ * 8 + NZ_:                                             \
    if constexpr (NE_ <= NEK && NZ_ <= NZK) {                     \
      if (FORCE) force_block<NE_, NZ_, true>(S, A, sc, cap);      \
      else symm_block<NE_, NZ_, true>(S, A, sc, cap);             \
    }                                                             \
    break;
    switch (A.ne * 8 + A.nz) {
      NNP_TOP(1, 4) NNP_TOP(1, 5) NNP_TOP(1, 6)
      NNP_TOP(2, 4) NNP_TOP(2, 5) NNP_TOP(2, 6)
      NNP_TOP(3, 4) NNP_TOP(3, 5) NNP_TOP(3, 6)
      NNP_TOP(4, 4) NNP_TOP(4, 5) NNP_TOP(4, 6)
      default: break;
    }
#undef NNP_TOP
    return;
  }
  const int z = A.nz <= 3 ? 3 : (A.nz <= 5 ? 5 : 6);
  const int key = A.ne * 8 + z;
#define NNP_CASE(NE_, NZ_)                                   \
  case NE_ * 8 + NZ_:                                        \
    if constexpr (NE_ <= NEK && NZ_ <= NZK) {                \
      if (FORCE) force_block<NE_, NZ_, false>(S, A, sc, cap); \
      else symm_block<NE_, NZ_, false>(S, A, sc, cap);        \
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

// Radial function of family phi without the cutoff (BasisR::symm, basis_radial.cpp:302-364), with
// x = r - rs and arg = -eta x; FP32, exponentials through __expf.
__device__ __forceinline__ float radial_value(int phi, float eta, float rs, float d) {
  const float x = d - rs, arg = -eta * x;
  switch (phi) {
    case RAD_GAUSSIAN: return __expf(-eta * x * x);
    case RAD_TANH: return 0.5f * (tanhf(arg) + 1.0f);
    case RAD_SOFTPLUS: return arg > 0.f ? arg + log1pf(__expf(-arg)) : log1pf(__expf(arg));
    case RAD_LOGCOSH: return arg > 0.f ? arg + 0.5f * log1pf(__expf(-2.0f * arg)) : 0.5f * log1pf(__expf(2.0f * arg));
    case RAD_SWISH:
      if (arg > 0.f) { const float e = __expf(-arg); return arg / (1.0f + e); }
      if (arg < 0.f) { const float e = __expf(arg); return arg * e / (1.0f + e); }
      return 0.f;
    default:  // RAD_MISH
      if (arg > 0.f) { const float e = __expf(-arg); return arg * (2.0f * e + 1.0f) / (2.0f * e * (e + 1.0f) + 1.0f); }
      if (arg < 0.f) { const float e = __expf(arg); return arg * e * (e + 2.0f) / (e * (e + 2.0f) + 2.0f); }
      return 0.f;
  }
}

// The per-function term of BasisR::force (basis_radial.cpp:371-444): amp -= dE/dG_i times this,
// the reference's expressions for each family (cut, gcut: cutoff value and derivative).
__device__ __forceinline__ float radial_force_term(int phi, float eta, float rs, float d, float cut, float gcut) {
  const float x = d - rs, arg = -eta * x;
  switch (phi) {
    case RAD_GAUSSIAN: return __expf(-eta * x * x) * (-2.0f * eta * x * cut + gcut);
    case RAD_TANH: {
      const float t = tanhf(arg);
      return 0.5f * (-eta * (1.0f - t * t) * cut + (1.0f + t) * gcut);
    }
    case RAD_SOFTPLUS:
      if (arg > 0.f) { const float e = __expf(-arg); return -eta / (1.0f + e) * cut + (arg + log1pf(e)) * gcut; }
      else { const float e = __expf(arg); return -eta * e / (1.0f + e) * cut + log1pf(e) * gcut; }
    case RAD_LOGCOSH:
      if (arg > 0.f) { const float e = __expf(-2.0f * arg); return -eta / (1.0f + e) * cut + (arg + 0.5f * log1pf(e)) * gcut; }
      else { const float e = __expf(2.0f * arg); return -eta * e / (1.0f + e) * cut + 0.5f * log1pf(e) * gcut; }
    case RAD_SWISH:
      if (arg > 0.f) {
        const float e = __expf(-arg), den = 1.0f / (1.0f + e);
        return (-eta * (1.0f + e * (1.0f + arg)) * den * cut + arg * gcut) * den;
      } else {
        const float e = __expf(arg), den = 1.0f / (1.0f + e);
        return (-eta * (1.0f + arg + e) * den * cut + arg * gcut) * e * den;
      }
    default:  // RAD_MISH
      if (arg > 0.f) {
        const float e = __expf(-arg), den = 1.0f / (2.0f * e * (e + 1.0f) + 1.0f);
        return (-eta * (1.0f + e * (4.0f + e * (4.0f * arg + 6.0f + e * 4.0f * (arg + 1.0f)))) * den * cut +
                arg * (2.0f * e + 1.0f) * gcut) * den;
      } else {
        const float e = __expf(arg), den = 1.0f / (e * (e + 2.0f) + 2.0f);
        return (-eta * (e * (e * (e + 4.0f) + 4.0f * arg + 6.0f) + 4.0f * (arg + 1.0f)) * den * cut + arg * (e + 2.0f) * gcut) * den * e;
      }
  }
}

// When every basis of centre type I shares one cutoff function and radius, evaluate it once per
// staged neighbour (value and derivative into S.fc / S.gc) for all blocks to read.
__device__ __forceinline__ bool cutoff_cache(const WarpSmem& S, const PotParams& P, int I, int n) {
  if (!P.ccut[I]) return false;
  const int lane = threadIdx.x & 31;
  for (int p = lane; p < n; p += 32) {
    float f, g;
    cutoff_fg(P.ccut[I], S.d[p], P.crc[I], P.cpirc[I], P.crci[I], f, g);
    S.fc[p] = f;
    S.gc[p] = g;
  }
  __syncwarp();
  return true;
}

// ------------------------------------------------------------------------------------ symm
template <int NEK, int NZK, bool GEN>
__global__ void __launch_bounds__(128) symm_kernel(const __grid_constant__ PotParams P, int a0, int natoms, int cap,
                                                   const int* __restrict__ type, const int* __restrict__ nb_j,
                                                   const unsigned char* __restrict__ nb_t, const float4* __restrict__ nb_r,
                                                   const int* __restrict__ nb_cnt, float* __restrict__ G, int gstride,
                                                   float* __restrict__ mom, int mstride, const int* __restrict__ order) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int i = a0 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= a0 + natoms) return;
  if (order) i = order[i];  // whole structures, the densest first
  const WarpSmem S = carve(smem + warp * warp_smem_floats(cap, NEK, false), cap, NEK, false);
  const int I = clamp_type(type[i], P.ntypes);
  const int n = stage_neighbors(S, i, cap, P.ntypes, type, nb_j, nb_t, nb_r, nb_cnt);
  const bool cc = cutoff_cache(S, P, I, n);
  float* Gi = G + (size_t)i * gstride;
  for (int k = P.nin[I] + lane; k < gstride; k += 32) Gi[k] = 0.f;

  // ---- radial: G2 of neighbour type J (BasisR::symm, basis_radial.cpp:302-310); functions in
  // groups of four, lanes over the type's neighbours
  for (int J = 0; J < P.ntypes; ++J) {
    const RadialP& R = P.rad[I][J];
    const int p0 = S.toff[J], p1 = S.toff[J + 1];
    for (int f0 = 0; f0 < R.n; f0 += 4) {
      float rs[4], eta[4], acc[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const bool on = f0 + k < R.n;
        rs[k] = on ? R.rs[f0 + k] : 0.f;
        eta[k] = on ? R.eta[f0 + k] : 0.f;
        acc[k] = 0.f;
      }
      for (int p = p0 + lane; p < p1; p += 32) {
        const float d = S.d[p];
        float fc, gc;
        if (cc) fc = S.fc[p];
        else cutoff_fg(R.cut, d, R.rc, R.pirc, R.rci, fc, gc);
        if (R.phi == RAD_GAUSSIAN) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float x = d - rs[k];
            acc[k] = fmaf(__expf(-eta[k] * x * x), fc, acc[k]);
          }
        } else {
#pragma unroll
          for (int k = 0; k < 4; ++k) acc[k] = fmaf(radial_value(R.phi, eta[k], rs[k], d), fc, acc[k]);
        }
      }
      {
        const float v = warp_sum4(acc[0], acc[1], acc[2], acc[3]);
        const int k = (lane >> 3) & 3;
        if ((lane & 7) == 0 && f0 + k < R.n) Gi[R.off + f0 + k] = v * R.norm;
      }
    }
  }

  // ---- angular blocks (J <= K): G4
  const bool msh = P.msh[I] != 0;
  if (msh) symm_mom_shared<GEN>(S, P, I, cc, mom ? mom + (size_t)i * mstride : nullptr, Gi);
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0) continue;
      const int j0 = S.toff[J], nJ = S.toff[J + 1] - j0;
      const int k0 = S.toff[K], nK = S.toff[K + 1] - k0;
      if (A.mom) {
        if (!msh)
          symm_mom_block<GEN>(S, A, P.atab, cc, J == K, j0, nJ, k0, nK, mom ? mom + (size_t)i * mstride + A.moff : nullptr, Gi);
        if (!A.top) continue;
        __syncwarp();
      }
      block_pair_factors<GEN>(S, A, j0, j0 + nJ, cap, true);
      if (K != J) block_pair_factors<GEN>(S, A, k0, k0 + nK, cap, true);
      __syncwarp();
      if constexpr (GEN) {
        if (A.fn) {
          symm_block_fn(S, A, P.atab + A.tab, make_sched(J, K, j0, nJ, k0, nK), Gi);
          __syncwarp();
          continue;
        }
      }
      run_block<false, NEK, NZK, GEN>(S, A, make_sched(J, K, j0, nJ, k0, nK), cap);
      __syncwarp();
      for (int f = lane; f < A.n; f += 32) {
        const int cell = (int)P.atab[A.tab + f];
        if (!A.top || cell % NZ_MAX == A.nz - 1) Gi[A.off + f] = A.norm * S.scratch[cell];
      }
      __syncwarp();
    }
}

// ------------------------------------------------------------------------------------ force
template <int NEK, int NZK, bool GEN>
__global__ void __launch_bounds__(128, 5) force_kernel(const __grid_constant__ PotParams P, int a0, int natoms, int cap,
                                                    const int* __restrict__ type, const int* __restrict__ nb_j,
                                                    const unsigned char* __restrict__ nb_t, const float4* __restrict__ nb_r,
                                                    const int* __restrict__ nb_cnt, const float* __restrict__ dEdG, int gstride,
                                                    const float* __restrict__ mom, int mstride, const int* __restrict__ nb_code,
                                                    long long* __restrict__ facc, const int* __restrict__ order,
                                                    int* __restrict__ status) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int i = a0 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= a0 + natoms) return;
  if (order) i = order[i];  // whole structures, the densest first
  const bool kx = GEN && P.kx;  // a compile-time false in the GAUSS-only instances
  const WarpSmem S = carve(smem + warp * warp_smem_floats(cap, NEK, kx, gstride + mstride), cap, NEK, kx);
  float* gm = S.gi + gstride;  // the centre's stored moments
  const int I = clamp_type(type[i], P.ntypes);
  // the centre's dE/dG row (read by every block) and moment row into shared memory, in flight
  // while the neighbours are staged (rows are 16-byte aligned: gstride and mstride are
  // multiples of four floats)
  for (int k = 4 * lane; k < P.nin[I]; k += 128) cp_async16(S.gi + k, dEdG + (size_t)i * gstride + k);
  cp_async_commit();
  if (mstride > 0)
    for (int k = 4 * lane; k < mstride; k += 128) cp_async16(gm + k, mom + (size_t)i * mstride + k);
  cp_async_commit();
  const int n = stage_neighbors(S, i, cap, P.ntypes, type, nb_j, nb_t, nb_r, nb_cnt);
  const bool cc = cutoff_cache(S, P, I, n);
  cp_async_wait<1>();  // the dE/dG row
  __syncwarp();
  const float* gi = S.gi;

  // ---- radial chain rule: W_p = BasisR::force(d) * u_p (basis_radial.cpp:371-380, nnp.cpp:441-446);
  // functions in groups of four (independent exponentials in flight), GAUSSIAN inline
  for (int J = 0; J < P.ntypes; ++J) {
    const RadialP& R = P.rad[I][J];
    const float* __restrict__ sJ = gi + R.off;
    for (int p = S.toff[J] + lane; p < S.toff[J + 1]; p += 32) {
      const float d = S.d[p];
      float fc, gc;
      if (cc) {
        fc = S.fc[p];
        gc = S.gc[p];
      } else {
        cutoff_fg(R.cut, d, R.rc, R.pirc, R.rci, fc, gc);
      }
      float amp = 0.f;
      if (R.phi == RAD_GAUSSIAN) {
#pragma unroll 1
        for (int f0 = 0; f0 < R.n; f0 += 4) {
          float t[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int f = min(f0 + k, R.n - 1);
            const float eta = R.eta[f], x = d - R.rs[f];
            const float w = (f0 + k < R.n) ? sJ[f] : 0.f;
            t[k] = w * __expf(-eta * x * x) * fmaf(-2.0f * eta * x, fc, gc);
          }
          amp -= (t[0] + t[1]) + (t[2] + t[3]);
        }
      } else {
#pragma unroll 1
        for (int f = 0; f < R.n; ++f) amp -= sJ[f] * radial_force_term(R.phi, R.eta[f], R.rs[f], d, fc, gc);
      }
      amp *= R.norm;
      S.wx[p] = amp * S.ux[p];
      S.wy[p] = amp * S.uy[p];
      S.wz[p] = amp * S.uz[p];
    }
  }
  __syncwarp();

  cp_async_wait<0>();  // the moment row
  __syncwarp();

  // ---- angular chain rule
  const bool msh = P.msh[I] != 0;
  if (msh) force_mom_shared<GEN>(S, P, I, cc, gm, gi);
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0) continue;
      const int j0 = S.toff[J], nJ = S.toff[J + 1] - j0;
      const int k0 = S.toff[K], nK = S.toff[K + 1] - k0;
      if (nJ == 0 || nK == 0 || (J == K && nJ < 2)) continue;
      if (A.mom) {
        if (!msh) force_mom_block<GEN>(S, A, P.atab, cc, J == K, j0, nJ, k0, nK, gm + A.moff, gi);
        if (!A.top) continue;
        __syncwarp();
      }
      block_pair_factors<GEN>(S, A, j0, j0 + nJ, cap, false);
      if (K != J) block_pair_factors<GEN>(S, A, k0, k0 + nK, cap, false);
      if constexpr (GEN) {
        if (A.fn) {
          __syncwarp();
          force_block_fn(S, A, P.atab + A.tab, make_sched(J, K, j0, nJ, k0, nK), gi);
          __syncwarp();
          continue;
        }
      }
      // dE/dG on the function grid, one lane per grid cell (duplicates of a cell add up in file order)
      for (int c = lane; c < NE_MAX * NL * NZ_MAX; c += 32) {
        float v = 0.f;
        for (int f = 0; f < A.n; ++f)
          if (A.gidx[f] == c) v += gi[A.off + f];
        S.scratch[c] = v;
      }
      __syncwarp();
      run_block<true, NEK, NZK, GEN>(S, A, make_sched(J, K, j0, nJ, k0, nK), cap);
      __syncwarp();
    }

  // NNP::force (nnp.cpp:466-478): the centre gains every slot's vector and the neighbour of a
  // minimum-image slot loses it, summed in fixed point (each slot rounded once; the neighbours'
  // adds arrive from other warps in any order, and integer sums do not depend on it)
  long long ox = 0, oy = 0, oz = 0;
  bool bad = false;
  for (int p = lane; p < n; p += 32) {
    const float wx = S.wx[p], wy = S.wy[p], wz = S.wz[p];
    // a NaN or infinity propagates through the sum; the host discards the call's results
    bad = bad || !(fabsf(wx) + fabsf(wy) + fabsf(wz) < FORCE_MAX_ABS);
    const long long qx = force_fixed(wx), qy = force_fixed(wy), qz = force_fixed(wz);
    ox += qx;
    oy += qy;
    oz += qz;
    const size_t g = (size_t)i * cap + S.orig[p];
    if (code_min(nb_code[g])) {
      long long* fj = facc + 3 * (size_t)nb_j[g];
      red_add(fj, -qx);
      red_add(fj + 1, -qy);
      red_add(fj + 2, -qz);
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&status[ST_ERROR], ERR_FORCE_RANGE);
  ox = warp_sum_ll(ox);
  oy = warp_sum_ll(oy);
  oz = warp_sum_ll(oz);
  if (lane < 3) red_add(facc + 3 * (size_t)i + lane, lane == 0 ? ox : (lane == 1 ? oy : oz));
}

// ------------------------------------------------------------------------------------ tangent
// The force term of the force trainer's loss (loss of NNPTEF::error, src/nnp/nnptef.cpp:1043-1135)
// reaches the network parameters through dE/dG: with t_k = dloss/dF_k, the descriptor-space
// weights are u_if = sum_k t_k . dF_k/d(dE/dG_if), F as NNP::force builds it (nnp.cpp:416-482).
// Per neighbour slot p of centre i, the neighbour's tangent counts only for the minimum image:
// delta_p = t_i - (min_p ? t_j : 0).  Then for a radial function u_f = -sum_p dG_f/dr (delta_p . u_p)
// and for an angular one u_f = -sum_triplets (dG_f/dcos dcos + dG_f/dr_a (delta_a . u_a) +
// dG_f/dr_b (delta_b . u_b)), dcos = delta_a.(u_b - cos u_a)/r_a + delta_b.(u_a - cos u_b)/r_b:
// minus the tangent of the descriptors along the masked displacement field.  Blocks that are not
// GAUSS moment blocks take the triplet loop here, all families through ang_h.
// Moment blocks of the GAUSS family take the tangent through their moments: G_f = sum_c T[f][c] V[c]
// with V[e][n] = <M^J_n, M^K_n> (half of it less the j == k terms for J == K), so along the
// displacements dG_f = sum_c T[f][c] dV[c], dV = <dM^J_n, M^K_n> + <M^J_n, dM^K_n> (halved, less
// half the diagonal's tangent, for J == K).  Per slot, with dd = u . delta and du = (delta - dd u)/r,
// the pair weight w = exp(-ie r^alpha) f moves by dw = exp(-ie r^alpha) (f' - ie alpha r^(alpha-1) f) dd
// and the monomial u^(a,b,c) by a u^(a-1,b,c) du_x + b u^(a,b-1,c) du_y + c u^(a,b,c-1) du_z.
// Lane groups as in build_moments; M as build_moments writes it, dM likewise, and
// dDg[(set*ne + e)*(MOM_N+1) + n] the tangent of sum w^2 |u|^2n.
static __device__ void build_moment_tangents(const WarpSmem& S, const AngP& A, bool cc, int nsets, int lo0, int hi0, int lo1, int hi1,
                                      float* __restrict__ M, float* __restrict__ dM, float* __restrict__ dDg) {
  const int lane = threadIdx.x & 31;
  const int pairs = nsets * A.ne;
  int L = 32;
  while (L * pairs > 32) L >>= 1;
  const int grp = lane / L, sub = lane % L;
  const bool active = grp < pairs;
  const int set = active ? grp / A.ne : 0, e = active ? grp % A.ne : 0;
  const int lo = active ? (set ? lo1 : lo0) : 0, hi = active ? (set ? hi1 : hi0) : 0;
  float acc[MOM_C], dacc[MOM_C], ddg[MOM_N + 1];
#pragma unroll
  for (int r = 0; r < MOM_C; ++r) {
    acc[r] = 0.f;
    dacc[r] = 0.f;
  }
#pragma unroll
  for (int n = 0; n <= MOM_N; ++n) ddg[n] = 0.f;
  const float ie = A.ietap[e];
  for (int p = lo + sub; p < hi; p += L) {
    const float d = S.d[p], ux = S.ux[p], uy = S.uy[p], uz = S.uz[p], inv = S.inv[p];
    const float tx = S.wx[p], ty = S.wy[p], tz = S.wz[p];
    float f, g;
    if (cc) {
      f = S.fc[p];
      g = S.gc[p];
    } else {
      cutoff_fg(A.cut, d, A.rc, A.pirc, A.rci, f, g);
    }
    const float h = __expf(-ie * powi(d, A.alpha));
    const float w = h * f;
    const float dd = tx * ux + ty * uy + tz * uz;
    const float dw = h * (g - ie * (float)A.alpha * powi(d, A.alpha - 1) * f) * dd;
    const float dux = (tx - dd * ux) * inv, duy = (ty - dd * uy) * inv, duz = (tz - dd * uz) * inv;
    float px[MOM_N + 1], py[MOM_N + 1], pz[MOM_N + 1];
    px[0] = 1.f;
    py[0] = 1.f;
    pz[0] = 1.f;
#pragma unroll
    for (int k = 1; k <= MOM_N; ++k) {
      px[k] = px[k - 1] * ux;
      py[k] = py[k - 1] * uy;
      pz[k] = pz[k - 1] * uz;
    }
#pragma unroll
    for (int n = 0; n <= MOM_N; ++n)
#pragma unroll
      for (int a = n; a >= 0; --a)
#pragma unroll
        for (int b = n - a; b >= 0; --b) {
          const int c = n - a - b;
          const float yz = py[b] * pz[c];
          const float m = px[a] * yz;
          float dm = 0.f;
          if (a > 0) dm = fmaf((float)a * px[a - 1] * yz, dux, dm);
          if (b > 0) dm = fmaf((float)b * px[a] * (py[b - 1] * pz[c]), duy, dm);
          if (c > 0) dm = fmaf((float)c * px[a] * (py[b] * pz[c - 1]), duz, dm);
          acc[mom_idx(a, b, c)] = fmaf(w, m, acc[mom_idx(a, b, c)]);
          dacc[mom_idx(a, b, c)] = fmaf(dw, m, fmaf(w, dm, dacc[mom_idx(a, b, c)]));
        }
    // d(w^2 |u|^2n) = 2 w dw |u|^2n + 2 n w^2 |u|^2(n-1) (u . du)
    const float u2 = ux * ux + uy * uy + uz * uz, udu = ux * dux + uy * duy + uz * duz;
    float un = 1.f, unm = 0.f;
#pragma unroll
    for (int n = 0; n <= MOM_N; ++n) {
      ddg[n] += 2.0f * w * (dw * un + (float)n * w * unm * udu);
      unm = un;
      un *= u2;
    }
  }
  for (int o = L >> 1; o > 0; o >>= 1) {
#pragma unroll
    for (int r = 0; r < MOM_C; ++r) {
      acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
      dacc[r] += __shfl_xor_sync(0xffffffffu, dacc[r], o);
    }
#pragma unroll
    for (int n = 0; n <= MOM_N; ++n) ddg[n] += __shfl_xor_sync(0xffffffffu, ddg[n], o);
  }
  if (active && sub == 0) {
#pragma unroll
    for (int r = 0; r < MOM_C; ++r) {
      M[(set * A.ne + e) * MOM_C + r] = acc[r];
      dM[(set * A.ne + e) * MOM_C + r] = dacc[r];
    }
#pragma unroll
    for (int n = 0; n <= MOM_N; ++n) dDg[(set * A.ne + e) * (MOM_N + 1) + n] = ddg[n];
  }
}

// dV of one (J, K) pair of moment sets for width e and degree n
static __device__ __forceinline__ float mom_tangent_inner(const float* __restrict__ MJ, const float* __restrict__ dMJ, const float* __restrict__ MK,
                                                   const float* __restrict__ dMK, int n, bool same, float ddiag) {
  float s = 0.f;
  for (int r = mom_off(n); r < mom_off(n + 1); ++r) s = fmaf(c_mom_mult[r], fmaf(dMJ[r], MK[r], MJ[r] * dMK[r]), s);
  return same ? 0.5f * (s - ddiag) : s;
}

// u_f = -dG_f of one GAUSS moment block (its own moments)
static __device__ void tangent_mom_block(const WarpSmem& S, const AngP& A, const float* __restrict__ atab, bool cc, bool same, int j0, int nJ,
                                  int k0, int nK, float* __restrict__ Ui) {
  const int lane = threadIdx.x & 31;
  const int ns = same ? 1 : 2, nec = A.ne * MOM_C;
  float* MS = S.ex;               // [set][e][MOM_C]
  float* dMS = S.ex + ns * nec;   // [set][e][MOM_C]
  float* dDg = S.ex + 2 * ns * nec;  // [set][e][MOM_N+1]
  build_moment_tangents(S, A, cc, ns, j0, j0 + nJ, k0, k0 + nK, MS, dMS, dDg);
  __syncwarp();
  float* dV = S.scratch;
  if (lane < A.ne * (MOM_N + 1)) {
    const int e = lane / (MOM_N + 1), n = lane % (MOM_N + 1);
    const int kof = (same ? 0 : nec) + e * MOM_C;
    dV[lane] = mom_tangent_inner(MS + e * MOM_C, dMS + e * MOM_C, MS + kof, dMS + kof, n, same, dDg[e * (MOM_N + 1) + n]);
  }
  __syncwarp();
  const int w = A.ne * (MOM_N + 1);
  const float* __restrict__ T = atab + A.tab + A.n;
  for (int f = lane; f < A.n; f += 32) {
    float v = 0.f;
    for (int c = 0; c < w; ++c) v = fmaf(T[f * w + c], dV[c], v);
    Ui[A.off + f] = -v;
  }
  __syncwarp();
}

// u_f = -dG_f of every moment block of centre type I from the shared moments (all GAUSS)
static __device__ void tangent_mom_shared(const WarpSmem& S, const PotParams& P, int I, bool cc, float* __restrict__ Ui) {
  const int lane = threadIdx.x & 31;
  const AngP& R = P.ang[I][P.mrep[I]];
  const int ns = P.mns[I], ne = R.ne, nec = ne * MOM_C;
  const int sp0 = P.msp[I][0], sp1 = ns > 1 ? P.msp[I][1] : sp0;
  float* MS = S.ex;
  float* dMS = S.ex + ns * nec;
  float* dDg = S.ex + 2 * ns * nec;
  build_moment_tangents(S, R, cc, ns, S.toff[sp0], S.toff[sp0 + 1], S.toff[sp1], S.toff[sp1 + 1], MS, dMS, dDg);
  __syncwarp();
  int pk = 0, nk = 0, nb = 0, nf = 0;
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0 || !A.mom || nb >= 3) continue;
      pk |= (J | (K << 2)) << (4 * nb);
      nk |= A.n << (8 * nb);
      nf += A.n;
      ++nb;
    }
  const int w = ne * (MOM_N + 1);
  float* dV = S.scratch;
  for (int t = lane; t < nb * w; t += 32) {
    const int k = t / w, c = t - k * w, e = c / (MOM_N + 1), n = c - e * (MOM_N + 1);
    const int J = (pk >> (4 * k)) & 3, K = (pk >> (4 * k + 2)) & 3;
    const int oJ = mom_set(P, I, J) * nec + e * MOM_C, oK = mom_set(P, I, K) * nec + e * MOM_C;
    dV[t] = mom_tangent_inner(MS + oJ, dMS + oJ, MS + oK, dMS + oK, n, J == K, dDg[(mom_set(P, I, J) * ne + e) * (MOM_N + 1) + n]);
  }
  __syncwarp();
  for (int t = lane; t < nf; t += 32) {
    int k = 0, f = t;
    while (k + 1 < nb && f >= ((nk >> (8 * k)) & 255)) {
      f -= (nk >> (8 * k)) & 255;
      ++k;
    }
    const AngP& A = P.ang[I][lidx((pk >> (4 * k)) & 3, (pk >> (4 * k + 2)) & 3)];
    const float* __restrict__ T = P.atab + A.tab + A.n + f * w;
    float v = 0.f;
    for (int c = 0; c < w; ++c) v = fmaf(T[c], dV[k * w + c], v);
    Ui[A.off + f] = -v;
  }
  __syncwarp();
}

template <int NE, int NZ>
__device__ void tangent_block(const WarpSmem& S, const AngP& A, const Sched& sc, int cap) {
  const int lane = threadIdx.x & 31;
  float acc[NE][NL][NZ];
#pragma unroll
  for (int e = 0; e < NE; ++e)
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
      for (int m = 0; m < NZ; ++m) acc[e][l][m] = 0.f;
  const bool sum = ang_sum_family(A.phi);
  const float lam0 = A.lam[0], lam1 = A.lam[1];
  for (int q = 0; q * 32 < sc.nown; ++q) {
    const int x = q * 32 + lane;
    const int a = sc.xb + min(x, sc.nown - 1);
    const float uax = S.ux[a], uay = S.uy[a], uaz = S.uz[a], ia = S.inv[a];
    const float dax = S.wx[a], day = S.wy[a], daz = S.wz[a];
    const float fa = S.fc[a], ga = S.gc[a], pa = S.dpa[a];
    const float dda = dax * uax + day * uay + daz * uaz;
    for (int dd = sc.d0; dd <= sc.d1; ++dd) {
      const int nx = (sc.tri && 2 * dd == sc.nJ) ? (sc.nJ >> 1) : sc.nown;
      if (x < nx) {
        int y = x + dd;
        if (y >= sc.mod) y -= sc.mod;
        const int b = sc.yb + y;
        const float ubx = S.ux[b], uby = S.uy[b], ubz = S.uz[b], ib = S.inv[b];
        const float dbx = S.wx[b], dby = S.wy[b], dbz = S.wz[b];
        const float fb = S.fc[b], gb = S.gc[b], pb = S.dpa[b];
        const float cs = uax * ubx + uay * uby + uaz * ubz;
        const float ddb = dbx * ubx + dby * uby + dbz * ubz;
        const float xa = dax * ubx + day * uby + daz * ubz, xb = dbx * uax + dby * uay + dbz * uaz;
        const float dcos = (xa - cs * dda) * ia + (xb - cs * ddb) * ib;
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
#pragma unroll
        for (int e = 0; e < NE; ++e) {
          if (e >= A.ne) break;
          float R, ka, kb;
          if (sum) {
            R = ang_h(A.phi, A.ietap[e] * (S.ex[a] + S.ex[b]), ka);
            kb = ka;
          } else {
            R = S.ex[e * cap + a] * S.ex[e * cap + b];
            ka = S.kx[e * cap + a];
            kb = S.kx[e * cap + b];
          }
          const float ie = A.ietap[e];
          const float td = R * (fb * (ga - ie * ka * pa) * dda + fa * (gb - ie * kb * pb) * ddb);
          const float tc = 0.5f * fa * fb * R * dcos;
          const float tc0 = lam0 * tc, tc1 = lam1 * tc;
#pragma unroll
          for (int m = 0; m < NZ; ++m) {
            acc[e][0][m] = fmaf(qd[0][m], tc0, fmaf(p[0][m], td, acc[e][0][m]));
            acc[e][1][m] = fmaf(qd[1][m], tc1, fmaf(p[1][m], td, acc[e][1][m]));
          }
        }
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

template <int NEK, int NZK>
__global__ void __launch_bounds__(128) tangent_kernel(const __grid_constant__ PotParams P, int a0, int natoms, int cap,
                                                      const int* __restrict__ type, const int* __restrict__ nb_j,
                                                      const unsigned char* __restrict__ nb_t, const float4* __restrict__ nb_r,
                                                      const int* __restrict__ nb_code, const int* __restrict__ nb_cnt,
                                                      const float4* __restrict__ tvec, float* __restrict__ U, int gstride) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = a0 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= a0 + natoms) return;
  const WarpSmem S = carve(smem + warp * warp_smem_floats(cap, NEK, true), cap, NEK, true);
  const int I = clamp_type(type[i], P.ntypes);
  const int n = stage_neighbors(S, i, cap, P.ntypes, type, nb_j, nb_t, nb_r, nb_cnt);
  const bool cc = cutoff_cache(S, P, I, n);
  // masked displacement of each staged slot
  const float4 ti = tvec[i];
  for (int p = lane; p < n; p += 32) {
    const size_t g = (size_t)i * cap + S.orig[p];
    const bool mn = code_min(nb_code[g]);
    const float4 tj = mn ? tvec[nb_j[g]] : make_float4(0.f, 0.f, 0.f, 0.f);
    S.wx[p] = ti.x - tj.x;
    S.wy[p] = ti.y - tj.y;
    S.wz[p] = ti.z - tj.z;
  }
  __syncwarp();
  float* Ui = U + (size_t)i * gstride;
  for (int k = P.nin[I] + lane; k < gstride; k += 32) Ui[k] = 0.f;

  // radial: u_f = -norm sum_p dG_f/dr (delta_p . u_p), dG_f/dr per function as BasisR::force uses it
  for (int J = 0; J < P.ntypes; ++J) {
    const RadialP& R = P.rad[I][J];
    const int p0 = S.toff[J], p1 = S.toff[J + 1];
    for (int f0 = 0; f0 < R.n; f0 += 4) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      for (int p = p0 + lane; p < p1; p += 32) {
        const float d = S.d[p];
        float fc, gc;
        if (cc) { fc = S.fc[p]; gc = S.gc[p]; }
        else cutoff_fg(R.cut, d, R.rc, R.pirc, R.rci, fc, gc);
        const float proj = S.wx[p] * S.ux[p] + S.wy[p] * S.uy[p] + S.wz[p] * S.uz[p];
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (f0 + k < R.n) acc[k] = fmaf(radial_force_term(R.phi, R.eta[f0 + k], R.rs[f0 + k], d, fc, gc), proj, acc[k]);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float v = warp_sum(acc[k]);
        if (lane == 0 && f0 + k < R.n) Ui[R.off + f0 + k] = -v * R.norm;
      }
    }
  }
  __syncwarp();

  // angular: GAUSS moment blocks through their moments (a split block's top level, and every
  // other block, through the triplet loop)
  const bool msh = P.msh[I] != 0;
  bool mgauss = true;  // every moment block of this centre type is GAUSS
  for (int q = 0; q < P.ntypes * (P.ntypes + 1) / 2; ++q)
    if (P.ang[I][q].n > 0 && P.ang[I][q].mom && P.ang[I][q].phi != ANG_GAUSS) mgauss = false;
  if (msh && mgauss) tangent_mom_shared(S, P, I, cc, Ui);
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0) continue;
      const int j0 = S.toff[J], nJ = S.toff[J + 1] - j0;
      const int k0 = S.toff[K], nK = S.toff[K + 1] - k0;
      const bool by_mom = A.mom && (msh ? mgauss : A.phi == ANG_GAUSS);
      if (by_mom) {
        if (!msh) tangent_mom_block(S, A, P.atab, cc, J == K, j0, nJ, k0, nK, Ui);
        if (!A.top) continue;
        __syncwarp();
      }
      block_pair_factors<true>(S, A, j0, j0 + nJ, cap, false);
      if (K != J) block_pair_factors<true>(S, A, k0, k0 + nK, cap, false);
      __syncwarp();
      tangent_block<NEK, NZK>(S, A, make_sched(J, K, j0, nJ, k0, nK), cap);
      __syncwarp();
      for (int f = lane; f < A.n; f += 32) {
        const int cell = (int)P.atab[A.tab + f];
        if (!by_mom || cell % NZ_MAX == A.nz - 1) Ui[A.off + f] = -A.norm * S.scratch[cell];
      }
      __syncwarp();
    }
}


// the force kernels of potentials with a non-GAUSS angular family (descriptor_force_gen.cu)
int launch_force_gen(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st);
size_t force_smem_bytes(int cap, int ne, int warps, bool kx, int gstride);

}  // namespace nnpgpu
