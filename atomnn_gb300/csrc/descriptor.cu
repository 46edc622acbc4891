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

// ------------------------------------------------------------------------------------ symm
template <int NE, int NZ>
__global__ void __launch_bounds__(128) symm_kernel(const __grid_constant__ PotParams P, int a0, int natoms, int cap,
                                                   const int* __restrict__ type, const int* __restrict__ nb_j,
                                                   const float4* __restrict__ nb_r, const int* __restrict__ nb_cnt,
                                                   float* __restrict__ G, int gstride) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = a0 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= a0 + natoms) return;
  const WarpSmem S = carve(smem + warp * warp_smem_floats(cap, NE), cap, NE);
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

  // ---- angular blocks (J <= K): G4 (BasisA::symm, basis_angular.cpp:406-421)
  for (int J = 0; J < P.ntypes; ++J)
    for (int K = J; K < P.ntypes; ++K) {
      const AngP& A = P.ang[I][lidx(J, K)];
      if (A.n == 0) continue;
      const int j0 = S.toff[J], nJ = S.toff[J + 1] - j0;
      const int k0 = S.toff[K], nK = S.toff[K + 1] - k0;
      block_pair_factors(S, A, j0, j0 + nJ, cap, true);
      if (K != J) block_pair_factors(S, A, k0, k0 + nK, cap, true);
      __syncwarp();
      float acc[NE][NL][NZ];
#pragma unroll
      for (int e = 0; e < NE; ++e)
#pragma unroll
        for (int l = 0; l < NL; ++l)
#pragma unroll
          for (int m = 0; m < NZ; ++m) acc[e][l][m] = 0.f;
      const bool tri = (J == K);
      int xb, nown, yb, mod, d0, d1;
      if (tri) { xb = j0; yb = j0; nown = nJ; mod = nJ; d0 = 1; d1 = nJ / 2; }
      else if (nJ <= nK) { xb = j0; nown = nJ; yb = k0; mod = nK; d0 = 0; d1 = nK - 1; }
      else { xb = k0; nown = nK; yb = j0; mod = nJ; d0 = 0; d1 = nJ - 1; }
      if (nown == 0) d1 = d0 - 1;
      const float lam0 = A.lam[0], lam1 = A.lam[1];
      for (int dd = d0; dd <= d1; ++dd) {
        const int nx = (tri && 2 * dd == nJ) ? (nJ >> 1) : nown;
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
          if (q * 32 >= nx) break;
          const int x = q * 32 + lane;
          if (x < nx) {
            int y = x + dd;
            if (y >= mod) y -= mod;
            const int a = xb + x, b = yb + y;
            const float cs = S.ux[a] * S.ux[b] + S.uy[a] * S.uy[b] + S.uz[a] * S.uz[b];
            float p[NL][NZ];
#pragma unroll
            for (int l = 0; l < NL; ++l) {
              p[l][0] = fabsf(0.5f * (1.0f + (l == 0 ? lam0 : lam1) * cs));
#pragma unroll
              for (int m = 1; m < NZ; ++m) p[l][m] = p[l][m - 1] * p[l][m - 1];
            }
#pragma unroll
            for (int e = 0; e < NE; ++e)
              if (e < A.ne) {
                const float E = S.ex[e * cap + a] * S.ex[e * cap + b];
#pragma unroll
                for (int l = 0; l < NL; ++l)
#pragma unroll
                  for (int m = 0; m < NZ; ++m)
                    if (m < A.nz) acc[e][l][m] = fmaf(p[l][m], E, acc[e][l][m]);
              }
          }
        }
      }
      // reduce the grid and scatter it to the block's file functions
#pragma unroll
      for (int e = 0; e < NE; ++e)
#pragma unroll
        for (int l = 0; l < NL; ++l)
#pragma unroll
          for (int m = 0; m < NZ; ++m) {
            const float v = warp_sum(acc[e][l][m]);
            if (lane == 0) S.scratch[(e * NL + l) * NZ_MAX + m] = v;
          }
      __syncwarp();
      for (int f = lane; f < A.n; f += 32) Gi[A.off + f] = A.norm * S.scratch[A.gidx[f]];
      __syncwarp();
    }
}

// ------------------------------------------------------------------------------------ force
template <int NE, int NZ>
__global__ void __launch_bounds__(128) force_kernel(const __grid_constant__ PotParams P, int a0, int natoms, int cap,
                                                    const int* __restrict__ type, const int* __restrict__ nb_j,
                                                    const float4* __restrict__ nb_r, const int* __restrict__ nb_cnt,
                                                    const float* __restrict__ dEdG, int gstride, float4* __restrict__ W) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = a0 + blockIdx.x * (blockDim.x >> 5) + warp;
  if (i >= a0 + natoms) return;
  const WarpSmem S = carve(smem + warp * warp_smem_floats(cap, NE), cap, NE);
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

  // ---- angular chain rule (BasisA::force, basis_angular.cpp:456-507; nnp.cpp:448-479)
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
      float sg[NE][NL][NZ];
#pragma unroll
      for (int e = 0; e < NE; ++e)
#pragma unroll
        for (int l = 0; l < NL; ++l)
#pragma unroll
          for (int m = 0; m < NZ; ++m) sg[e][l][m] = S.scratch[(e * NL + l) * NZ_MAX + m];
      float ie[NE];
#pragma unroll
      for (int e = 0; e < NE; ++e) ie[e] = (e < A.ne) ? A.ietap[e] : 0.f;
      const float lam0 = A.lam[0], lam1 = A.lam[1];
      const float hn = -0.5f * A.norm, nn = -A.norm;

      const bool tri = (J == K);
      int xb, nown, yb, mod, d0, d1;
      if (tri) { xb = j0; yb = j0; nown = nJ; mod = nJ; d0 = 1; d1 = nJ / 2; }
      else if (nJ <= nK) { xb = j0; nown = nJ; yb = k0; mod = nK; d0 = 0; d1 = nK - 1; }
      else { xb = k0; nown = nK; yb = j0; mod = nJ; d0 = 0; d1 = nJ - 1; }
      float wo[QMAX][3];
#pragma unroll
      for (int q = 0; q < QMAX; ++q) wo[q][0] = wo[q][1] = wo[q][2] = 0.f;
      for (int dd = d0; dd <= d1; ++dd) {
        const int nx = (tri && 2 * dd == nJ) ? (nJ >> 1) : nown;
#pragma unroll
        for (int q = 0; q < QMAX; ++q) {
          if (q * 32 >= nx) break;
          const int x = q * 32 + lane;
          if (x < nx) {
            int y = x + dd;
            if (y >= mod) y -= mod;
            const int a = xb + x, b = yb + y;
            const float uax = S.ux[a], uay = S.uy[a], uaz = S.uz[a];
            const float ubx = S.ux[b], uby = S.uy[b], ubz = S.uz[b];
            const float cs = uax * ubx + uay * uby + uaz * ubz;
            float p[NL][NZ], qd[NL][NZ];
#pragma unroll
            for (int l = 0; l < NL; ++l) {
              p[l][0] = fabsf(0.5f * (1.0f + (l == 0 ? lam0 : lam1) * cs));
              qd[l][0] = 1.0f;
#pragma unroll
              for (int m = 1; m < NZ; ++m) {
                qd[l][m] = 2.0f * qd[l][m - 1] * p[l][m - 1];
                p[l][m] = p[l][m - 1] * p[l][m - 1];
              }
            }
            float Q = 0.f, Q2 = 0.f, Pp = 0.f;
#pragma unroll
            for (int e = 0; e < NE; ++e)
              if (e < A.ne) {
                const float E = S.ex[e * cap + a] * S.ex[e * cap + b];
                float qe = 0.f, pe = 0.f;
#pragma unroll
                for (int l = 0; l < NL; ++l) {
                  float ql = 0.f, pl = 0.f;
#pragma unroll
                  for (int m = 0; m < NZ; ++m) {
                    ql = fmaf(sg[e][l][m], p[l][m], ql);
                    pl = fmaf(sg[e][l][m], qd[l][m], pl);
                  }
                  qe += ql;
                  pe = fmaf(l == 0 ? lam0 : lam1, pl, pe);
                }
                Q = fmaf(E, qe, Q);
                Q2 = fmaf(E * ie[e], qe, Q2);
                Pp = fmaf(E, pe, Pp);
              }
            const float fa = S.fc[a], fb = S.fc[b];
            const float phi = hn * fa * fb * Pp;
            const float eta0 = nn * fb * (S.gc[a] * Q - S.dpa[a] * Q2);
            const float eta1 = nn * fa * (S.gc[b] * Q - S.dpa[b] * Q2);
            const float ia = S.inv[a], ib = S.inv[b];
            const float Aa = -phi * cs * ia + eta0, Ba = phi * ia;
            const float Ab = -phi * cs * ib + eta1, Bb = phi * ib;
            wo[q][0] += Aa * uax + Ba * ubx;
            wo[q][1] += Aa * uay + Ba * uby;
            wo[q][2] += Aa * uaz + Ba * ubz;
            S.wx[b] += Ab * ubx + Bb * uax;
            S.wy[b] += Ab * uby + Bb * uay;
            S.wz[b] += Ab * ubz + Bb * uaz;
          }
          __syncwarp();
        }
      }
#pragma unroll
      for (int q = 0; q < QMAX; ++q) {
        const int x = q * 32 + lane;
        if (x < nown) {
          S.wx[xb + x] += wo[q][0];
          S.wy[xb + x] += wo[q][1];
          S.wz[xb + x] += wo[q][2];
        }
      }
      __syncwarp();
    }

  // write the per-slot contributions in the list's own slot order
  float4* Wi = W + (size_t)i * cap;
  for (int p = lane; p < n; p += 32) Wi[S.orig[p]] = make_float4(S.wx[p], S.wy[p], S.wz[p], 0.f);
}

size_t symm_smem_bytes(int cap, int ne, int warps) { return sizeof(float) * warp_smem_floats(cap, ne) * warps; }
size_t force_smem_bytes(int cap, int ne, int warps) { return sizeof(float) * warp_smem_floats(cap, ne) * warps; }

template <int NE, int NZ>
static int launch_symm_t(const BatchDev& B, const PotParams& P, int warps, cudaStream_t st) {
  const size_t smem = symm_smem_bytes(B.cap, NE, warps);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(symm_kernel<NE, NZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  symm_kernel<NE, NZ><<<(B.natoms + warps - 1) / warps, 32 * warps, smem, st>>>(P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_r,
                                                                                  B.nb_cnt, B.G, B.gstride);
  return 0;
}
template <int NE, int NZ>
static int launch_force_t(const BatchDev& B, const PotParams& P, int warps, cudaStream_t st) {
  const size_t smem = force_smem_bytes(B.cap, NE, warps);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(force_kernel<NE, NZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  force_kernel<NE, NZ><<<(B.natoms + warps - 1) / warps, 32 * warps, smem, st>>>(P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_r,
                                                                                   B.nb_cnt, B.dEdG, B.gstride, B.W);
  return 0;
}

// Template instance covering (ne, nz): ne in {2,4}, nz in {5,6}.
int launch_symm(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st) {
  if (B.natoms == 0) return 0;
  if (ne <= 2 && nz <= 5) return launch_symm_t<2, 5>(B, P, warps, st);
  if (ne <= 4 && nz <= 5) return launch_symm_t<4, 5>(B, P, warps, st);
  if (ne <= 4 && nz <= 6) return launch_symm_t<4, 6>(B, P, warps, st);
  return -1;
}
int launch_force(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st) {
  if (B.natoms == 0) return 0;
  if (ne <= 2 && nz <= 5) return launch_force_t<2, 5>(B, P, warps, st);
  if (ne <= 4 && nz <= 5) return launch_force_t<4, 5>(B, P, warps, st);
  if (ne <= 4 && nz <= 6) return launch_force_t<4, 6>(B, P, warps, st);
  return -1;
}

}  // namespace nnpgpu
