// common.cuh - shared definitions of the GB300 NNP kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nnpgpu {

// ---- limits of the GPU path (checked on the host when the potential is loaded)
constexpr int NT_MAX = 4;                          // atom types
constexpr int NB_MAX = NT_MAX * (NT_MAX + 1) / 2;  // angular blocks per centre type
constexpr int NR_MAX = 32;                         // radial functions per (centre, neighbour) type
constexpr int NA_MAX = 64;                         // angular functions per block
constexpr int NE_MAX = 4;                          // distinct angular widths per block
constexpr int NL = 2;                              // distinct lambda values per block
constexpr int NZ_MAX = 6;                          // zeta = 2^m, m < NZ_MAX
constexpr int NIN_MAX = 256;                       // network inputs
constexpr int MOM_N = 4;                           // largest zeta of a moment-tensor block
constexpr int MOM_C = 35;                          // symmetric tensor components of degree 0..MOM_N
constexpr int MOM_Q = 20;                          // components of degree 0..MOM_N-1
constexpr int MOM_EX = 8 * MOM_Q;                  // per-width floats a moment block needs in shared memory
constexpr int NLAYER_MAX = 4;                      // network layers (hidden + output)
constexpr int HID_MAX = 256;                       // nodes per layer

enum { CUT_STEP = 1, CUT_COS = 2, CUT_TANH = 3 };
// radial families (PhiRN, src/nnp/basis_radial.hpp:25-33) and angular pair factors (PhiAN,
// src/nnp/basis_angular.hpp:25-32)
enum { RAD_GAUSSIAN = 1, RAD_TANH = 2, RAD_SOFTPLUS = 3, RAD_LOGCOSH = 4, RAD_SWISH = 5, RAD_MISH = 6 };
enum { ANG_GAUSS = 1, ANG_IPOWP = 2, ANG_IPOWS = 3, ANG_SECHP = 4, ANG_SECHS = 5 };
enum { ACT_LINEAR = 1, ACT_SIGMOID = 2, ACT_TANH = 3 };
// IPOWS and SECHS take r_ij^alpha + r_ik^alpha as one argument; the other families are products
__host__ __device__ inline bool ang_sum_family(int phi) { return phi == ANG_IPOWS || phi == ANG_SECHS; }

// Radial basis of centre type I against neighbour type J (BasisR, src/nnp/basis_radial.hpp:53-94).
struct RadialP {
  int n, off, cut, phi;
  float rc, pirc, rci, norm;
  float rs[NR_MAX], eta[NR_MAX];
};

// Angular basis of centre type I against neighbour pair block (J,K) (BasisA,
// src/nnp/basis_angular.hpp:53-115).  The block's functions are mapped onto a grid (distinct
// 1/eta^alpha) x (distinct lambda) x (zeta = 2^m); gidx[f] is the grid cell
// (e*NL + l)*NZ_MAX + m of file function f.  phi is the radial factor (ANG_*): GAUSS, IPOWP and
// SECHP are products h(r_ij) h(r_ik), IPOWS and SECHS functions of r_ij^alpha + r_ik^alpha.
// mom = 1 marks a block evaluated through moment tensors (a product family, every zeta <= 4,
// |lambda| <= 1); its moments start at float moff of the atom's row.  tab is the block's offset
// in PotParams::atab: n grid cells (as floats), then for a moment block the n x (ne*(MOM_N+1))
// matrix M[f][e*(MOM_N+1)+k] = norm * (coefficient of cos^k in function f's angular term) when f
// has width e, 0 otherwise.  fn = 1 marks a block that leaves the grid (a zeta that is not a
// power of two up to 2^(NZ_MAX-1), more than NE_MAX widths or NL lambdas): it takes the
// per-function triplet path, and tab holds per function (1/eta^alpha, lambda, zeta, 0).
// top = 1 marks a split GAUSS block: its functions with zeta <= MOM_N take
// the moment path (mom = 1, their rows of M as above), the others all have the block's largest
// zeta 2^(nz-1) and take the triplet path, which evaluates only that grid level (their rows of
// M are zero).  When the centre type's moment blocks share their moments, the columns of M
// follow the widths of block PotParams::mrep.
struct AngP {
  int n, off, cut, alpha;
  float rc, pirc, rci, norm;
  int ne, nl, nz, mom;
  int moff, phi, tab, fn;
  int top;
  float ietap[NE_MAX];
  float lam[NL];
  signed char gidx[NA_MAX];
};

struct PotParams {
  int ntypes;
  float rc;
  int nin[NT_MAX];
  int mstride;  // floats of moment storage per atom (0: no moment blocks)
  int kx;       // 1: a triplet-path block of IPOWP or SECHP needs per-pair derivative weights
  int gen;      // 1: some angular block has a family other than GAUSS
  int pad;
  const float* atab;  // per-block tables of the angular functions (AngP::tab), device memory
  // cutoff shared by every basis of centre type I (ccut 0: the bases differ)
  int ccut[NT_MAX];
  float crc[NT_MAX], cpirc[NT_MAX], crci[NT_MAX];
  // shared moments of centre type I (msh 1): its moment blocks (at most three) share one pair
  // weight and involve the mns <= 2 neighbour species msp[I][0..mns); mrep is the block with the
  // most widths (the others' widths are among its, and its pair weight stands for all); the
  // stored moments are [set][width of mrep][MOM_C]
  int msh[NT_MAX], mns[NT_MAX], mrep[NT_MAX];
  int msp[NT_MAX][2];
  RadialP rad[NT_MAX][NT_MAX];
  AngP ang[NT_MAX][NB_MAX];
};

__host__ __device__ inline int lidx(int i, int j) { return (i >= j) ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// One atomic network on the device (NN::ANN, src/ml/nn.hpp:218-341).  Weights are row-major
// [out][in] (as ANN::w_), plus a transposed copy [in][out] for the forward GEMMs.
struct NetP {
  int nin, nlayer, act, pad;
  int nodes[NLAYER_MAX];
  const float* w[NLAYER_MAX];   // [nodes[l]][cols(l)]
  const float* wt[NLAYER_MAX];  // [cols(l)][nodes[l]]
  const float* b[NLAYER_MAX];
  const float* inpw;
  const float* inpb;
  float outw, outb;
  double evac;  // species vacuum energy (Type::energy, src/nnp/type.hpp)
};
struct NetsP {
  NetP net[NT_MAX];
};

// Per-structure geometry of a batch.  mode: 0 non-periodic, 1 image shells (some shell > 0),
// 2 single image (all shells 0: at most one image of each atom within the cutoff), 3 single
// image with the candidate pairs taken from a resident skin list (skin_j/skin_code/skin_cnt,
// local atom indices, skin_cap slots per atom) instead of all atoms of the structure, 4 single
// image with the candidates taken from a cell list: nc[k] cells along fractional axis k, each
// at least rc/reach wide, and the (2 reach + 1)^3 cells around the centre's cell searched;
// the structure's cells occupy entries [cell0, cell0 + nc0*nc1*nc2] of the batch's cell arrays
// (the last entry is the end sentinel).
struct StrucMeta {
  int atom0, natoms, mode, nimg;
  int img0, skin_cap, cell0, reach;
  const int* skin_j;
  const int* skin_code;
  const int* skin_cnt;
  const void* pad3;
  double R[9], RInv[9];  // column-major
  double dMax2, fro;
  double shifts[18];     // +col0, -col0, +col1, -col1, +col2, -col2 (Cell::init, src/struc/cell.cpp:63-69)
  float Rf[9];
  float margin;          // FP32 filter margin on r^2
  int nc[3];             // cell grid (mode 4)
  int pad4;
  float dmax2f, fro2f;   // FP32 copies of dMax2 and fro^2, and of the shifts, for the FP32 tests
  float shiftsf[18];
  // image shells (mode 1): the images of lattice vectors sorted by decreasing norm (perm[a] is
  // the column of sorted vector a) run over [-shell[a], shell[a]]; an image n can be within rc
  // of a difference o only if |(R^-1 o)_c - n_c| <= hrc[c] = rc |row c of R^-1| + margin
  float rinvf[9];        // R^-1 in FP32, column-major
  float hrc[3];
  int shell[3], perm[3];
};
// One lattice shift of the image box, in the reference's enumeration order (vf = v in FP32).
struct ImgEntry {
  double v[3];
  int n[3];
  float vf[3];
  int pad;
};

// Device status words (one int array per context).
// Forces are summed in 64-bit fixed point with FORCE_FRAC_BITS fractional bits (2^-32 eV/A): each
// neighbour slot's FP32 contribution is rounded once to that grid, and integer sums are exact and
// commutative, so a force does not depend on the order in which warps add to it.  A contribution
// that is not finite or whose components' magnitudes add up to FORCE_MAX_ABS or more (where the
// sums could wrap) is reported as ERR_FORCE_RANGE, and the call's results are discarded.
constexpr float FORCE_MAX_ABS = 1.0e9f;
constexpr int FORCE_FRAC_BITS = 32;
enum { ST_MAXCOUNT = 0, ST_ERROR = 2, ST_DEBUG = 8, ST_WORDS = 32 };
enum { ERR_BAD_POSITION = 1, ERR_BAD_TYPE = 2, ERR_TIMEOUT = 8, ERR_DRAIN = 16, ERR_FORCE_RANGE = 32 };

#ifdef __CUDACC__
// ---- exact FP64 helpers: fixed evaluation order and no FMA contraction, so that the GPU
// reproduces the oracle's (and the reference's) rounding of Cell::diff and |r|^2 bit for bit.
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double sqn3(double x, double y, double z) { return dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z)); }
// o = M v, M column-major, summed in index order
__device__ __forceinline__ void matvec(const double* M, double v0, double v1, double v2, double& o0, double& o1, double& o2) {
  o0 = dadd(dadd(dmul(M[0], v0), dmul(M[3], v1)), dmul(M[6], v2));
  o1 = dadd(dadd(dmul(M[1], v0), dmul(M[4], v1)), dmul(M[7], v2));
  o2 = dadd(dadd(dmul(M[2], v0), dmul(M[5], v1)), dmul(M[8], v2));
}
// math::special::mod(n,-0.5,0.5) (src/math/special.hpp:43-46); fmod(x,1) == x - trunc(x) exactly.
__device__ __forceinline__ double modhalf(double n) {
  const double x = dsub(n, -0.5);
  const double a = dsub(x, trunc(x));
  const double b = dadd(a, 1.0);
  const double c = dsub(b, trunc(b));
  return dadd(c, -0.5);
}
// Cell::diff (src/struc/cell.cpp:103-128): minimum-image difference p1-p2 with the 6-shift
// fallback; D receives the integer translation (diff = p1 - p2 - R*D).
__device__ __forceinline__ void cell_diff(const StrucMeta& S, double p0, double p1, double p2, double q0, double q1, double q2,
                                          double& o0, double& o1, double& o2, int D[3]) {
  double f0, f1, f2;
  matvec(S.RInv, dsub(p0, q0), dsub(p1, q1), dsub(p2, q2), f0, f1, f2);
  const double m0 = modhalf(f0), m1 = modhalf(f1), m2 = modhalf(f2);
  D[0] = (int)llrint(f0 - m0);
  D[1] = (int)llrint(f1 - m1);
  D[2] = (int)llrint(f2 - m2);
  matvec(S.R, m0, m1, m2, o0, o1, o2);
  if (sqn3(o0, o1, o2) > S.dMax2) {
    double dmin2 = sqn3(o0, o1, o2), r0 = o0, r1 = o1, r2 = o2;
    int best = -1;
    for (int k = 0; k < 6; ++k) {
      const double t0 = dadd(o0, S.shifts[3 * k]), t1 = dadd(o1, S.shifts[3 * k + 1]), t2 = dadd(o2, S.shifts[3 * k + 2]);
      const double d2 = sqn3(t0, t1, t2);
      if (d2 < dmin2) { dmin2 = d2; r0 = t0; r1 = t1; r2 = t2; best = k; }
    }
    if (best >= 0) {  // constant indices keep D in registers
      const int step = (best % 2 == 0) ? -1 : 1;
      if (best < 2) D[0] += step;
      else if (best < 4) D[1] += step;
      else D[2] += step;
    }
    o0 = r0; o1 = r1; o2 = r2;
  }
}

#endif  // __CUDACC__

// Neighbour slot code: bits 0-29 hold the lattice translation (3 x 10 bit, offset 512), bit 30
// the minimum-image flag.
__host__ __device__ inline int pack_code(int t0, int t1, int t2, bool mn) {
  return ((t0 + 512) & 0x3ff) | (((t1 + 512) & 0x3ff) << 10) | (((t2 + 512) & 0x3ff) << 20) | (mn ? (1 << 30) : 0);
}
__host__ __device__ inline bool code_min(int c) { return (c >> 30) & 1; }
__host__ __device__ inline int code_t(int c, int k) { return ((c >> (10 * k)) & 0x3ff) - 512; }
// The code keeps a slot's lattice translation T modulo 1024 per axis (code_t, in [-512, 512)).  T
// differs from the difference of the two atoms' integer floors (dfloor = floor_i - floor_j) only by
// the rounding of Cell::diff and the image shell, far less than 512 cells: the full T is the value
// congruent to code_t nearest to dfloor.
__host__ __device__ inline int code_t_full(int c, int k, int dfloor) {
  const int low = code_t(c, k);
  const int q = dfloor - low + 512;
  const int m = q >= 0 ? q / 1024 : -((-q + 1023) / 1024);  // floor(q / 1024)
  return low + 1024 * m;
}

#ifdef __CUDACC__
// Asynchronous 16-byte global -> shared copies (cp.async), committed in groups and waited
// for by group count: rows and candidates are requested ahead of the instruction that reads them.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Round to nearest, ties to even (as rintf), for |x| < 2^22, with plain FP32 adds: adding
// 1.5*2^23 leaves the rounded integer in the low mantissa bits.  k receives it as an int.
__device__ __forceinline__ float round_even(float x, int& k) {
  const float big = 12582912.0f;
  const float t = __fadd_rn(x, big);
  k = __float_as_int(t) - 0x4B400000;
  return __fsub_rn(t, big);
}

// ---- cutoff functions (Basis::cut_func / cut_grad, src/nnp/basis.cpp:80-120), FP32
__device__ __forceinline__ void cutoff_fg(int cut, float d, float rc, float pirc, float rci, float& f, float& g) {
  if (cut == CUT_COS) {
    if (d < rc) {
      float s, c;
      __sincosf(d * pirc, &s, &c);
      f = 0.5f * (c + 1.0f);
      g = -0.5f * pirc * s;
    } else {
      f = (d > rc) ? 0.f : 0.5f * (__cosf(d * pirc) + 1.0f);
      g = 0.f;
    }
  } else if (cut == CUT_TANH) {
    const float t = (d > rc) ? 0.f : tanhf(1.0f - d * rci);
    f = t * t * t;
    g = (d < rc) ? -3.0f * t * t * (1.0f - t * t) * rci : 0.f;
  } else {  // STEP
    f = (d > rc) ? 0.f : 1.f;
    g = 0.f;
  }
}

// Radial factor of the angular families (BasisA::symm/force, basis_angular.cpp:406-640) at
// x = ietap * r^alpha (product families) or ietap * (r_ij^alpha + r_ik^alpha) (sum families):
// returns h(x) and sets kap so that dh/dx = -kap * h.  GAUSS: exp(-x), kap 1; IPOWP/IPOWS:
// 1/(1+x), kap = h; SECHP/SECHS: sech(x), kap = sqrt(1 - sech^2) = |tanh x| as the reference
// writes it, here from e = exp(-|x|) without the cancellation of 1 - sech^2.
__device__ __forceinline__ float ang_h(int phi, float x, float& kap) {
  if (phi == ANG_IPOWP || phi == ANG_IPOWS) {
    const float h = 1.0f / (1.0f + x);
    kap = h;
    return h;
  }
  if (phi == ANG_SECHP || phi == ANG_SECHS) {
    const float e = __expf(-fabsf(x)), e2 = e * e, den = 1.0f / (1.0f + e2);
    kap = (1.0f - e2) * den;
    return 2.0f * e * den;
  }
  kap = 1.0f;
  return __expf(-x);
}

// species index clamped into the table (invalid input is flagged by frac_kernel)
__device__ __forceinline__ int clamp_type(int t, int ntypes) { return t < 0 ? 0 : (t >= ntypes ? ntypes - 1 : t); }

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Reduce-scatter of four per-lane values over the warp in five shuffles: afterwards the lanes
// with (lane >> 3) & 3 == k hold the warp sum of v_k.
__device__ __forceinline__ float warp_sum4(float v0, float v1, float v2, float v3) {
  const int lane = threadIdx.x & 31;
  const bool h16 = lane & 16, h8 = lane & 8;
  float a = h16 ? v2 : v0, b = h16 ? v3 : v1;  // kept: the pair of values of this half
  a += __shfl_xor_sync(0xffffffffu, h16 ? v0 : v2, 16);
  b += __shfl_xor_sync(0xffffffffu, h16 ? v1 : v3, 16);
  float k = h8 ? b : a;  // kept: one value of the pair
  k += __shfl_xor_sync(0xffffffffu, h8 ? a : b, 8);
  k += __shfl_xor_sync(0xffffffffu, k, 4);
  k += __shfl_xor_sync(0xffffffffu, k, 2);
  k += __shfl_xor_sync(0xffffffffu, k, 1);
  return k;
}
__device__ __forceinline__ long long force_fixed(float w) { return __float2ll_rn(w * (float)(1ull << FORCE_FRAC_BITS)); }
__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// fire-and-forget 64-bit integer add (two's complement: negative values subtract)
__device__ __forceinline__ void red_add(long long* p, long long v) { atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v); }
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

#endif  // __CUDACC__

}  // namespace nnpgpu
