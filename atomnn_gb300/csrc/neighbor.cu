// neighbor.cu - neighbour-list build on the GPU (NeighborList::build, src/struc/neighbor.cpp:59-171).
//
// One warp per centre atom.  Lists are written in the reference's order (neighbour atom j
// ascending, then the reference's lattice-shift enumeration order) into fixed-stride slots
// [i*cap, i*cap+count_i).
//
// Decisions are made in FP32 from wrapped fractional coordinates (s = frac(R^-1 r)) and
// per-atom integer floors, so that the translation Cell::diff picks is known exactly.  Every
// FP32 decision carries a rounding margin; a pair whose FP32 value falls within the margin of
// a decision boundary (cutoff, half-cell rounding of Cell::diff, its 6-shift fallback test,
// equidistant images) is redone in FP64 with the reference's own formula, evaluated in the
// same order without FMA contraction.  The pair sets therefore equal the oracle's bit for bit
// while almost no FP64 work is done (GB300's FP64 rate is about 1/64 of its FP32 rate).
#include "common.cuh"
#include "kernels.h"

namespace nnpgpu {

// The fourth component of an atom's wrapped coordinates carries, as int bits, its species (bits
// 0-1) and, when all three fit in 9 bits, its integer floors (bits 2-10, 11-19, 20-28, each +256;
// bit 31 set): one 16-byte load then gives a candidate everything the single-image test needs.
__device__ __forceinline__ int pack_w(int sp, int f0, int f1, int f2) {
  const bool fit = f0 >= -256 && f0 < 256 && f1 >= -256 && f1 < 256 && f2 >= -256 && f2 < 256;
  return fit ? (sp | ((f0 + 256) << 2) | ((f1 + 256) << 11) | ((f2 + 256) << 20) | (int)(1u << 31)) : sp;
}
__device__ __forceinline__ int w_species(const float4& s) { return __float_as_int(s.w) & 3; }
// the floors of the atom whose wrapped coordinates are s: from s.w, else from its sfloor entry
__device__ __forceinline__ int4 w_floors(const float4& s, const int4* __restrict__ sfl, int k) {
  const unsigned w = (unsigned)__float_as_int(s.w);
  if (!(w >> 31)) return sfl[k];
  return make_int4((int)((w >> 2) & 511) - 256, (int)((w >> 11) & 511) - 256, (int)((w >> 20) & 511) - 256, 0);
}

// Wrapped fractional coordinates (FP32) and integer floors of R^-1 r, per atom.  Atoms of a
// cell-list structure (mode 4) are also binned: atom_cell[i] and the cell's atom count.
__global__ void frac_kernel(int a0, int natoms, int ntypes, const int* __restrict__ type, const double* __restrict__ posn,
                            const int* __restrict__ atom_struc, const StrucMeta* __restrict__ meta, float4* __restrict__ sfrac,
                            int4* __restrict__ sfloor, int* __restrict__ atom_cell, int* __restrict__ cell_cnt, int* __restrict__ status) {
  const int i = a0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a0 + natoms) return;
  const StrucMeta& S = meta[atom_struc[i]];
  const double p0 = posn[3 * i], p1 = posn[3 * i + 1], p2 = posn[3 * i + 2];
  const bool finite = isfinite(p0) && isfinite(p1) && isfinite(p2);
  if (!finite) atomicOr(&status[ST_ERROR], ERR_BAD_POSITION);
  if (type && (type[i] < 0 || type[i] >= ntypes)) atomicOr(&status[ST_ERROR], ERR_BAD_TYPE);
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
  int4 fl = make_int4(0, 0, 0, 0);
  if (S.mode != 0 && finite) {
    double f[3];
    matvec(S.RInv, p0, p1, p2, f[0], f[1], f[2]);
    float sf[3];
    int fi[3];
    for (int k = 0; k < 3; ++k) {
      const double fk = floor(f[k]);
      float v = (float)(f[k] - fk);
      int q = (fabs(fk) < 1e9) ? (int)fk : 0;
      if (v >= 1.0f) { v = 0.0f; ++q; }
      sf[k] = v;
      fi[k] = q;
    }
    s = make_float4(sf[0], sf[1], sf[2], 0.f);
    fl = make_int4(fi[0], fi[1], fi[2], 0);
  }  else {
    s = make_float4((float)p0, (float)p1, (float)p2, 0.f);
  }
  s.w = __int_as_float(pack_w(type ? clamp_type(type[i], ntypes) : 0, fl.x, fl.y, fl.z));
  sfrac[i] = s;
  sfloor[i] = fl;
  if (S.mode == 4) {
    const int cx = min((int)(s.x * (float)S.nc[0]), S.nc[0] - 1);
    const int cy = min((int)(s.y * (float)S.nc[1]), S.nc[1] - 1);
    const int cz = min((int)(s.z * (float)S.nc[2]), S.nc[2] - 1);
    const int c = S.cell0 + (cz * S.nc[1] + cy) * S.nc[0] + cx;
    atom_cell[i] = c;
    atomicAdd(&cell_cnt[c], 1);
  }
}

// Exclusive scan of the cell counts of each cell-list structure (one CTA per structure):
// cell_start[c] = the first position of cell c in cell_atoms; the entry after the last cell
// is the structure's end.
__global__ void __launch_bounds__(256) cell_scan_kernel(int s0, const StrucMeta* __restrict__ meta, const int* __restrict__ cell_cnt,
                                                        int* __restrict__ cell_start) {
  const StrucMeta& S = meta[s0 + blockIdx.x];
  if (S.mode != 4) return;
  __shared__ int wsum[8];
  __shared__ int carry;
  const int ncell = S.nc[0] * S.nc[1] * S.nc[2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = S.atom0;
  __syncthreads();
  for (int base = 0; base < ncell; base += 1024) {
    int v[4], t = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = base + 4 * threadIdx.x + q;
      v[q] = c < ncell ? cell_cnt[S.cell0 + c] : 0;
      t += v[q];
    }
    int incl = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int x = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += x;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    int before = carry;
    for (int k = 0; k < w; ++k) before += wsum[k];
    int run = before + incl - t;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = base + 4 * threadIdx.x + q;
      if (c < ncell) cell_start[S.cell0 + c] = run;
      run += v[q];
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int k = 0; k < 8; ++k) carry += wsum[k];
    __syncthreads();
  }
  if (threadIdx.x == 0) cell_start[S.cell0 + ncell] = carry;
}

// Places each atom of a cell-list structure into its cell, with cell-ordered copies of its
// wrapped coordinates and floors (the candidates of a stencil run are then contiguous in
// memory).  The count is taken back down to zero on the way, so the counts are clean for the
// next call.  The order within a cell does not matter: the neighbour kernel sorts every list by
// neighbour index.
__global__ void cell_fill_kernel(int a0, int natoms, const int* __restrict__ atom_struc, const StrucMeta* __restrict__ meta,
                                 const int* __restrict__ atom_cell, int* __restrict__ cell_cnt, const int* __restrict__ cell_start,
                                 int* __restrict__ cell_atoms, const float4* __restrict__ sfrac, const int4* __restrict__ sfloor,
                                 float4* __restrict__ sfrac_c, int4* __restrict__ sfloor_c, int* __restrict__ cell_of) {
  const int i = a0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a0 + natoms) return;
  if (meta[atom_struc[i]].mode != 4) return;
  const int c = atom_cell[i];
  const int pos = cell_start[c] + atomicSub(&cell_cnt[c], 1) - 1;
  cell_atoms[pos] = i;
  cell_of[pos] = c;
  sfrac_c[pos] = sfrac[i];
  sfloor_c[pos] = sfloor[i];
}

__device__ __forceinline__ void emit(int slot, int cap, int j, float rx, float ry, float rz, float dr, int code,
                                     int* __restrict__ nb_j, float4* __restrict__ nb_r, int* __restrict__ nb_code,
                                     unsigned char* __restrict__ nb_t, const float4* __restrict__ sfrac) {
  if (slot < cap) {
    nb_j[slot] = j;
    nb_r[slot] = make_float4(rx, ry, rz, dr);
    nb_code[slot] = code;
    if (nb_t) nb_t[slot] = (unsigned char)w_species(sfrac[j]);
  }
}

__device__ __forceinline__ void rf_mul(const StrucMeta& S, float d0, float d1, float d2, float& r0, float& r1, float& r2) {
  r0 = S.Rf[0] * d0 + S.Rf[3] * d1 + S.Rf[6] * d2;
  r1 = S.Rf[1] * d0 + S.Rf[4] * d1 + S.Rf[7] * d2;
  r2 = S.Rf[2] * d0 + S.Rf[5] * d1 + S.Rf[8] * d2;
}

// FP32 version of Cell::diff for the image-shell path.  Returns false when a decision is too
// close to call in FP32 (the caller then uses the FP64 replay).
__device__ __forceinline__ bool cell_diff_f32(const StrucMeta& S, const float4& si, const int4& fi, const float4& sj,
                                              const int4& fj, float& o0, float& o1, float& o2, int D[3]) {
  const float eps = 1e-5f;
  const float dl[3] = {si.x - sj.x, si.y - sj.y, si.z - sj.z};
  const int di[3] = {fi.x - fj.x, fi.y - fj.y, fi.z - fj.z};
  float d[3];
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // mod(f,-0.5,0.5) rounds half-integers up: D = floor(f + 0.5)
    const float t = dl[k] + 0.5f;  // in (-0.5, 1.5): the floor is one of -1, 0, 1
    const float fk = (t >= 1.0f) ? 1.0f : ((t >= 0.0f) ? 0.0f : -1.0f);
    const float fr = t - fk;
    if (fr < eps || fr > 1.0f - eps) ok = false;
    d[k] = dl[k] - fk;
    D[k] = (int)fk + di[k];
  }
  rf_mul(S, d[0], d[1], d[2], o0, o1, o2);
  const float m = S.margin;
  const float n2 = o0 * o0 + o1 * o1 + o2 * o2;
  const float dmax2 = S.dmax2f;
  if (fabsf(n2 - dmax2) <= m) ok = false;
  if (n2 > dmax2) {
    float best = n2, second = 3.4e38f, b0 = o0, b1 = o1, b2 = o2;
    int bk = -1;
    for (int k = 0; k < 6; ++k) {
      const float t0 = o0 + S.shiftsf[3 * k], t1 = o1 + S.shiftsf[3 * k + 1], t2 = o2 + S.shiftsf[3 * k + 2];
      const float q = t0 * t0 + t1 * t1 + t2 * t2;
      if (q < best) { second = best; best = q; b0 = t0; b1 = t1; b2 = t2; bk = k; }
      else if (q < second) second = q;
    }
    if (second - best <= m) ok = false;
    if (bk >= 0) {  // constant indices keep D in registers
      const int step = (bk % 2 == 0) ? -1 : 1;
      if (bk < 2) D[0] += step;
      else if (bk < 4) D[1] += step;
      else D[2] += step;
    }
    o0 = b0; o1 = b1; o2 = b2;
  }
  return ok;
}

// Single-image decision (modes 2 and 4) for centre i and candidate j: the Cell::diff image of
// j is kept when |diff|^2 <= rc^2.  FP32 from the wrapped fractional coordinates, with the FP64
// replay of Cell::diff when |diff|^2 lies within the margin of rc^2.
// sj = the candidate's wrapped coordinates, loaded by the caller ahead of use; its floors are
// packed in sj.w, or else sfl[jf] (the atom's own entry, or its cell-ordered copy).
__device__ __forceinline__ bool single_image(const StrucMeta& S, const float4& si, const int4& fi, int j, const float4 sj,
                                             const int4* __restrict__ sfl, int jf, const double* __restrict__ posn, double pi0, double pi1,
                                             double pi2, double rc2, float rc2f, float m, float& r0, float& r1, float& r2, float& dr,
                                             int D[3]) {
  const float dl0 = si.x - sj.x, dl1 = si.y - sj.y, dl2 = si.z - sj.z;
  int k0, k1, k2;
  const float q0 = round_even(dl0, k0), q1 = round_even(dl1, k1), q2 = round_even(dl2, k2);
  rf_mul(S, dl0 - q0, dl1 - q1, dl2 - q2, r0, r1, r2);
  const float d2f = r0 * r0 + r1 * r1 + r2 * r2;
  if (d2f > rc2f + m) return false;
  const int4 fj = w_floors(sj, sfl, jf);
  D[0] = k0 + fi.x - fj.x;
  D[1] = k1 + fi.y - fj.y;
  D[2] = k2 + fi.z - fj.z;
  if (d2f < rc2f - m) {
    dr = sqrtf(d2f);
    return true;
  }
  double o0, o1, o2;
  cell_diff(S, pi0, pi1, pi2, posn[3 * j], posn[3 * j + 1], posn[3 * j + 2], o0, o1, o2, D);
  const double d2 = sqn3(o0, o1, o2);
  r0 = (float)o0;
  r1 = (float)o1;
  r2 = (float)o2;
  dr = (float)sqrt(d2);
  return d2 <= rc2;
}

// Per-warp shared memory of the cell-list path: staged slots (cap), candidate ranges and the
// bit mask used to rank the staged neighbours by index.
constexpr int NB_RANGES = 128;  // >= 2 (2*3+1)^2 rows of the widest stencil (reach 3)
constexpr int NB_MASK_WORDS = 128;  // structures up to 4096 atoms rank through the bit mask
__host__ __device__ inline size_t nb_warp_smem(int cap) { return (size_t)cap * 24 + 4 * (2 * NB_RANGES + 2 * NB_MASK_WORDS); }
size_t neighbor_smem_bytes(int cap, int warps) { return (size_t)warps * nb_warp_smem(cap); }

// 8 CTAs of 4 warps per SM (64 registers): the candidate loop is latency-bound, and the extra
// resident warps pay for the few spilled registers
__global__ void __launch_bounds__(128, 8) neighbor_kernel(int a0, int natoms, int cap, double rc, const double* __restrict__ posn,
                                                       const float4* __restrict__ sfrac, const int4* __restrict__ sfloor,
                                                       const int* __restrict__ atom_struc, const StrucMeta* __restrict__ meta,
                                                       const ImgEntry* __restrict__ imgs,
                                                       const int* __restrict__ cell_start, const int* __restrict__ cell_atoms,
                                                       const float4* __restrict__ sfrac_c, const int4* __restrict__ sfloor_c,
                                                       int* __restrict__ nb_j, float4* __restrict__ nb_r, int* __restrict__ nb_code,
                                                       unsigned char* __restrict__ nb_t, int* __restrict__ nb_cnt,
                                                       int* __restrict__ status, const int* __restrict__ order,
                                                       const int* __restrict__ cell_of) {
  const int lane = threadIdx.x & 31;
  int i = a0 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= a0 + natoms) return;
  if (order) i = order[i];  // whole structures, the slowest first
  const int kpos = i;       // for a cell-list structure: the centre's position in cell order
  const StrucMeta& S = meta[atom_struc[i]];
  // cell-list centres in cell order: the warps of a CTA (and of an SM) then search overlapping
  // stencils and share the candidates' lines in L1
  if (S.mode == 4) i = cell_atoms[i];
  const double rc2 = rc * rc;
  const float rc2f = (float)rc2, m = S.margin;
  const int j0 = S.atom0, nj = S.natoms;
  const double pi0 = posn[3 * i], pi1 = posn[3 * i + 1], pi2 = posn[3 * i + 2];
  int* const oj = nb_j + (size_t)i * cap;
  float4* const orr = nb_r + (size_t)i * cap;
  int* const oc = nb_code + (size_t)i * cap;
  unsigned char* const ot = nb_t ? nb_t + (size_t)i * cap : nullptr;
  const unsigned lt = (1u << lane) - 1u;
  int count = 0;  // warp-uniform

  if (S.mode == 2) {
    // single image: keep the Cell::diff image if |diff|^2 <= rc^2 (the only shift is zero)
    const float4 si = sfrac[i];
    const int4 fi = sfloor[i];
    float4 sn = lane < nj ? sfrac[j0 + lane] : make_float4(0.f, 0.f, 0.f, 0.f);  // one chunk ahead
    for (int c = 0; c < nj; c += 32) {
      const int jl = c + lane;
      const int j = j0 + jl;
      const float4 sj = sn;
      if (jl + 32 < nj) sn = sfrac[j + 32];
      bool keep = false;
      float r0 = 0.f, r1 = 0.f, r2 = 0.f, dr = 0.f;
      int D[3] = {0, 0, 0};
      if (jl < nj && j != i) keep = single_image(S, si, fi, j, sj, sfloor, j, posn, pi0, pi1, pi2, rc2, rc2f, m, r0, r1, r2, dr, D);
      const unsigned mk = __ballot_sync(0xffffffffu, keep);
      if (keep) emit(count + __popc(mk & lt), cap, j, r0, r1, r2, dr, pack_code(D[0], D[1], D[2], true), oj, orr, oc, ot, sfrac);
      count += __popc(mk);
    }
  } else if (S.mode == 4) {
    // cell list: the candidates are the atoms of the (2 reach + 1)^3 cells around the centre's
    // cell, visited as contiguous x-runs of cells (two runs where the stencil wraps); accepted
    // neighbours are staged in shared memory and written out in increasing index order.
    extern __shared__ __align__(16) unsigned char nb_smem[];
    unsigned char* wbase = nb_smem + (size_t)(threadIdx.x >> 5) * nb_warp_smem(cap);
    float4* st_r = (float4*)wbase;
    int* st_j = (int*)(st_r + cap);
    int* st_c = st_j + cap;
    int* rb = st_c + cap;           // range begin (position in cell_atoms)
    int* rp = rb + NB_RANGES;       // range prefix (candidate numbering)
    unsigned* msk = (unsigned*)(rp + NB_RANGES);
    int* wpre = (int*)(msk + NB_MASK_WORDS);
    const int k = S.reach, nx = S.nc[0], ny = S.nc[1], nz = S.nc[2];
    const int side = 2 * k + 1, nrow = side * side;
    const int ci = cell_of[kpos] - S.cell0;  // read beside cell_atoms[kpos], not after it
    const int cx = ci % nx, cy = (ci / nx) % ny, cz = ci / (nx * ny);
    // ranges 2q, 2q+1 of row q: start[] is monotone, so a run of cells is one slice of cell_atoms
    int len[4], beg[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int r = 4 * lane + t;
      const int q = r >> 1;
      int begin = 0, n = 0;
      if (q < nrow) {
        int y = cy + (q % side) - k, z = cz + (q / side) - k;
        y += (y < 0) ? ny : ((y >= ny) ? -ny : 0);
        z += (z < 0) ? nz : ((z >= nz) ? -nz : 0);
        const int row = S.cell0 + (z * ny + y) * nx;
        const int xlo = cx - k, xhi = cx + k;
        int a, b;  // cells [a, b] of this part, b < a means empty
        if (xlo < 0) {
          a = (r & 1) ? 0 : xlo + nx;
          b = (r & 1) ? xhi : nx - 1;
        } else if (xhi >= nx) {
          a = (r & 1) ? 0 : xlo;
          b = (r & 1) ? xhi - nx : nx - 1;
        } else {
          a = xlo;
          b = (r & 1) ? xlo - 1 : xhi;
        }
        if (b >= a) {
          begin = cell_start[row + a];
          n = cell_start[row + b + 1] - begin;
        }
      }
      len[t] = n;
      beg[t] = begin;
    }
    // candidate numbering (prefix of the run lengths) and the non-empty runs compacted in order:
    // rb[k], rp[k] = begin in cell_atoms and first candidate number of the k-th non-empty run
    const int lsum = len[0] + len[1] + len[2] + len[3];
    const int lne = (len[0] > 0) + (len[1] > 0) + (len[2] > 0) + (len[3] > 0);
    int incl = lsum, incn = lne;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      const int w = __shfl_up_sync(0xffffffffu, incn, o);
      if (lane >= o) {
        incl += v;
        incn += w;
      }
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int nne = __shfl_sync(0xffffffffu, incn, 31);
    int run = incl - lsum, kk = incn - lne;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      if (len[t] > 0) {
        rb[kk] = beg[t];
        rp[kk] = run;
        ++kk;
      }
      run += len[t];
    }
    __syncwarp();
    // up to 32 * NB_MASK_WORDS candidates: a bit mask of the runs' first candidates and its word
    // prefix (the ranking buffers, free until the lists are written) give a candidate's run as a
    // rank, two independent shared-memory levels instead of a binary search
    const bool by_rank = total <= 32 * NB_MASK_WORDS;
    if (by_rank) {
#pragma unroll
      for (int t = 0; t < NB_MASK_WORDS / 32; ++t) msk[lane + 32 * t] = 0u;
      __syncwarp();
      for (int q = lane; q < nne; q += 32) atomicOr(&msk[rp[q] >> 5], 1u << (rp[q] & 31));
      __syncwarp();
      int wc[NB_MASK_WORDS / 32], ws = 0;
#pragma unroll
      for (int t = 0; t < NB_MASK_WORDS / 32; ++t) {
        wc[t] = __popc(msk[4 * lane + t]);
        ws += wc[t];
      }
      int winc = ws;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, winc, o);
        if (lane >= o) winc += v;
      }
      int wrun = winc - ws;
#pragma unroll
      for (int t = 0; t < NB_MASK_WORDS / 32; ++t) {
        wpre[4 * lane + t] = wrun;
        wrun += wc[t];
      }
      __syncwarp();
    }
    const float4 si = sfrac_c[kpos];  // the centre's own entries, at its cell-order position
    const int4 fi = sfloor_c[kpos];
    // candidate qd -> its position in cell_atoms: the last non-empty run starting at or before qd
    auto candidate = [&](int qd) -> int {
      int kr;
      if (by_rank) {
        const int w = qd >> 5;
        kr = wpre[w] + __popc(msk[w] & (0xffffffffu >> (31 - (qd & 31)))) - 1;
      } else {
        int lo = 0, hi = nne - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (rp[mid] <= qd) lo = mid;
          else hi = mid - 1;
        }
        kr = lo;
      }
      return rb[kr] + qd - rp[kr];
    };
    // the next chunk's candidates and coordinates are fetched while this chunk is decided; the
    // coordinates come from the cell-ordered copy (contiguous along a run)
    int pn = lane < total ? candidate(lane) : -1;
    int jn = pn >= 0 ? cell_atoms[pn] : -1;
    float4 sn = pn >= 0 ? sfrac_c[pn] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int c = 0; c < total; c += 32) {
      const int j = jn, pj = pn;
      const float4 sj = sn;
      const int qn = c + 32 + lane;
      if (qn < total) {
        pn = candidate(qn);
        jn = cell_atoms[pn];
        sn = sfrac_c[pn];
      }
      bool keep = false;
      float r0 = 0.f, r1 = 0.f, r2 = 0.f, dr = 0.f;
      int D[3] = {0, 0, 0};
      if (c + lane < total && j != i)
        keep = single_image(S, si, fi, j, sj, sfloor_c, pj, posn, pi0, pi1, pi2, rc2, rc2f, m, r0, r1, r2, dr, D);
      const unsigned mk = __ballot_sync(0xffffffffu, keep);
      const int slot = count + __popc(mk & lt);
      if (keep && slot < cap) {
        st_j[slot] = j | (w_species(sj) << 30);  // species in the top two bits
        st_r[slot] = make_float4(r0, r1, r2, dr);
        st_c[slot] = pack_code(D[0], D[1], D[2], true);
      }
      count += __popc(mk);
    }
    __syncwarp();
    const int n = min(count, cap);
    if (nj <= 32 * NB_MASK_WORDS) {
      // rank = number of staged neighbours with a smaller index, read off a bit mask
#pragma unroll
      for (int t = 0; t < NB_MASK_WORDS / 32; ++t) msk[lane + 32 * t] = 0u;
      __syncwarp();
      for (int e = lane; e < n; e += 32) {
        const int jl = (st_j[e] & 0x3fffffff) - j0;
        atomicOr(&msk[jl >> 5], 1u << (jl & 31));
      }
      __syncwarp();
      int wc[NB_MASK_WORDS / 32], ws = 0;
#pragma unroll
      for (int t = 0; t < NB_MASK_WORDS / 32; ++t) {
        wc[t] = __popc(msk[4 * lane + t]);
        ws += wc[t];
      }
      int winc = ws;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, winc, o);
        if (lane >= o) winc += v;
      }
      int wrun = winc - ws;
#pragma unroll
      for (int t = 0; t < NB_MASK_WORDS / 32; ++t) {
        wpre[4 * lane + t] = wrun;
        wrun += wc[t];
      }
      __syncwarp();
      for (int e = lane; e < n; e += 32) {
        const int jg = st_j[e] & 0x3fffffff, jl = jg - j0;
        const int rank = wpre[jl >> 5] + __popc(msk[jl >> 5] & ((1u << (jl & 31)) - 1u));
        oj[rank] = jg;
        if (ot) ot[rank] = (unsigned char)((unsigned)st_j[e] >> 30);
        orr[rank] = st_r[e];
        oc[rank] = st_c[e];
      }
    } else {
      for (int e = lane; e < n; e += 32) {
        const int jg = st_j[e] & 0x3fffffff;
        int rank = 0;
        for (int f = 0; f < n; ++f) rank += ((st_j[f] & 0x3fffffff) < jg) ? 1 : 0;
        oj[rank] = jg;
        if (ot) ot[rank] = (unsigned char)((unsigned)st_j[e] >> 30);
        orr[rank] = st_r[e];
        oc[rank] = st_c[e];
      }
    }
  } else if (S.mode == 3) {
    // resident skin list (built with a larger cutoff at some earlier positions): the candidates
    // are its (j, T) entries in their stored order (j ascending); each is re-decided exactly as
    // in mode 2 for the current positions.
    const float4 si = sfrac[i];
    const int4 fi = sfloor[i];
    const int il = i - j0;
    const int ns = S.skin_cnt[il];
    const int* sj_l = S.skin_j + (size_t)il * S.skin_cap;
    const int* sc_l = S.skin_code + (size_t)il * S.skin_cap;
    for (int c = 0; c < ns; c += 32) {
      const int s = c + lane;
      bool keep = false;
      float r0 = 0.f, r1 = 0.f, r2 = 0.f, dr = 0.f;
      int T[3] = {0, 0, 0};
      int j = -1;
      if (s < ns) {
        const int jl = sj_l[s];
        const int code = sc_l[s];
        j = j0 + jl;
        const float4 sj = sfrac[j];
        const int4 fj = w_floors(sj, sfloor, j);
        T[0] = code_t_full(code, 0, fi.x - fj.x);
        T[1] = code_t_full(code, 1, fi.y - fj.y);
        T[2] = code_t_full(code, 2, fi.z - fj.z);
        // f_i - f_j - T = (s_i - s_j) + (floor_i - floor_j - T): the integer part is exact
        const float d0 = (si.x - sj.x) + (float)(fi.x - fj.x - T[0]);
        const float d1 = (si.y - sj.y) + (float)(fi.y - fj.y - T[1]);
        const float d2 = (si.z - sj.z) + (float)(fi.z - fj.z - T[2]);
        rf_mul(S, d0, d1, d2, r0, r1, r2);
        const float d2f = r0 * r0 + r1 * r1 + r2 * r2;
        if (d2f < rc2f - m) {
          keep = true;
          dr = sqrtf(d2f);
        } else if (d2f <= rc2f + m) {
          double o0, o1, o2;
          int D[3];
          cell_diff(S, pi0, pi1, pi2, posn[3 * j], posn[3 * j + 1], posn[3 * j + 2], o0, o1, o2, D);
          const double dd = sqn3(o0, o1, o2);
          keep = (D[0] == T[0] && D[1] == T[1] && D[2] == T[2]) && dd <= rc2;
          r0 = (float)o0; r1 = (float)o1; r2 = (float)o2;
          dr = (float)sqrt(dd);
        }
      }
      const unsigned mk = __ballot_sync(0xffffffffu, keep);
      if (keep) emit(count + __popc(mk & lt), cap, j, r0, r1, r2, dr, pack_code(T[0], T[1], T[2], true), oj, orr, oc, ot, sfrac);
      count += __popc(mk);
    }
  } else if (S.mode == 1) {
    // image shells: for each j, every shift of the box around the Cell::diff image (reference order)
    const ImgEntry* im = imgs + S.img0;
    const int nimg = S.nimg;
    const float4 si = sfrac[i];
    const int4 fi = sfloor[i];
    for (int c = 0; c < nj; c += 32) {
      const int jl = c + lane;
      const int j = j0 + jl;
      float o0 = 0.f, o1 = 0.f, o2 = 0.f;
      double p0 = 0, p1 = 0, p2 = 0;
      int D[3] = {0, 0, 0};
      int cnt = 0, best = -1;
      bool exact = false;  // FP64 replay for this pair
      // the images that can lie within rc of the difference: a box in the sorted lattice
      // coordinates, visited in the reference's order (image n = ((a+s0)(2s1+1) + b+s1)(2s2+1) + c+s2)
      int lo[3] = {0, 0, 0}, hi[3] = {-1, -1, -1};
      if (jl < nj) {
        const float4 sj = sfrac[j];
        bool ok = cell_diff_f32(S, si, fi, sj, w_floors(sj, sfloor, j), o0, o1, o2, D);
        if (ok) {
          const float fr[3] = {S.rinvf[0] * o0 + S.rinvf[3] * o1 + S.rinvf[6] * o2, S.rinvf[1] * o0 + S.rinvf[4] * o1 + S.rinvf[7] * o2,
                               S.rinvf[2] * o0 + S.rinvf[5] * o1 + S.rinvf[8] * o2};
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const int col = S.perm[a];
            const float f = col == 0 ? fr[0] : (col == 1 ? fr[1] : fr[2]);
            const float h = col == 0 ? S.hrc[0] : (col == 1 ? S.hrc[1] : S.hrc[2]);
            lo[a] = max(-S.shell[a], (int)ceilf(f - h));
            hi[a] = min(S.shell[a], (int)floorf(f + h));
          }
          float mn = 3.4e38f, second = 3.4e38f;
          for (int a0 = lo[0]; a0 <= hi[0] && ok; ++a0)
            for (int a1 = lo[1]; a1 <= hi[1] && ok; ++a1)
              for (int a2 = lo[2]; a2 <= hi[2]; ++a2) {
                const int n = ((a0 + S.shell[0]) * (2 * S.shell[1] + 1) + (a1 + S.shell[1])) * (2 * S.shell[2] + 1) + (a2 + S.shell[2]);
                const float t0 = o0 - im[n].vf[0], t1 = o1 - im[n].vf[1], t2 = o2 - im[n].vf[2];
                const float d2 = t0 * t0 + t1 * t1 + t2 * t2;
                if (fabsf(d2 - rc2f) <= m) { ok = false; break; }
                const bool keep = (j != i) ? (d2 <= rc2f) : (1e-6f < d2 && d2 <= rc2f);
                if (keep) {
                  ++cnt;
                  if (j != i) {
                    if (d2 < mn) { second = mn; mn = d2; best = n; }
                    else if (d2 < second) second = d2;
                  }
                }
              }
          // a near tie between the two closest kept images could flip the minimum-image flag;
          // with fewer than two kept images (or for the self pair) there is no tie to resolve
          if (ok && best >= 0 && second < 3.0e38f && second - mn <= m) ok = false;
          // the reference seeds the minimum search with |R|_F (neighbor.cpp:132)
          if (ok && best >= 0 && mn >= S.fro2f - m) ok = false;
        }
        if (!ok) {
          exact = true;
          cnt = 0;
          best = -1;
          cell_diff(S, pi0, pi1, pi2, posn[3 * j], posn[3 * j + 1], posn[3 * j + 2], p0, p1, p2, D);
          double mnd = S.fro;
          for (int n = 0; n < nimg; ++n) {
            const double t0 = dsub(p0, im[n].v[0]), t1 = dsub(p1, im[n].v[1]), t2 = dsub(p2, im[n].v[2]);
            const double d2 = sqn3(t0, t1, t2);
            const bool keep = (j != i) ? (d2 <= rc2) : (1e-6 < d2 && d2 <= rc2);
            if (keep) {
              ++cnt;
              if (j != i) {
                const double dr = sqrt(d2);
                if (dr < mnd) { mnd = dr; best = n; }
              }
            }
          }
        }
      }
      // exclusive scan of per-lane counts keeps j-major order
      int incl = cnt;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      int slot = count + incl - cnt;
      if (cnt > 0) {
        // the exact replay visits every image, the FP32 path its box
        if (exact) {
          lo[0] = -S.shell[0]; lo[1] = -S.shell[1]; lo[2] = -S.shell[2];
          hi[0] = S.shell[0]; hi[1] = S.shell[1]; hi[2] = S.shell[2];
        }
        for (int a0 = lo[0]; a0 <= hi[0]; ++a0)
          for (int a1 = lo[1]; a1 <= hi[1]; ++a1)
            for (int a2 = lo[2]; a2 <= hi[2]; ++a2) {
              const int n = ((a0 + S.shell[0]) * (2 * S.shell[1] + 1) + (a1 + S.shell[1])) * (2 * S.shell[2] + 1) + (a2 + S.shell[2]);
              float t0, t1, t2, dr;
              bool keep;
              if (exact) {
                const double e0 = dsub(p0, im[n].v[0]), e1 = dsub(p1, im[n].v[1]), e2 = dsub(p2, im[n].v[2]);
                const double d2 = sqn3(e0, e1, e2);
                keep = (j != i) ? (d2 <= rc2) : (1e-6 < d2 && d2 <= rc2);
                t0 = (float)e0; t1 = (float)e1; t2 = (float)e2;
                dr = keep ? (float)sqrt(d2) : 0.f;
              } else {
                t0 = o0 - im[n].vf[0]; t1 = o1 - im[n].vf[1]; t2 = o2 - im[n].vf[2];
                const float d2 = t0 * t0 + t1 * t1 + t2 * t2;
                keep = (j != i) ? (d2 <= rc2f) : (1e-6f < d2 && d2 <= rc2f);
                dr = sqrtf(d2);
              }
              if (keep) {
                emit(slot, cap, j, t0, t1, t2, dr, pack_code(D[0] + im[n].n[0], D[1] + im[n].n[1], D[2] + im[n].n[2], n == best), oj, orr, oc,
                     ot, sfrac);
                ++slot;
              }
            }
      }
      count += __shfl_sync(0xffffffffu, incl, 31);
    }
  } else {
    // non-periodic: plain differences; the reference leaves min=false here (src/struc/neighbor.cpp:149-169)
    const float4 si = sfrac[i];
    for (int c = 0; c < nj; c += 32) {
      const int jl = c + lane;
      bool keep = false;
      float r0 = 0.f, r1 = 0.f, r2 = 0.f, dr = 0.f;
      if (jl < nj) {
        const int j = j0 + jl;
        const float4 sj = sfrac[j];
        const float a = si.x - sj.x, b = si.y - sj.y, cc = si.z - sj.z;
        const float d2f = a * a + b * b + cc * cc;
        const float rcw = (float)rc + 0.5f;  // FP32 prefilter only; the decision is FP64
        if (d2f <= rcw * rcw) {
          const double t0 = dsub(pi0, posn[3 * j]), t1 = dsub(pi1, posn[3 * j + 1]), t2 = dsub(pi2, posn[3 * j + 2]);
          const double d2 = sqn3(t0, t1, t2);
          keep = 1e-6 < d2 && d2 <= rc2;
          r0 = (float)t0; r1 = (float)t1; r2 = (float)t2;
          dr = (float)sqrt(d2);
        }
      }
      const unsigned mk = __ballot_sync(0xffffffffu, keep);
      if (keep) emit(count + __popc(mk & lt), cap, j0 + jl, r0, r1, r2, dr, pack_code(0, 0, 0, false), oj, orr, oc, ot, sfrac);
      count += __popc(mk);
    }
  }
  if (lane == 0) {
    nb_cnt[i] = count;
    if (count > cap) atomicMax(&status[ST_MAXCOUNT], count);
  }
}

void launch_neighbors(const BatchDev& B, cudaStream_t st, int warps) {
  warps = warps < 1 ? 1 : (warps > 4 ? 4 : warps);
  if (B.natoms == 0) return;
  frac_kernel<<<(B.natoms + 127) / 128, 128, 0, st>>>(B.a0, B.natoms, B.ntypes, B.type, B.posn, B.atom_struc, B.meta, B.sfrac,
                                                      B.sfloor, B.atom_cell, B.cell_cnt, B.status);
  size_t smem = 0;
  if (B.ncells > 0) {
    cell_scan_kernel<<<B.nstruc, 256, 0, st>>>(B.s0, B.meta, B.cell_cnt, B.cell_start);
    cell_fill_kernel<<<(B.natoms + 127) / 128, 128, 0, st>>>(B.a0, B.natoms, B.atom_struc, B.meta, B.atom_cell, B.cell_cnt, B.cell_start,
                                                             B.cell_atoms, B.sfrac, B.sfloor, B.sfrac_c, B.sfloor_c, B.cell_of);
    smem = neighbor_smem_bytes(B.cap, warps);
    static bool attr = false;  // skin lists may ask for up to 1024 slots per atom (106 KB)
    if (!attr) attr = cudaFuncSetAttribute(neighbor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  }
  const int blocks = (B.natoms + warps - 1) / warps;
  neighbor_kernel<<<blocks, 32 * warps, smem, st>>>(B.a0, B.natoms, B.cap, B.rc, B.posn, B.sfrac, B.sfloor, B.atom_struc, B.meta, B.imgs,
                                             B.cell_start, B.cell_atoms, B.sfrac_c, B.sfloor_c, B.nb_j, B.nb_r, B.nb_code, B.nb_t,
                                             B.nb_cnt, B.status, B.nb_order, B.cell_of);
}

}  // namespace nnpgpu
