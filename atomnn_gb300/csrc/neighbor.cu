// neighbor.cu - neighbour-list build on the GPU (NeighborList::build, src/struc/neighbor.cpp:59-171).
//
// One warp per centre atom.  Lists are written in the reference's order (neighbour atom j
// ascending, then the reference's lattice-shift enumeration order) into fixed-stride slots
// [i*cap, i*cap+count_i).  Set membership is decided in FP64 with the reference's own formula
// (Cell::diff then |diff - R_n|^2 <= rc^2, evaluated in the same order and without FMA
// contraction), so the pair sets equal the oracle's bit for bit.  An FP32 prefilter on wrapped
// fractional coordinates discards far pairs before the FP64 test.
#include "common.cuh"
#include "kernels.h"

namespace nnpgpu {

// Fractional coordinates wrapped to [0,1), FP32, for the prefilter.
__global__ void frac_kernel(int a0, int natoms, int ntypes, const int* __restrict__ type, const double* __restrict__ posn,
                            const int* __restrict__ atom_struc,
                            const StrucMeta* __restrict__ meta, float4* __restrict__ sfrac, int* __restrict__ status) {
  const int i = a0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a0 + natoms) return;
  const StrucMeta& S = meta[atom_struc[i]];
  const double p0 = posn[3 * i], p1 = posn[3 * i + 1], p2 = posn[3 * i + 2];
  if (!isfinite(p0) || !isfinite(p1) || !isfinite(p2)) atomicOr(&status[ST_ERROR], ERR_BAD_POSITION);
  if (type && (type[i] < 0 || type[i] >= ntypes)) atomicOr(&status[ST_ERROR], ERR_BAD_TYPE);
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
  if (S.mode != 0) {
    double f0, f1, f2;
    matvec(S.RInv, p0, p1, p2, f0, f1, f2);
    f0 -= floor(f0);
    f1 -= floor(f1);
    f2 -= floor(f2);
    s = make_float4((float)f0, (float)f1, (float)f2, 0.f);
  } else {
    s = make_float4((float)p0, (float)p1, (float)p2, 0.f);
  }
  sfrac[i] = s;
}

__device__ __forceinline__ void emit(int slot, int cap, int j, float rx, float ry, float rz, float dr, int code,
                                     int* __restrict__ nb_j, float4* __restrict__ nb_r, int* __restrict__ nb_code) {
  if (slot < cap) {
    nb_j[slot] = j;
    nb_r[slot] = make_float4(rx, ry, rz, dr);
    nb_code[slot] = code;
  }
}

__global__ void __launch_bounds__(128) neighbor_kernel(int a0, int natoms, int cap, double rc, const double* __restrict__ posn,
                                                       const float4* __restrict__ sfrac, const int* __restrict__ atom_struc,
                                                       const StrucMeta* __restrict__ meta, const ImgEntry* __restrict__ imgs,
                                                       int* __restrict__ nb_j, float4* __restrict__ nb_r,
                                                       int* __restrict__ nb_code, int* __restrict__ nb_cnt,
                                                       int* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int i = a0 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= a0 + natoms) return;
  const StrucMeta& S = meta[atom_struc[i]];
  const double rc2 = rc * rc;
  const int j0 = S.atom0, nj = S.natoms;
  const double pi0 = posn[3 * i], pi1 = posn[3 * i + 1], pi2 = posn[3 * i + 2];
  int* const oj = nb_j + (size_t)i * cap;
  float4* const orr = nb_r + (size_t)i * cap;
  int* const oc = nb_code + (size_t)i * cap;
  const unsigned lt = (1u << lane) - 1u;
  int count = 0;  // warp-uniform

  if (S.mode == 2) {
    // single image: keep the Cell::diff image if |diff|^2 <= rc^2 (the only shift is zero)
    const float4 si = sfrac[i];
    const float rc2hi = (float)rc2 + S.margin;
    for (int c = 0; c < nj; c += 32) {
      const int jl = c + lane;
      bool keep = false;
      double o0 = 0, o1 = 0, o2 = 0, d2 = 0;
      int D[3] = {0, 0, 0};
      if (jl < nj && j0 + jl != i) {
        const float4 sj = sfrac[j0 + jl];
        float d0 = si.x - sj.x, d1 = si.y - sj.y, d2f = si.z - sj.z;
        d0 -= rintf(d0);
        d1 -= rintf(d1);
        d2f -= rintf(d2f);
        const float r0 = S.Rf[0] * d0 + S.Rf[3] * d1 + S.Rf[6] * d2f;
        const float r1 = S.Rf[1] * d0 + S.Rf[4] * d1 + S.Rf[7] * d2f;
        const float r2 = S.Rf[2] * d0 + S.Rf[5] * d1 + S.Rf[8] * d2f;
        if (r0 * r0 + r1 * r1 + r2 * r2 <= rc2hi) {
          const int j = j0 + jl;
          cell_diff(S, pi0, pi1, pi2, posn[3 * j], posn[3 * j + 1], posn[3 * j + 2], o0, o1, o2, D);
          d2 = sqn3(o0, o1, o2);
          keep = d2 <= rc2;
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int slot = count + __popc(m & lt);
        emit(slot, cap, j0 + jl, (float)o0, (float)o1, (float)o2, (float)sqrt(d2), pack_code(D[0], D[1], D[2], true), oj, orr, oc);
      }
      count += __popc(m);
    }
  } else if (S.mode == 1) {
    // image shells: for each j, every shift of the box around the Cell::diff image (reference order)
    const ImgEntry* im = imgs + S.img0;
    const int nimg = S.nimg;
    for (int c = 0; c < nj; c += 32) {
      const int jl = c + lane;
      const int j = j0 + jl;
      double o0 = 0, o1 = 0, o2 = 0;
      int D[3] = {0, 0, 0};
      int cnt = 0, best = -1;
      if (jl < nj) {
        cell_diff(S, pi0, pi1, pi2, posn[3 * j], posn[3 * j + 1], posn[3 * j + 2], o0, o1, o2, D);
        double mn = S.fro;
        for (int n = 0; n < nimg; ++n) {
          const double t0 = dsub(o0, im[n].v[0]), t1 = dsub(o1, im[n].v[1]), t2 = dsub(o2, im[n].v[2]);
          const double d2 = sqn3(t0, t1, t2);
          const bool keep = (j != i) ? (d2 <= rc2) : (1e-6 < d2 && d2 <= rc2);
          if (keep) {
            ++cnt;
            if (j != i) {
              const double dr = sqrt(d2);
              if (dr < mn) { mn = dr; best = n; }
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
        for (int n = 0; n < nimg; ++n) {
          const double t0 = dsub(o0, im[n].v[0]), t1 = dsub(o1, im[n].v[1]), t2 = dsub(o2, im[n].v[2]);
          const double d2 = sqn3(t0, t1, t2);
          const bool keep = (j != i) ? (d2 <= rc2) : (1e-6 < d2 && d2 <= rc2);
          if (keep) {
            emit(slot, cap, j, (float)t0, (float)t1, (float)t2, (float)sqrt(d2),
                 pack_code(D[0] + im[n].n[0], D[1] + im[n].n[1], D[2] + im[n].n[2], n == best), oj, orr, oc);
            ++slot;
          }
        }
      }
      count += __shfl_sync(0xffffffffu, incl, 31);
    }
  } else {
    // non-periodic: plain differences; the reference leaves min=false here (src/struc/neighbor.cpp:149-169)
    for (int c = 0; c < nj; c += 32) {
      const int jl = c + lane;
      bool keep = false;
      double t0 = 0, t1 = 0, t2 = 0, d2 = 0;
      if (jl < nj) {
        const int j = j0 + jl;
        t0 = dsub(pi0, posn[3 * j]);
        t1 = dsub(pi1, posn[3 * j + 1]);
        t2 = dsub(pi2, posn[3 * j + 2]);
        d2 = sqn3(t0, t1, t2);
        keep = 1e-6 < d2 && d2 <= rc2;
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        emit(count + __popc(m & lt), cap, j0 + jl, (float)t0, (float)t1, (float)t2, (float)sqrt(d2), pack_code(0, 0, 0, false), oj,
             orr, oc);
      }
      count += __popc(m);
    }
  }
  if (lane == 0) {
    nb_cnt[i] = count;
    if (count > cap) atomicMax(&status[ST_MAXCOUNT], count);
  }
}

// Transposed index for the force gather.  For every minimum-image slot (i,s) -> j, find the
// minimum-image slot of j's list that points back to i and store there the global slot id of
// (i,s).  Lists are sorted by neighbour index, so each lane binary-searches its own target.
// A source without a partner (possible only for pairs within rounding of the cutoff, or ties
// between equidistant images) is recorded as an orphan and added by a serial fix-up pass.
__global__ void __launch_bounds__(128) reverse_kernel(int a0, int natoms, int cap, const int* __restrict__ nb_j,
                                                      const int* __restrict__ nb_code, const int* __restrict__ nb_cnt,
                                                      int* __restrict__ nb_rev, int* __restrict__ orphans, int orphan_cap,
                                                      int* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int i = a0 + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= a0 + natoms) return;
  const int n = min(nb_cnt[i], cap);
  for (int s = lane; s < n; s += 32) {
    const size_t src = (size_t)i * cap + s;
    if (!code_min(nb_code[src])) continue;
    const int j = nb_j[src];
    const int nj = min(nb_cnt[j], cap);
    const int* L = nb_j + (size_t)j * cap;
    int lo = 0, hi = nj;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (L[mid] < i) lo = mid + 1;
      else hi = mid;
    }
    int found = -1;
    for (int t = lo; t < nj && L[t] == i; ++t)
      if (code_min(nb_code[(size_t)j * cap + t])) { found = t; break; }
    if (found >= 0) {
      nb_rev[(size_t)j * cap + found] = (int)src;
    } else {
      const int k = atomicAdd(&status[ST_ORPHANS], 1);
      if (k < orphan_cap) orphans[k] = (int)src;
    }
  }
}

void launch_neighbors(const BatchDev& B, cudaStream_t st) {
  if (B.natoms == 0) return;
  frac_kernel<<<(B.natoms + 127) / 128, 128, 0, st>>>(B.a0, B.natoms, B.ntypes, B.type, B.posn, B.atom_struc, B.meta, B.sfrac, B.status);
  const int blocks = (B.natoms + 3) / 4;
  neighbor_kernel<<<blocks, 128, 0, st>>>(B.a0, B.natoms, B.cap, B.rc, B.posn, B.sfrac, B.atom_struc, B.meta, B.imgs, B.nb_j, B.nb_r,
                                          B.nb_code, B.nb_cnt, B.status);
}

void launch_reverse(const BatchDev& B, cudaStream_t st) {
  if (B.natoms == 0) return;
  cudaMemsetAsync(B.nb_rev + (size_t)B.a0 * B.cap, 0xff, sizeof(int) * (size_t)B.natoms * B.cap, st);
  reverse_kernel<<<(B.natoms + 3) / 4, 128, 0, st>>>(B.a0, B.natoms, B.cap, B.nb_j, B.nb_code, B.nb_cnt, B.nb_rev, B.orphans,
                                                     B.orphan_cap, B.status);
}

}  // namespace nnpgpu
