// nnpgpu.cpp - the C ABI (include/nnpgpu.h): context, batch set-up and the launch sequence.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <stdexcept>

#include "context.h"

using namespace nnpgpu;

namespace nnpgpu {

int set_error(nnpgpu_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

static int cuda_fail(nnpgpu_ctx* c, cudaError_t e, const char* where) {
  return set_error(c, NNPGPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

bool ensure(nnpgpu_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.bytes) return true;
  size_t want = std::max(bytes, b.bytes + b.bytes / 2);
  want = (want + 255) & ~(size_t)255;
  if (c->budget && c->used - b.bytes + want > c->budget) {
    want = bytes;
    if (c->used - b.bytes + want > c->budget) return false;
  }
  if (b.p) cudaFree(b.p);
  c->used -= b.bytes;
  b.p = nullptr;
  b.bytes = 0;
  if (cudaMalloc(&b.p, want) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  b.bytes = want;
  c->used += want;
  c->buf_generation++;
  return true;
}

bool ensure_host(nnpgpu_ctx* c, HostBuf& b, size_t bytes) {
  (void)c;
  if (bytes <= b.bytes) return true;
  size_t want = std::max(bytes, b.bytes + b.bytes / 2);
  if (b.p) cudaFreeHost(b.p);
  b.p = nullptr;
  b.bytes = 0;
  if (cudaMallocHost(&b.p, want) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  b.bytes = want;
  return true;
}

static double nrm3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// Cell grid of a single-image structure (mode 2 -> 4).  Along fractional axis k the cell
// count is the largest nc with width h_k / nc >= rc / reach + slack (h_k = 1/|row k of R^-1|,
// the distance between the cell's faces), so that any atom within rc of a centre lies within
// reach cells of the centre's cell; nc >= 2 reach + 1 keeps the stencil's cells distinct.  The
// reach with the fewest candidates wins; brute force stays when cells would not pay.
static void choose_cells(StrucMeta& m, int natoms, double rc) {
  double h[3];
  for (int k = 0; k < 3; ++k) {
    const double a = m.RInv[k], b = m.RInv[3 + k], c = m.RInv[6 + k];
    h[k] = 1.0 / std::sqrt(a * a + b * b + c * c);
  }
  double best = 0.5;  // candidate fraction that the cell path must beat
  for (int reach = 1; reach <= 3; ++reach) {
    const double w = rc / reach + 1e-4 * rc + 1e-3;
    int nc[3];
    bool ok = true;
    double cells = 1;
    for (int k = 0; k < 3; ++k) {
      const double q = std::floor(h[k] / w);
      nc[k] = q > 1024 ? 1024 : (int)q;
      ok = ok && nc[k] >= 2 * reach + 1;
      cells *= nc[k];
    }
    if (!ok || cells > 4.0 * natoms + 64) continue;
    const double frac = std::pow(2.0 * reach + 1, 3) / cells;
    if (frac < best) {
      best = frac;
      m.mode = 4;
      m.reach = reach;
      for (int k = 0; k < 3; ++k) m.nc[k] = nc[k];
    }
  }
}

void make_meta(const double* cell, int atom0, int natoms, double rc, StrucMeta& m, std::vector<ImgEntry>& imgs) {
  std::memset(&m, 0, sizeof(m));
  m.atom0 = atom0;
  m.natoms = natoms;
  double fro = 0;
  for (int k = 0; k < 9; ++k) {
    m.R[k] = cell ? cell[k] : 0.0;
    fro += m.R[k] * m.R[k];
  }
  fro = std::sqrt(fro);
  m.fro = fro;
  if (!(fro > 0)) {
    m.mode = 0;
    return;
  }
  auto M = [&](int r, int c) { return m.R[3 * c + r]; };
  // inverse by cofactors (Cell::init, src/struc/cell.cpp:49)
  const double c00 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
  const double c01 = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
  const double c02 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
  const double det = M(0, 0) * c00 + M(0, 1) * c01 + M(0, 2) * c02;
  if (det == 0 || !std::isfinite(det)) throw PotError(NNPGPU_ERR_INVALID, "singular or non-finite cell");
  const double id = 1.0 / det;
  double inv[3][3];
  inv[0][0] = c00 * id;
  inv[1][0] = c01 * id;
  inv[2][0] = c02 * id;
  inv[0][1] = (M(0, 2) * M(2, 1) - M(0, 1) * M(2, 2)) * id;
  inv[1][1] = (M(0, 0) * M(2, 2) - M(0, 2) * M(2, 0)) * id;
  inv[2][1] = (M(0, 1) * M(2, 0) - M(0, 0) * M(2, 1)) * id;
  inv[0][2] = (M(0, 1) * M(1, 2) - M(0, 2) * M(1, 1)) * id;
  inv[1][2] = (M(0, 2) * M(1, 0) - M(0, 0) * M(1, 2)) * id;
  inv[2][2] = (M(0, 0) * M(1, 1) - M(0, 1) * M(1, 0)) * id;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) m.RInv[3 * c + r] = inv[r][c];
  double col[3][3];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) col[c][r] = m.R[3 * c + r];
  double dmax = nrm3(col[0]);
  for (int c = 1; c < 3; ++c) dmax = std::min(dmax, nrm3(col[c]));
  dmax *= 0.5;
  m.dMax2 = dmax * dmax;
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) {
      m.shifts[6 * c + r] = col[c][r];
      m.shifts[6 * c + 3 + r] = -col[c][r];
    }
  for (int k = 0; k < 9; ++k) m.Rf[k] = (float)m.R[k];
  for (int k = 0; k < 18; ++k) m.shiftsf[k] = (float)m.shifts[k];
  m.dmax2f = (float)m.dMax2;
  m.fro2f = (float)(fro * fro);
  // image shells (NeighborList::build, src/struc/neighbor.cpp:70-95), lattice vectors sorted
  // by decreasing norm with a stable order for ties
  int perm[3] = {0, 1, 2};
  std::stable_sort(perm, perm + 3, [&](int a, int b) { return nrm3(col[a]) > nrm3(col[b]); });
  const double* R0 = col[perm[0]];
  const double* R1 = col[perm[1]];
  const double* R2 = col[perm[2]];
  const double cx[3] = {R0[1] * R1[2] - R0[2] * R1[1], R0[2] * R1[0] - R0[0] * R1[2], R0[0] * R1[1] - R0[1] * R1[0]};
  const double dot2 = R2[0] * cx[0] + R2[1] * cx[1] + R2[2] * cx[2];
  // shell ratios bounded in FP64 before the integer conversion: a near-flat cell gives huge ratios
  const double ratio[3] = {2.0 * rc / nrm3(R0), 2.0 * rc / (nrm3(cx) / nrm3(R0)), 2.0 * rc / std::fabs(dot2 / (nrm3(R0) * nrm3(R1)))};
  int shell[3];
  double nimg_total = 1;
  for (int c = 0; c < 3; ++c) {
    if (!std::isfinite(ratio[c]) || ratio[c] > 1e6) throw PotError(NNPGPU_ERR_INVALID, "cell too thin for the cutoff (lattice image shells)");
    shell[c] = (int)std::floor(ratio[c]);
    nimg_total *= 2.0 * shell[c] + 1;
  }
  if (nimg_total > 1e6) throw PotError(NNPGPU_ERR_INVALID, "cell too thin for the cutoff: more than 1e6 lattice images");
  double Lsum = nrm3(col[0]) + nrm3(col[1]) + nrm3(col[2]);
  m.margin = (float)(2.0 * rc * (Lsum * 1e-6 + 1e-5) + 1e-4 * rc * rc);
  if (shell[0] == 0 && shell[1] == 0 && shell[2] == 0) {
    m.mode = 2;
    choose_cells(m, natoms, rc);
    return;
  }
  m.mode = 1;
  set_image_box(m, inv, rc, shell, perm);
  m.img0 = (int)imgs.size();
  for (int i = -shell[0]; i <= shell[0]; ++i)
    for (int j = -shell[1]; j <= shell[1]; ++j)
      for (int k = -shell[2]; k <= shell[2]; ++k) {
        ImgEntry e;
        std::memset(&e, 0, sizeof(e));
        for (int x = 0; x < 3; ++x) {
          e.v[x] = i * R0[x] + j * R1[x] + k * R2[x];
          e.vf[x] = (float)e.v[x];
        }
        e.n[perm[0]] = i;
        e.n[perm[1]] = j;
        e.n[perm[2]] = k;
        imgs.push_back(e);
      }
  m.nimg = (int)imgs.size() - m.img0;
}

// Neighbour capacity estimate from the densest structure (rounded up to 32).
static int estimate_cap(const nnpgpu_ctx* c, int nstruc, const int* natoms, const double* cell) {
  double best = 16;
  const double rc = c->pot.rc;
  const double sphere = 4.0 / 3.0 * M_PI * (rc + 0.5) * (rc + 0.5) * (rc + 0.5);
  for (int s = 0; s < nstruc; ++s) {
    const double* R = cell + 9 * s;
    const double vol = std::fabs(R[0] * (R[4] * R[8] - R[7] * R[5]) - R[3] * (R[1] * R[8] - R[7] * R[2]) + R[6] * (R[1] * R[5] - R[4] * R[2]));
    double nb;
    if (vol > 0) nb = natoms[s] / vol * sphere * 1.1 + 16;
    else nb = natoms[s];
    best = std::max(best, nb);
  }
  int cap = (int)std::ceil(best / 32.0) * 32;
  if (c->cap_hint > 0) cap = (c->cap_hint + 31) / 32 * 32;  // explicit or learned capacity
  return std::min(cap, 1024);
}

int run_pipeline(nnpgpu_ctx* c, const BatchDev& B, int flags, cudaStream_t st) {
  const bool want_force = flags & NNPGPU_FORCE;
  const bool want_energy = flags & NNPGPU_ENERGY;
  const bool prof = c->prof_on && (flags & NNPGPU_BATCHED);
  cudaStreamCaptureStatus cap_state = cudaStreamCaptureStatusNone;
  if (prof) cudaStreamIsCapturing(st, &cap_state);
  // inside a capture the events become external event-record nodes of the graph
  const unsigned ev_flags = (cap_state == cudaStreamCaptureStatusActive) ? cudaEventRecordExternal : cudaEventRecordDefault;
  auto mark = [&](int k) {
    if (prof) cudaEventRecordWithFlags(c->prof_ev[k], st, ev_flags);
  };
  mark(0);
  launch_neighbors(B, st, c->tune.warps_nbr);
  mark(1);
  if (want_force) cudaMemsetAsync(B.facc + 3 * (size_t)B.a0, 0, sizeof(long long) * 3 * (size_t)B.natoms, st);
  mark(2);
  if (launch_symm(B, c->P, c->ne, c->nz, c->tune.warps_symm, st) != 0) return set_error(c, NNPGPU_ERR_UNSUPPORTED, "no symm kernel instance");
  mark(3);
  if (want_energy || want_force) {
    launch_type_sort(B, c->pot.ntypes, st);
    if (flags & NNPGPU_BF16) {
      const int rcode = launch_network_bf16(B, c->nets, c->tcbuf, c->pot.ntypes, st, c->tcnets ? c->tcnets->data() : nullptr,
                                            want_force ? 1 : 0, c->tc_wait_limit);
      if (rcode == -1) return set_error(c, NNPGPU_ERR_UNSUPPORTED, "BF16 network path unavailable for this potential");
      if (rcode != 0) return cuda_fail(c, cudaGetLastError(), "tensor-core network set-up");
    } else {
      launch_network_fp32(B, c->nets, c->pot.ntypes, c->tune.nn_tile, st);
    }
    mark(4);
    if (want_force)
      if (launch_force(B, c->P, c->ne, c->nz, c->tune.warps_force, st) != 0) return set_error(c, NNPGPU_ERR_UNSUPPORTED, "no force kernel instance");
    mark(5);
    launch_gather(B, c->nets, !(flags & NNPGPU_NO_VACUUM), want_force, st);
  } else {
    mark(4);
    mark(5);
  }
  mark(6);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, "kernel launch");
  return NNPGPU_OK;
}

}  // namespace nnpgpu

// ------------------------------------------------------------------------------------------
namespace {


// Validates the batch description and uploads geometry metadata; sizes all batch buffers.
// True when the device already holds the geometry of exactly this batch description (same
// cutoff, capacity, atom counts, cells, skin lists and buffers): repeated steps of one batch then
// skip the per-structure set-up and its upload.
static bool meta_cached(const nnpgpu_ctx* c, int nstruc, const int* natoms, const double* cell, int cap, const SkinRef* skins) {
  const MetaCache& m = c->meta_cache;
  if (!m.valid || m.generation != c->buf_generation || m.rc != c->pot.rc || m.cap != cap || m.U.nstruc != nstruc) return false;
  if (nstruc == 0) return true;
  if (std::memcmp(m.natoms.data(), natoms, sizeof(int) * nstruc) != 0) return false;
  if (std::memcmp(m.cell.data(), cell, sizeof(double) * 9 * nstruc) != 0) return false;
  for (int s = 0; s < nstruc; ++s) {
    const SkinRef r = skins ? skins[s] : SkinRef();
    if (m.skins[4 * s] != r.j || m.skins[4 * s + 1] != r.code || m.skins[4 * s + 2] != r.cnt || m.skins[4 * s + 3] != (const void*)(intptr_t)r.cap)
      return false;
  }
  return true;
}

int prepare(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* cell, int cap, Uploaded& U, cudaStream_t st,
            const SkinRef* skins = nullptr) {
  if (nstruc < 0 || (nstruc > 0 && (!natoms || !cell))) return set_error(c, NNPGPU_ERR_INVALID, "invalid batch description");
  if (meta_cached(c, nstruc, natoms, cell, cap, skins)) {
    U = c->meta_cache.U;
    cudaMemsetAsync(c->status.p, 0, sizeof(int) * ST_WORDS, st);
    return NNPGPU_OK;
  }
  c->meta_cache.valid = false;
  U.nstruc = nstruc;
  U.offsets.assign(nstruc + 1, 0);
  for (int s = 0; s < nstruc; ++s) {
    if (natoms[s] < 0) return set_error(c, NNPGPU_ERR_INVALID, "negative atom count");
    U.offsets[s + 1] = U.offsets[s] + natoms[s];
  }
  U.natoms = U.offsets[nstruc];
  std::vector<ImgEntry> imgs;
  U.metas.resize(nstruc);
  try {
    for (int s = 0; s < nstruc; ++s) {
      make_meta(cell + 9 * s, U.offsets[s], natoms[s], c->pot.rc, U.metas[s], imgs);
      if (skins && skins[s].cnt && (U.metas[s].mode == 2 || U.metas[s].mode == 4)) {
        U.metas[s].mode = 3;
        U.metas[s].skin_j = skins[s].j;
        U.metas[s].skin_code = skins[s].code;
        U.metas[s].skin_cnt = skins[s].cnt;
        U.metas[s].skin_cap = skins[s].cap;
      }
    }
  } catch (PotError& e) {
    return set_error(c, e.code, e.what());
  }
  U.ncells = 0;
  for (int s = 0; s < nstruc; ++s)
    if (U.metas[s].mode == 4) {
      U.metas[s].cell0 = U.ncells;
      U.ncells += U.metas[s].nc[0] * U.metas[s].nc[1] * U.metas[s].nc[2] + 1;
    }
  if (imgs.empty()) imgs.resize(1);
  U.cap = cap;
  const size_t N = std::max(U.natoms, 1);
  const size_t NC = N * cap;
  bool ok = true;
  ok = ok && ensure(c, c->posn, sizeof(double) * 3 * N) && ensure(c, c->type, sizeof(int) * N) &&
       ensure(c, c->atom_struc, sizeof(int) * N) && ensure(c, c->meta, sizeof(StrucMeta) * std::max(nstruc, 1)) &&
       ensure(c, c->imgs, sizeof(ImgEntry) * imgs.size()) && ensure(c, c->sfrac, sizeof(float4) * N) && ensure(c, c->sfloor, sizeof(int4) * N) &&
       ensure(c, c->nb_j, sizeof(int) * NC) && ensure(c, c->nb_r, sizeof(float4) * NC) && ensure(c, c->nb_code, sizeof(int) * NC) &&
       ensure(c, c->nb_t, NC) &&
       ensure(c, c->nb_cnt, sizeof(int) * N) &&
       ensure(c, c->G, sizeof(float) * N * c->gstride) && ensure(c, c->dEdG, sizeof(float) * N * c->gstride) &&
       ensure(c, c->eatom, sizeof(float) * N) && ensure(c, c->perm, sizeof(int) * N) &&
       ensure(c, c->type_count, sizeof(int) * type_sort_ints((int)N)) && ensure(c, c->facc, sizeof(long long) * 3 * N) &&
       ensure(c, c->force, sizeof(double) * 3 * N) && ensure(c, c->energy, sizeof(double) * std::max(nstruc, 1)) &&
       ensure(c, c->status, sizeof(int) * ST_WORDS) && ensure(c, c->nb_order, sizeof(int) * N) && ensure(c, c->at_order, sizeof(int) * N) && (c->P.mstride == 0 || ensure(c, c->mom, sizeof(float) * N * c->P.mstride));
  if (ok && U.ncells > 0) {
    // cell counts must start at zero: fresh memory is cleared, later calls leave them at zero
    const size_t before = c->cell_cnt.bytes;  // a grown buffer is a new allocation
    ok = ensure(c, c->cell_cnt, sizeof(int) * U.ncells) && ensure(c, c->cell_start, sizeof(int) * U.ncells) &&
         ensure(c, c->cell_atoms, sizeof(int) * N) && ensure(c, c->atom_cell, sizeof(int) * N) && ensure(c, c->cell_of, sizeof(int) * N) &&
         ensure(c, c->sfrac_c, sizeof(float4) * N) && ensure(c, c->sfloor_c, sizeof(int4) * N);
    if (ok && c->cell_cnt.bytes != before) cudaMemsetAsync(c->cell_cnt.p, 0, c->cell_cnt.bytes, st);
  }
  if (!ok) return set_error(c, NNPGPU_ERR_OOM, "device allocation failed or HBM budget exceeded");
  // atom -> structure map and metadata
  std::vector<int> as(N, 0);
  for (int s = 0; s < nstruc; ++s)
    for (int a = U.offsets[s]; a < U.offsets[s + 1]; ++a) as[a] = s;
  // the neighbour kernel's warp order: structures by candidate pairs per centre, most first
  std::vector<int> sord(nstruc), order;
  order.reserve(N);
  {
    std::vector<double> cost(nstruc);
    for (int s = 0; s < nstruc; ++s) {
      const StrucMeta& m = U.metas[s];
      double cand = m.natoms;
      if (m.mode == 1) cand *= m.nimg;
      else if (m.mode == 3) cand = m.skin_cap;
      else if (m.mode == 4) cand *= std::pow(2.0 * m.reach + 1.0, 3) / ((double)m.nc[0] * m.nc[1] * m.nc[2]);
      cost[s] = cand;
    }
    for (int s = 0; s < nstruc; ++s) sord[s] = s;
    std::stable_sort(sord.begin(), sord.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    for (int s : sord)
      for (int a = U.offsets[s]; a < U.offsets[s + 1]; ++a) order.push_back(a);
    order.resize(N, 0);
    // the descriptor and chain-rule kernels: densest structures first (their cost per atom grows
    // with the neighbours per atom); isolated structures last
    for (int s = 0; s < nstruc; ++s) {
      const StrucMeta& m = U.metas[s];
      const double* R = m.R;
      const double vol = std::fabs(R[0] * (R[4] * R[8] - R[7] * R[5]) - R[3] * (R[1] * R[8] - R[7] * R[2]) + R[6] * (R[1] * R[5] - R[4] * R[2]));
      cost[s] = (m.mode != 0 && vol > 0) ? m.natoms / vol : 0.0;
    }
    for (int s = 0; s < nstruc; ++s) sord[s] = s;
    std::stable_sort(sord.begin(), sord.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    for (int s : sord)
      for (int a = U.offsets[s]; a < U.offsets[s + 1]; ++a) order.push_back(a);
    order.resize(2 * N, 0);
  }
  const size_t meta_bytes = sizeof(StrucMeta) * nstruc, img_bytes = sizeof(ImgEntry) * imgs.size(), as_bytes = sizeof(int) * N;
  cudaStreamSynchronize(st);  // the staging buffer may still feed an earlier copy
  if (!ensure_host(c, c->h_meta, meta_bytes + img_bytes + 3 * as_bytes + 64)) return set_error(c, NNPGPU_ERR_OOM, "pinned host allocation failed");
  char* h = (char*)c->h_meta.p;
  std::memcpy(h, U.metas.data(), meta_bytes);
  std::memcpy(h + meta_bytes, imgs.data(), img_bytes);
  std::memcpy(h + meta_bytes + img_bytes, as.data(), as_bytes);
  std::memcpy(h + meta_bytes + img_bytes + as_bytes, order.data(), 2 * as_bytes);
  cudaMemcpyAsync(c->meta.p, h, meta_bytes, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->imgs.p, h + meta_bytes, img_bytes, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->atom_struc.p, h + meta_bytes + img_bytes, as_bytes, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->nb_order.p, h + meta_bytes + img_bytes + as_bytes, as_bytes, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->at_order.p, h + meta_bytes + img_bytes + 2 * as_bytes, as_bytes, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(c->status.p, 0, sizeof(int) * ST_WORDS, st);
  MetaCache& m = c->meta_cache;
  m.valid = true;
  m.generation = c->buf_generation;
  m.rc = c->pot.rc;
  m.cap = cap;
  m.natoms.assign(natoms, natoms + nstruc);
  m.cell.assign(cell, cell + 9 * (size_t)nstruc);
  m.skins.resize(4 * (size_t)nstruc);
  for (int s = 0; s < nstruc; ++s) {
    const SkinRef r = skins ? skins[s] : SkinRef();
    m.skins[4 * s] = r.j;
    m.skins[4 * s + 1] = r.code;
    m.skins[4 * s + 2] = r.cnt;
    m.skins[4 * s + 3] = (const void*)(intptr_t)r.cap;
  }
  m.U = U;
  return NNPGPU_OK;
}

BatchDev batch_view(nnpgpu_ctx* c, const Uploaded& U, const double* posn, const int* type, double* energy, double* force) {
  BatchDev B;
  B.natoms = U.natoms;
  B.nstruc = U.nstruc;
  B.cap = U.cap;
  B.rc = c->pot.rc;
  B.ntypes = c->pot.ntypes;
  B.posn = posn;
  B.type = type;
  B.atom_struc = (const int*)c->atom_struc.p;
  B.meta = (const StrucMeta*)c->meta.p;
  B.imgs = (const ImgEntry*)c->imgs.p;
  B.sfrac = (float4*)c->sfrac.p;
  B.sfloor = (int4*)c->sfloor.p;
  B.nb_j = (int*)c->nb_j.p;
  B.nb_r = (float4*)c->nb_r.p;
  B.nb_code = (int*)c->nb_code.p;
  B.nb_t = (unsigned char*)c->nb_t.p;
  B.nb_cnt = (int*)c->nb_cnt.p;
  B.ncells = U.ncells;
  if (U.ncells > 0) {
    B.cell_cnt = (int*)c->cell_cnt.p;
    B.cell_start = (int*)c->cell_start.p;
    B.cell_atoms = (int*)c->cell_atoms.p;
    B.atom_cell = (int*)c->atom_cell.p;
    B.cell_of = (int*)c->cell_of.p;
    B.sfrac_c = (float4*)c->sfrac_c.p;
    B.sfloor_c = (int4*)c->sfloor_c.p;
  }
  B.G = (float*)c->G.p;
  B.dEdG = (float*)c->dEdG.p;
  B.mom = (float*)c->mom.p;
  B.gstride = c->gstride;
  B.eatom = (float*)c->eatom.p;
  B.perm = (int*)c->perm.p;
  B.type_count = (int*)c->type_count.p;
  B.facc = (long long*)c->facc.p;
  B.nb_order = (const int*)c->nb_order.p;
  B.at_order = (const int*)c->at_order.p;
  B.force = force;
  B.energy = energy;
  B.status = (int*)c->status.p;
  return B;
}

// Enqueues the pipeline for the whole batch (batched) or one structure at a time (plain).
int enqueue(nnpgpu_ctx* c, const Uploaded& U, const BatchDev& Ball, int flags, cudaStream_t st) {
  if (flags & NNPGPU_BATCHED) {
    const nnpgpu_ctx::GraphKey key(U.natoms, U.nstruc, U.cap, flags, c->buf_generation, U.ncells, Ball.posn, Ball.type, Ball.energy,
                                   Ball.force);
    auto it = c->graphs.find(key);
    if (it != c->graphs.end()) {
      const cudaError_t e = cudaGraphLaunch(it->second, st);
      if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphLaunch");
      return NNPGPU_OK;
    }
    // first run of a shape is a plain launch sequence; the second one is captured
    if (c->shapes_seen[key]++ == 0) return run_pipeline(c, Ball, flags, st);
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return cuda_fail(c, cudaGetLastError(), "capture");
    const int rc = run_pipeline(c, Ball, flags, st);
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != NNPGPU_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    cudaGraphExec_t ex = nullptr;
    const cudaError_t e2 = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return cuda_fail(c, e2, "cudaGraphInstantiate");
    c->graphs[key] = ex;
    const cudaError_t e3 = cudaGraphLaunch(ex, st);
    if (e3 != cudaSuccess) return cuda_fail(c, e3, "cudaGraphLaunch");
    return NNPGPU_OK;
  }
  for (int s = 0; s < U.nstruc; ++s) {
    BatchDev B = Ball;
    B.a0 = U.offsets[s];
    B.natoms = U.offsets[s + 1] - U.offsets[s];
    B.nb_order = nullptr;  // the orders cover the whole batch
    B.at_order = nullptr;
    B.s0 = s;
    B.nstruc = 1;
    const int rc = run_pipeline(c, B, flags, st);
    if (rc != NNPGPU_OK) return rc;
  }
  return NNPGPU_OK;
}

void accumulate_profile(nnpgpu_ctx* c, int flags) {
  if (!c->prof_on || !(flags & NNPGPU_BATCHED)) return;
  for (int k = 0; k < NNPGPU_NSTAGES; ++k) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->prof_ev[k], c->prof_ev[k + 1]) == cudaSuccess) {
      c->prof_ms[k] += ms;
      c->prof_n[k] += 1;
    } else {
      cudaGetLastError();
    }
  }
}

void drop_graphs(nnpgpu_ctx* c) {
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
}

// Reads the status words after the stream finished; returns OK, a retry request (>0 = new
// capacity) or an error.
int check_status(nnpgpu_ctx* c, const int* st_words, int cap) {
  if (getenv("NNPGPU_DEBUG")) {
    std::fprintf(stderr, "nnpgpu status:");
    for (int k = 0; k < ST_WORDS; ++k) std::fprintf(stderr, " %d", st_words[k]);
    std::fprintf(stderr, "\n");
  }
  if (st_words[ST_ERROR] & ERR_BAD_POSITION) return set_error(c, NNPGPU_ERR_INVALID, "non-finite atom position");
  if (st_words[ST_ERROR] & ERR_BAD_TYPE) return set_error(c, NNPGPU_ERR_INVALID, "species index out of range");
  if (st_words[ST_ERROR] & ERR_FORCE_RANGE)
    return set_error(c, NNPGPU_ERR_INVALID, "a force contribution is not finite or above 1e9 eV/A (outside the fixed-point force sums)");
  if (st_words[ST_ERROR] & ERR_DRAIN)
    return set_error(c, NNPGPU_ERR_TIMEOUT,
                     "a bounded wait on the device ran out and the kernel's own copies did not finish either (tensor-core network); "
                     "destroy this context");
  if (st_words[ST_ERROR] & ERR_TIMEOUT) return set_error(c, NNPGPU_ERR_TIMEOUT, "a bounded wait on the device ran out (tensor-core network)");
  if (st_words[ST_MAXCOUNT] > cap) {
    const int need = (st_words[ST_MAXCOUNT] + 31) / 32 * 32;
    if (need > 256) return set_error(c, NNPGPU_ERR_CAPACITY, "more than 256 neighbours within the cutoff for some atom");
    return need;
  }
  return 0;
}

}  // namespace

// ------------------------------------------------------------------------------------------ C ABI
extern "C" int nnpgpu_create(const char* potfile, const nnpgpu_opts* opts, nnpgpu_ctx** out) {
  if (!out) return NNPGPU_ERR_INVALID;
  *out = nullptr;
  nnpgpu_ctx* c = new nnpgpu_ctx();
  try {
    c->device = opts ? opts->device : 0;
    c->verbose = opts ? opts->verbose : 0;
    c->budget = opts ? opts->hbm_budget_bytes : 0;
    c->cap_hint = opts ? opts->max_neighbors : 0;
    if (!potfile) throw PotError(NNPGPU_ERR_INVALID, "no potential file");
    c->potfile = potfile;
    c->pot = read_potential(potfile);
    build_tables(c->pot, c->P, c->ne, c->nz);
    c->max_nin = 0;
    for (int t = 0; t < c->pot.ntypes; ++t) c->max_nin = std::max(c->max_nin, c->pot.nin[t]);
    c->gstride = (c->max_nin + 15) / 16 * 16;
  } catch (PotError& e) {
    const int code = e.code;
    c->err = e.what();
    *out = c;  // keep the context so that the caller can read the message
    return code;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= c->device) {
    cudaGetLastError();
    *out = c;
    return set_error(c, NNPGPU_ERR_CUDA, "no CUDA device available (the engine has no CPU fallback)");
  }
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    *out = c;
    return cuda_fail(c, e, "device set-up");
  }
  // FP32 network weights: per type and layer w (row-major), wt (transposed), b, plus inpw/inpb
  std::vector<float> host;
  std::vector<size_t> offs;
  auto push = [&](const std::vector<float>& v) {
    while (host.size() % 4) host.push_back(0.f);
    offs.push_back(host.size());
    host.insert(host.end(), v.begin(), v.end());
  };
  for (int t = 0; t < c->pot.ntypes; ++t) {
    const HNet& n = c->pot.nets[t];
    const int L = (int)n.nodes.size();
    for (int l = 0; l < L; ++l) {
      const int R = n.nodes[l], C = l == 0 ? n.nin : n.nodes[l - 1];
      std::vector<float> w(n.w[l].begin(), n.w[l].end()), wt((size_t)R * C), b(n.b[l].begin(), n.b[l].end());
      for (int r = 0; r < R; ++r)
        for (int q = 0; q < C; ++q) wt[(size_t)q * R + r] = (float)n.w[l][(size_t)r * C + q];
      push(w);
      push(wt);
      push(b);
    }
    push(std::vector<float>(n.inpw.begin(), n.inpw.end()));
    push(std::vector<float>(n.inpb.begin(), n.inpb.end()));
  }
  push(build_ang_tables(c->pot, c->P));
  c->netbytes = host.size() * sizeof(float);
  if (cudaMalloc(&c->netbuf, c->netbytes) != cudaSuccess) {
    cudaGetLastError();
    *out = c;
    return set_error(c, NNPGPU_ERR_OOM, "could not allocate network weights");
  }
  c->used += c->netbytes;
  cudaMemcpy(c->netbuf, host.data(), c->netbytes, cudaMemcpyHostToDevice);
  size_t k = 0;
  const float* base = (const float*)c->netbuf;
  for (int t = 0; t < c->pot.ntypes; ++t) {
    const HNet& n = c->pot.nets[t];
    NetP& p = c->nets.net[t];
    p.nin = n.nin;
    p.nlayer = (int)n.nodes.size();
    p.act = n.act;
    for (int l = 0; l < p.nlayer; ++l) {
      p.nodes[l] = n.nodes[l];
      p.w[l] = base + offs[k++];
      p.wt[l] = base + offs[k++];
      p.b[l] = base + offs[k++];
    }
    p.inpw = base + offs[k++];
    p.inpb = base + offs[k++];
    p.outw = (float)n.outw[0];
    p.outb = (float)n.outb[0];
    p.evac = c->pot.types[t].energy;
  }
  c->P.atab = base + offs[k++];
  prepare_tc_weights(c);
  *out = c;
  return NNPGPU_OK;
}

extern "C" void nnpgpu_destroy(nnpgpu_ctx* c) {
  if (!c) return;
  c->serving.reset();
  drop_graphs(c);
  DevBuf* bufs[] = {&c->posn, &c->type, &c->atom_struc, &c->meta, &c->imgs, &c->sfrac, &c->sfloor, &c->nb_j, &c->nb_r, &c->nb_code, &c->nb_cnt,
                    &c->G, &c->dEdG, &c->eatom, &c->perm, &c->type_count, &c->facc, &c->nb_order, &c->at_order, &c->force, &c->energy,
                    &c->status, &c->cell_cnt, &c->cell_start, &c->cell_atoms, &c->atom_cell, &c->cell_of, &c->mom, &c->nb_t,
                    &c->tr_eref, &c->tr_dcdo, &c->tr_err, &c->tr_part, &c->tr_grad, &c->symm_in, &c->tr_fref, &c->tr_t,
                    &c->tr_fatom, &c->tr_fstruc, &c->tr_u, &c->sfrac_c, &c->sfloor_c};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  if (c->netbuf) cudaFree(c->netbuf);
  if (c->tcbuf) cudaFree(c->tcbuf);
  if (c->h_meta.p) cudaFreeHost(c->h_meta.p);
  if (c->h_in.p) cudaFreeHost(c->h_in.p);
  if (c->h_out.p) cudaFreeHost(c->h_out.p);
  for (int k = 0; k <= NNPGPU_NSTAGES; ++k)
    if (c->prof_ev[k]) cudaEventDestroy(c->prof_ev[k]);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int nnpgpu_profile_enable(nnpgpu_ctx* c, int on) {
  if (!c || !c->stream) return NNPGPU_ERR_INVALID;
  if (on && !c->prof_ev[0])
    for (int k = 0; k <= NNPGPU_NSTAGES; ++k)
      if (cudaEventCreate(&c->prof_ev[k]) != cudaSuccess) return cuda_fail(c, cudaGetLastError(), "cudaEventCreate");
  // graphs captured with a different tracing setting must not be replayed
  if ((on != 0) != c->prof_on) {
    drop_graphs(c);
    c->shapes_seen.clear();
  }
  c->prof_on = on != 0;
  for (int k = 0; k < NNPGPU_NSTAGES; ++k) { c->prof_ms[k] = 0; c->prof_n[k] = 0; }
  return NNPGPU_OK;
}

extern "C" int nnpgpu_profile_read(const nnpgpu_ctx* c, int stage, double* total_ms, long long* count) {
  if (!c || stage < 0 || stage >= NNPGPU_NSTAGES) return NNPGPU_ERR_INVALID;
  if (total_ms) *total_ms = c->prof_ms[stage];
  if (count) *count = c->prof_n[stage];
  return NNPGPU_OK;
}

extern "C" const char* nnpgpu_profile_stage_name(int stage) {
  static const char* names[NNPGPU_NSTAGES] = {"neighbors", "force_clear", "descriptors", "networks", "chain_rule", "forces_energy"};
  return (stage >= 0 && stage < NNPGPU_NSTAGES) ? names[stage] : "?";
}

extern "C" const char* nnpgpu_last_error(const nnpgpu_ctx* c) { return c ? c->err.c_str() : "no context"; }
extern "C" int nnpgpu_ntypes(const nnpgpu_ctx* c) { return c ? c->pot.ntypes : 0; }
extern "C" int nnpgpu_type_index(const nnpgpu_ctx* c, const char* name) {
  if (!c || !name) return -1;
  auto it = c->pot.index.find(name);
  return it == c->pot.index.end() ? -1 : it->second;
}
extern "C" double nnpgpu_cutoff(const nnpgpu_ctx* c) { return c ? c->pot.rc : 0.0; }
extern "C" int nnpgpu_ninput(const nnpgpu_ctx* c, int type) {
  if (!c || type < 0 || type >= c->pot.ntypes) return -1;
  return c->pot.nin[type];
}

// True for page-locked host memory (cudaMallocHost, cudaHostRegister, a pinned torch tensor):
// copies from and to it are DMA transfers that need no staging.
static bool host_pinned(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

static int compute_impl(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* posn, const int* species, const double* cell,
                        int flags, double* energy, double* force, float* symm, bool device_io, cudaStream_t st,
                        const SkinRef* skins = nullptr) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  cudaSetDevice(c->device);
  if (!st) st = c->stream;
  if ((flags & NNPGPU_ENERGY) && !energy) return set_error(c, NNPGPU_ERR_INVALID, "energy output missing");
  if ((flags & NNPGPU_FORCE) && !force) return set_error(c, NNPGPU_ERR_INVALID, "force output missing");
  if ((flags & NNPGPU_SYMM) && !symm) return set_error(c, NNPGPU_ERR_INVALID, "symm output missing");
  int total = 0;
  for (int s = 0; s < nstruc; ++s) total += natoms ? natoms[s] : 0;
  if (total > 0 && (!posn || !species)) return set_error(c, NNPGPU_ERR_INVALID, "positions or species missing");
  // species outside the potential are flagged on the device (every kernel clamps before it
  // indexes by species) and fail the call with the same error: no serial pass over the atoms here
  int cap = std::min(256, estimate_cap(c, nstruc, natoms, cell));  // the descriptor kernels take at most 256 slots
  // page-locked caller buffers are read and written by DMA directly; others go through the
  // context's pinned staging buffers
  const bool direct_in = !device_io && total > 0 && host_pinned(posn) && host_pinned(species);
  const bool direct_force = !device_io && (flags & NNPGPU_FORCE) && total > 0 && host_pinned(force);
  for (int attempt = 0; attempt < 4; ++attempt) {
    Uploaded U;
    int rc = prepare(c, nstruc, natoms, cell, cap, U, st, skins);
    if (rc != NNPGPU_OK) return rc;
    const size_t N = total;
    const double* dposn = posn;
    const int* dtype = species;
    if (direct_in) {
      cudaMemcpyAsync(c->posn.p, posn, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(c->type.p, species, sizeof(int) * N, cudaMemcpyHostToDevice, st);
      dposn = (const double*)c->posn.p;
      dtype = (const int*)c->type.p;
    } else if (!device_io) {
      // stage inputs through pinned memory
      const size_t in_bytes = sizeof(double) * 3 * N + sizeof(int) * N;
      if (!ensure_host(c, c->h_in, in_bytes + 64)) return set_error(c, NNPGPU_ERR_OOM, "pinned host allocation failed");
      char* h = (char*)c->h_in.p;
      std::memcpy(h, posn, sizeof(double) * 3 * N);
      std::memcpy(h + sizeof(double) * 3 * N, species, sizeof(int) * N);
      cudaMemcpyAsync(c->posn.p, h, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(c->type.p, h + sizeof(double) * 3 * N, sizeof(int) * N, cudaMemcpyHostToDevice, st);
      dposn = (const double*)c->posn.p;
      dtype = (const int*)c->type.p;
    }
    double* denergy = device_io ? energy : (double*)c->energy.p;
    double* dforce = (device_io && force) ? force : (double*)c->force.p;
    BatchDev B = batch_view(c, U, dposn, dtype, denergy ? denergy : (double*)c->energy.p, dforce);
    rc = enqueue(c, U, B, flags, st);
    if (rc != NNPGPU_OK) return rc;
    // outputs
    int hstat[ST_WORDS];
    if (!device_io) {
      const size_t out_bytes = sizeof(double) * (nstruc + 3 * N) + sizeof(int) * ST_WORDS;
      if (!ensure_host(c, c->h_out, out_bytes + 64)) return set_error(c, NNPGPU_ERR_OOM, "pinned host allocation failed");
      char* h = (char*)c->h_out.p;
      if (flags & NNPGPU_ENERGY) cudaMemcpyAsync(h, c->energy.p, sizeof(double) * nstruc, cudaMemcpyDeviceToHost, st);
      if (flags & NNPGPU_FORCE)
        cudaMemcpyAsync(direct_force ? (void*)force : (void*)(h + sizeof(double) * nstruc), c->force.p, sizeof(double) * 3 * N,
                        cudaMemcpyDeviceToHost, st);
      cudaMemcpyAsync(h + sizeof(double) * (nstruc + 3 * N), c->status.p, sizeof(int) * ST_WORDS, cudaMemcpyDeviceToHost, st);
      if (flags & NNPGPU_SYMM)
        cudaMemcpy2DAsync(symm, sizeof(float) * c->max_nin, c->G.p, sizeof(float) * c->gstride, sizeof(float) * c->max_nin, N,
                          cudaMemcpyDeviceToHost, st);
      const cudaError_t e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return cuda_fail(c, e, "compute");
      std::memcpy(hstat, h + sizeof(double) * (nstruc + 3 * N), sizeof(hstat));
      const int need = check_status(c, hstat, U.cap);
      if (need < 0) return need;
      if (need > 0) { cap = need; c->cap_hint = std::max(c->cap_hint, need); continue; }
      if (flags & NNPGPU_ENERGY) std::memcpy(energy, h, sizeof(double) * nstruc);
      if ((flags & NNPGPU_FORCE) && !direct_force) std::memcpy(force, h + sizeof(double) * nstruc, sizeof(double) * 3 * N);
      accumulate_profile(c, flags);
      return NNPGPU_OK;
    }
    if (flags & NNPGPU_SYMM)
      cudaMemcpy2DAsync(symm, sizeof(float) * c->max_nin, c->G.p, sizeof(float) * c->gstride, sizeof(float) * c->max_nin, N,
                        cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(hstat, c->status.p, sizeof(hstat), cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(c, e, "compute");
    const int need = check_status(c, hstat, U.cap);
    if (need < 0) return need;
    if (need > 0) { cap = need; c->cap_hint = std::max(c->cap_hint, need); continue; }
    accumulate_profile(c, flags);
    return NNPGPU_OK;
  }
  return set_error(c, NNPGPU_ERR_CAPACITY, "neighbour capacity retries exhausted");
}

namespace nnpgpu {
int compute_host(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* posn, const int* species, const double* cell, int flags,
                 double* energy, double* force, float* symm, const SkinRef* skins) {
  return compute_impl(c, nstruc, natoms, posn, species, cell, flags, energy, force, symm, false, nullptr, skins);
}

int compute_device_skins(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* d_posn, const int* d_species, const double* cell,
                         int flags, double* d_energy, double* d_force, cudaStream_t st, const SkinRef* skins) {
  return compute_impl(c, nstruc, natoms, d_posn, d_species, cell, flags, d_energy, d_force, nullptr, true, st, skins);
}

int build_skin(nnpgpu_ctx* c, int natoms, const double* posn, const double* cell, double rc_skin, int skin_cap, int* d_j, int* d_code,
               int* d_cnt, float4* d_r, int* max_count, bool posn_on_device) {
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  *max_count = 0;
  Uploaded U;
  // geometry for the larger cutoff (shells follow rc_skin); buffers sized for this structure
  const double saved = c->pot.rc;
  c->pot.rc = rc_skin;
  int rc = prepare(c, 1, &natoms, cell, skin_cap, U, st);
  c->pot.rc = saved;
  if (rc != NNPGPU_OK) return rc;
  cudaMemcpyAsync(c->posn.p, posn, sizeof(double) * 3 * natoms, posn_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
  BatchDev B = batch_view(c, U, (const double*)c->posn.p, nullptr, (double*)c->energy.p, (double*)c->force.p);
  B.rc = rc_skin;
  B.nb_t = nullptr;  // skin lists keep no species
  B.nb_j = d_j;
  B.nb_code = d_code;
  B.nb_cnt = d_cnt;
  B.nb_r = d_r;
  launch_neighbors(B, st);
  int hstat[ST_WORDS];
  cudaMemcpyAsync(hstat, c->status.p, sizeof(hstat), cudaMemcpyDeviceToHost, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "skin list");
  if (hstat[ST_ERROR]) return set_error(c, NNPGPU_ERR_INVALID, "invalid positions in a resident structure");
  if (hstat[ST_MAXCOUNT] > skin_cap) {
    *max_count = hstat[ST_MAXCOUNT];
    return NNPGPU_ERR_CAPACITY;
  }
  return NNPGPU_OK;
}
}  // namespace nnpgpu

extern "C" int nnpgpu_compute(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* posn, const int* species, const double* cell,
                              int flags, double* energy, double* force, float* symm) {
  return compute_impl(c, nstruc, natoms, posn, species, cell, flags, energy, force, symm, false, nullptr);
}

extern "C" int nnpgpu_compute_device(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* d_posn, const int* d_species,
                                     const double* cell, int flags, double* d_energy, double* d_force, float* d_symm, void* stream) {
  return compute_impl(c, nstruc, natoms, d_posn, d_species, cell, flags, d_energy, d_force, d_symm, true, (cudaStream_t)stream);
}

// Neighbour list of one structure at cutoff rc (the potential's when rc <= 0), at most
// max_slots device slots per atom.
static int neighbors_impl(nnpgpu_ctx* c, double rc_req, int max_slots, int natoms, const double* posn, const double* cell, int cap,
                          int* count, int* index, float* r, unsigned char* mn, int* shift) {
  if (!c || natoms < 0 || cap <= 0 || (natoms > 0 && (!posn || !count))) return set_error(c, NNPGPU_ERR_INVALID, "invalid arguments");
  if (!(rc_req <= 0) && !(rc_req < 1e6)) return set_error(c, NNPGPU_ERR_INVALID, "invalid cutoff");
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  const double zero[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const double* cl = cell ? cell : zero;
  // the geometry set-up (shells, cell grid) and the capacity estimate follow the requested cutoff
  const double saved = c->pot.rc;
  if (rc_req > 0) c->pot.rc = rc_req;
  const int est = estimate_cap(c, 1, &natoms, cl);
  const int dcap = std::min(max_slots, std::max(cap, est));
  Uploaded U;
  int rc = prepare(c, 1, &natoms, cl, (dcap + 31) / 32 * 32, U, st);
  c->pot.rc = saved;
  if (rc != NNPGPU_OK) return rc;
  cudaMemcpyAsync(c->posn.p, posn, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice, st);
  BatchDev B = batch_view(c, U, (const double*)c->posn.p, nullptr, (double*)c->energy.p, (double*)c->force.p);
  if (rc_req > 0) B.rc = rc_req;
  launch_neighbors(B, st);
  std::vector<int> hj((size_t)natoms * U.cap), hc((size_t)natoms * U.cap), hn(natoms);
  std::vector<float4> hr((size_t)natoms * U.cap);
  std::vector<int4> hf(natoms);  // the atoms' integer floors: the codes keep translations modulo 1024
  int hstat[ST_WORDS];
  cudaMemcpyAsync(hj.data(), c->nb_j.p, sizeof(int) * hj.size(), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hc.data(), c->nb_code.p, sizeof(int) * hc.size(), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hr.data(), c->nb_r.p, sizeof(float4) * hr.size(), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hn.data(), c->nb_cnt.p, sizeof(int) * natoms, cudaMemcpyDeviceToHost, st);
  if (shift) cudaMemcpyAsync(hf.data(), c->sfloor.p, sizeof(int4) * natoms, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hstat, c->status.p, sizeof(hstat), cudaMemcpyDeviceToHost, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "neighbors");
  if (hstat[ST_ERROR] & ERR_BAD_POSITION) return set_error(c, NNPGPU_ERR_INVALID, "non-finite atom position");
  int status = NNPGPU_OK;
  for (int i = 0; i < natoms; ++i) {
    count[i] = hn[i];
    if (hn[i] > cap) status = set_error(c, NNPGPU_ERR_CAPACITY, "neighbour list longer than cap");
    const int n = std::min(std::min(hn[i], cap), U.cap);
    for (int s = 0; s < n; ++s) {
      const size_t src = (size_t)i * U.cap + s, dst = (size_t)i * cap + s;
      if (index) index[dst] = hj[src];
      if (r) { r[4 * dst] = hr[src].x; r[4 * dst + 1] = hr[src].y; r[4 * dst + 2] = hr[src].z; r[4 * dst + 3] = hr[src].w; }
      if (mn) mn[dst] = code_min(hc[src]) ? 1 : 0;
      if (shift) {
        const int j = hj[src];
        const int4 fi = hf[i], fj = (j >= 0 && j < natoms) ? hf[j] : hf[i];
        shift[3 * dst] = code_t_full(hc[src], 0, fi.x - fj.x);
        shift[3 * dst + 1] = code_t_full(hc[src], 1, fi.y - fj.y);
        shift[3 * dst + 2] = code_t_full(hc[src], 2, fi.z - fj.z);
      }
    }
  }
  if (status == NNPGPU_OK && hstat[ST_MAXCOUNT] > U.cap)
    status = set_error(c, NNPGPU_ERR_CAPACITY, "neighbour list longer than " + std::to_string(max_slots));
  return status;
}

// Launch-shape autotuner.  Coordinate descent over the knobs of TuneCfg: each candidate value is
// timed on the caller's batch from the stage events recorded inside the captured launch
// sequence (best of `reps` graph replays after a warm-up run and the capture run), and the
// fastest value is kept before the next knob is tried.
static int tune_stage(nnpgpu_ctx* c, int* knob, const int* cand, int ncand, int stage, int nstruc, const int* natoms, const double* posn,
                      const int* species, const double* cell, int flags, double* energy, double* force, std::string& rep,
                      const char* name) {
  const int keep = *knob;
  int best = keep;
  double best_ms = 1e30;
  char buf[64];
  rep += name;
  rep += " {";
  for (int k = 0; k < ncand; ++k) {
    *knob = cand[k];
    drop_graphs(c);
    c->shapes_seen.clear();
    for (int w = 0; w < 2; ++w) {  // first run of the shape, then the captured run
      const int rc = compute_impl(c, nstruc, natoms, posn, species, cell, flags, energy, force, nullptr, false, nullptr);
      if (rc != NNPGPU_OK) { *knob = keep; return rc; }
    }
    double ms = 1e30;
    for (int r = 0; r < 3; ++r) {
      c->prof_ms[stage] = 0;
      c->prof_n[stage] = 0;
      const int rc = compute_impl(c, nstruc, natoms, posn, species, cell, flags, energy, force, nullptr, false, nullptr);
      if (rc != NNPGPU_OK) { *knob = keep; return rc; }
      if (c->prof_n[stage] > 0) ms = std::min(ms, c->prof_ms[stage] / (double)c->prof_n[stage]);
    }
    std::snprintf(buf, sizeof(buf), "%s%d: %.4f ms", k ? ", " : "", cand[k], ms);
    rep += buf;
    if (ms < best_ms) { best_ms = ms; best = cand[k]; }
  }
  *knob = best;
  std::snprintf(buf, sizeof(buf), "} -> %d; ", best);
  rep += buf;
  return NNPGPU_OK;
}

extern "C" int nnpgpu_autotune(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* posn, const int* species, const double* cell,
                               int flags, char* report, int report_len) {
  if (!c || nstruc <= 0 || !natoms || !posn || !species || !cell) return set_error(c, NNPGPU_ERR_INVALID, "invalid arguments");
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  flags = (flags & (NNPGPU_BF16 | NNPGPU_FORCE | NNPGPU_NO_VACUUM)) | NNPGPU_ENERGY | NNPGPU_BATCHED;
  size_t total = 0;
  for (int s = 0; s < nstruc; ++s) total += natoms[s] > 0 ? natoms[s] : 0;
  std::vector<double> energy(nstruc), force((flags & NNPGPU_FORCE) ? 3 * std::max<size_t>(total, 1) : 0);
  double* fp = (flags & NNPGPU_FORCE) ? force.data() : nullptr;
  const bool was_on = c->prof_on;
  int rc = nnpgpu_profile_enable(c, 1);
  if (rc != NNPGPU_OK) return rc;
  std::string rep;
  static const int warps[] = {1, 2, 4};
  static const int tiles[] = {16, 32, 64};
  rc = tune_stage(c, &c->tune.warps_nbr, warps, 3, 0, nstruc, natoms, posn, species, cell, flags, energy.data(), fp, rep, "warps_nbr");
  if (rc == NNPGPU_OK)
    rc = tune_stage(c, &c->tune.warps_symm, warps, 3, 2, nstruc, natoms, posn, species, cell, flags, energy.data(), fp, rep, "warps_symm");
  if (rc == NNPGPU_OK && !(flags & NNPGPU_BF16))
    rc = tune_stage(c, &c->tune.nn_tile, tiles, 3, 3, nstruc, natoms, posn, species, cell, flags, energy.data(), fp, rep, "nn_tile");
  if (rc == NNPGPU_OK && (flags & NNPGPU_FORCE))
    rc = tune_stage(c, &c->tune.warps_force, warps, 3, 4, nstruc, natoms, posn, species, cell, flags, energy.data(), fp, rep, "warps_force");
  const std::string err = c->err;
  nnpgpu_profile_enable(c, was_on ? 1 : 0);  // also drops the graphs captured while tuning
  drop_graphs(c);
  c->shapes_seen.clear();
  if (rc != NNPGPU_OK) {
    c->err = err;
    return rc;
  }
  if (report && report_len > 0) {
    std::snprintf(report, (size_t)report_len, "%s", rep.c_str());
  }
  return NNPGPU_OK;
}

extern "C" int nnpgpu_set_wait_limit(nnpgpu_ctx* c, int polls) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (polls < 0) return set_error(c, NNPGPU_ERR_INVALID, "wait limit: polls must be >= 0");
  c->tc_wait_limit = polls;
  drop_graphs(c);  // captured sequences hold the old limit
  c->shapes_seen.clear();
  return NNPGPU_OK;
}

extern "C" int nnpgpu_get_tune(const nnpgpu_ctx* c, int* warps_nbr, int* warps_symm, int* warps_force, int* nn_tile) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (warps_nbr) *warps_nbr = c->tune.warps_nbr;
  if (warps_symm) *warps_symm = c->tune.warps_symm;
  if (warps_force) *warps_force = c->tune.warps_force;
  if (nn_tile) *nn_tile = c->tune.nn_tile;
  return NNPGPU_OK;
}

extern "C" int nnpgpu_set_tune(nnpgpu_ctx* c, int warps_nbr, int warps_symm, int warps_force, int nn_tile) {
  if (!c) return NNPGPU_ERR_INVALID;
  auto ok_w = [](int w) { return w == 1 || w == 2 || w == 4; };
  if (!ok_w(warps_nbr) || !ok_w(warps_symm) || !ok_w(warps_force) || !(nn_tile == 16 || nn_tile == 32 || nn_tile == 64))
    return set_error(c, NNPGPU_ERR_INVALID, "launch shapes: warps 1, 2 or 4; FP32 network tile 16, 32 or 64");
  c->tune.warps_nbr = warps_nbr;
  c->tune.warps_symm = warps_symm;
  c->tune.warps_force = warps_force;
  c->tune.nn_tile = nn_tile;
  drop_graphs(c);  // captured sequences hold the old shapes
  c->shapes_seen.clear();
  return NNPGPU_OK;
}

static int net_param_count(const nnpgpu_ctx* c, int t) {
  const HNet& n = c->pot.nets[t];
  int s = 0;
  for (size_t l = 0; l < n.nodes.size(); ++l) s += n.nodes[l] * (1 + (l == 0 ? n.nin : n.nodes[l - 1]));
  return s;
}

extern "C" int nnpgpu_nparams(const nnpgpu_ctx* c, int type) {
  if (!c || type < 0 || type >= c->pot.ntypes) return -1;
  return net_param_count(c, type);
}

// The energy trainer's batch error and gradient (NNPTE::error, src/nnp/nnpte.cpp:870-921): one
// batched energy pass (FP32 networks, energies without the vacuum energies), then the loss and the
// parameter gradient on the device (network.cu).
extern "C" int nnpgpu_get_params(const nnpgpu_ctx* c, int type, double* p) {
  if (!c || type < 0 || type >= c->pot.ntypes || !p) return NNPGPU_ERR_INVALID;
  const HNet& n = c->pot.nets[type];
  size_t k = 0;
  for (size_t l = 0; l < n.nodes.size(); ++l)
    for (int r = 0; r < n.nodes[l]; ++r) p[k++] = n.b[l][r];
  for (size_t l = 0; l < n.nodes.size(); ++l) {
    const int C = l == 0 ? n.nin : n.nodes[l - 1];
    for (int m = 0; m < C; ++m)
      for (int r = 0; r < n.nodes[l]; ++r) p[k++] = n.w[l][(size_t)r * C + m];
  }
  return NNPGPU_OK;
}

extern "C" int nnpgpu_set_params(nnpgpu_ctx* c, int type, const double* p) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (type < 0 || type >= c->pot.ntypes || !p) return set_error(c, NNPGPU_ERR_INVALID, "set_params: invalid type or parameters");
  if (c->serving) return set_error(c, NNPGPU_ERR_BUSY, "set_params: stop serving first");
  HNet& n = c->pot.nets[type];
  const int np = net_param_count(c, type);
  for (int k = 0; k < np; ++k)
    if (!std::isfinite(p[k])) return set_error(c, NNPGPU_ERR_INVALID, "set_params: non-finite parameter");
  size_t k = 0;
  for (size_t l = 0; l < n.nodes.size(); ++l)
    for (int r = 0; r < n.nodes[l]; ++r) n.b[l][r] = p[k++];
  for (size_t l = 0; l < n.nodes.size(); ++l) {
    const int C = l == 0 ? n.nin : n.nodes[l - 1];
    for (int m = 0; m < C; ++m)
      for (int r = 0; r < n.nodes[l]; ++r) n.w[l][(size_t)r * C + m] = p[k++];
  }
  if (!c->netbuf) return NNPGPU_OK;  // no device: the host copy is all there is
  // device copies: FP32 weights in place, the tensor-core blob packed anew; captured graphs hold
  // the output bias and the blob pointer by value, so they are rebuilt on the next calls
  cudaSetDevice(c->device);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  const NetP& q = c->nets.net[type];
  for (size_t l = 0; l < n.nodes.size() && e == cudaSuccess; ++l) {
    const int R = n.nodes[l], C = l == 0 ? n.nin : n.nodes[l - 1];
    std::vector<float> w((size_t)R * C), wt((size_t)R * C), b(R);
    for (int r = 0; r < R; ++r) {
      b[r] = (float)n.b[l][r];
      for (int m = 0; m < C; ++m) {
        w[(size_t)r * C + m] = (float)n.w[l][(size_t)r * C + m];
        wt[(size_t)m * R + r] = (float)n.w[l][(size_t)r * C + m];
      }
    }
    e = cudaMemcpy((void*)q.w[l], w.data(), sizeof(float) * w.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy((void*)q.wt[l], wt.data(), sizeof(float) * wt.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy((void*)q.b[l], b.data(), sizeof(float) * b.size(), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "set_params");
  drop_graphs(c);
  c->shapes_seen.clear();
  if (c->tcbuf) {
    cudaFree(c->tcbuf);
    c->used -= c->tcbytes;
    c->tcbuf = nullptr;
    c->tcbytes = 0;
  }
  prepare_tc_weights(c);  // leaves the tensor-core path off if the networks do not fit it, as at creation
  return NNPGPU_OK;
}

extern "C" int nnpgpu_write_potential(nnpgpu_ctx* c, const char* path) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (!path) return set_error(c, NNPGPU_ERR_INVALID, "write_potential: no file");
  try {
    write_potential(c->pot, path);
  } catch (PotError& e) {
    return set_error(c, e.code, e.what());
  }
  return NNPGPU_OK;
}

extern "C" int nnpgpu_train_grad(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* posn, const int* species, const double* cell,
                                 const double* energy_ref, int loss, double delta, double* error, double* grad) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  if (nstruc <= 0 || !energy_ref || !error || !grad) return set_error(c, NNPGPU_ERR_INVALID, "train: invalid arguments");
  if (loss < 0 || loss > 3) return set_error(c, NNPGPU_ERR_INVALID, "train: loss must be 0 (MSE), 1 (MAE), 2 (HUBER) or 3 (ASINH)");
  if ((loss >= 2) && !(delta > 0)) return set_error(c, NNPGPU_ERR_INVALID, "train: HUBER and ASINH need delta > 0");
  for (int s = 0; s < nstruc; ++s)
    if (!natoms || natoms[s] <= 0) return set_error(c, NNPGPU_ERR_INVALID, "train: every structure needs atoms");
  std::vector<double> e(nstruc);
  int rc = compute_impl(c, nstruc, natoms, posn, species, cell, NNPGPU_ENERGY | NNPGPU_BATCHED | NNPGPU_NO_VACUUM, e.data(), nullptr,
                        nullptr, false, nullptr);
  if (rc != NNPGPU_OK) return rc;
  cudaStream_t st = c->stream;
  int total = 0, maxp = 0;
  for (int t = 0; t < c->pot.ntypes; ++t) {
    total += net_param_count(c, t);
    maxp = std::max(maxp, net_param_count(c, t));
  }
  const int pstride = (maxp + 3) / 4 * 4;
  const Uploaded& U = c->meta_cache.U;
  const int tiles = train_tiles(U.natoms, c->pot.ntypes);
  if (!ensure(c, c->tr_eref, sizeof(double) * nstruc) || !ensure(c, c->tr_dcdo, sizeof(double) * nstruc) ||
      !ensure(c, c->tr_err, sizeof(double) * 2) || !ensure(c, c->tr_part, sizeof(float) * (size_t)tiles * pstride) ||
      !ensure(c, c->tr_grad, sizeof(double) * total))
    return set_error(c, NNPGPU_ERR_OOM, "train: device allocation failed or HBM budget exceeded");
  BatchDev B = batch_view(c, U, (const double*)c->posn.p, (const int*)c->type.p, (double*)c->energy.p, (double*)c->force.p);
  cudaMemcpyAsync(c->tr_eref.p, energy_ref, sizeof(double) * nstruc, cudaMemcpyHostToDevice, st);
  if (launch_train(B, c->nets, c->pot.ntypes, (const double*)c->tr_eref.p, loss, delta, (double*)c->tr_dcdo.p, (double*)c->tr_err.p,
                   (float*)c->tr_part.p, pstride, (double*)c->tr_grad.p, maxp, st) != 0)
    return set_error(c, NNPGPU_ERR_UNSUPPORTED, "train: networks too wide for the gradient kernel's shared memory");
  cudaMemcpyAsync(error, c->tr_err.p, sizeof(double) * 2, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(grad, c->tr_grad.p, sizeof(double) * total, cudaMemcpyDeviceToHost, st);
  const cudaError_t err = cudaStreamSynchronize(st);
  if (err != cudaSuccess) return cuda_fail(c, err, "train");
  return NNPGPU_OK;
}

extern "C" int nnpgpu_train_force_grad(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* posn, const int* species,
                                       const double* cell, const double* energy_ref, const double* force_ref, double beta, int loss,
                                       double delta, double* error, double* grad) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  if (nstruc <= 0 || !energy_ref || !force_ref || !error || !grad) return set_error(c, NNPGPU_ERR_INVALID, "train_force: invalid arguments");
  if (loss < 0 || loss > 3) return set_error(c, NNPGPU_ERR_INVALID, "train_force: loss must be 0 (MSE), 1 (MAE), 2 (HUBER) or 3 (ASINH)");
  if ((loss >= 2) && !(delta > 0)) return set_error(c, NNPGPU_ERR_INVALID, "train_force: HUBER and ASINH need delta > 0");
  if (!(beta >= 0) || !std::isfinite(beta)) return set_error(c, NNPGPU_ERR_INVALID, "train_force: beta must be finite and >= 0");
  for (int I = 0; I < c->pot.ntypes; ++I)
    for (int q = 0; q < NB_MAX; ++q)
      if (c->P.ang[I][q].n > 0 && c->P.ang[I][q].fn)
        return set_error(c, NNPGPU_ERR_UNSUPPORTED,
                         "train_force: angular blocks with a real zeta or more than 4 widths or 2 lambdas are not implemented in the "
                         "force trainer's tangent pass (energies and forces support them)");
  size_t N = 0;
  for (int s = 0; s < nstruc; ++s) {
    if (!natoms || natoms[s] <= 0) return set_error(c, NNPGPU_ERR_INVALID, "train_force: every structure needs atoms");
    N += (size_t)natoms[s];
  }
  std::vector<double> e(nstruc), F(3 * N);
  int rc = compute_impl(c, nstruc, natoms, posn, species, cell, NNPGPU_ENERGY | NNPGPU_FORCE | NNPGPU_BATCHED | NNPGPU_NO_VACUUM, e.data(),
                        F.data(), nullptr, false, nullptr);
  if (rc != NNPGPU_OK) return rc;
  cudaStream_t st = c->stream;
  int total = 0, maxp = 0;
  for (int t = 0; t < c->pot.ntypes; ++t) {
    total += net_param_count(c, t);
    maxp = std::max(maxp, net_param_count(c, t));
  }
  const int pstride = (maxp + 3) / 4 * 4;
  const Uploaded& U = c->meta_cache.U;
  const int tiles = std::max(train_tiles(U.natoms, c->pot.ntypes), train_force_tiles(U.natoms, c->pot.ntypes));
  if (!ensure(c, c->tr_eref, sizeof(double) * nstruc) || !ensure(c, c->tr_dcdo, sizeof(double) * nstruc) ||
      !ensure(c, c->tr_err, sizeof(double) * 3) || !ensure(c, c->tr_part, sizeof(float) * (size_t)tiles * pstride) ||
      !ensure(c, c->tr_grad, sizeof(double) * total) || !ensure(c, c->tr_fref, sizeof(double) * 3 * N) ||
      !ensure(c, c->tr_t, sizeof(float4) * N) || !ensure(c, c->tr_fatom, sizeof(double) * N) ||
      !ensure(c, c->tr_fstruc, sizeof(double) * nstruc) || !ensure(c, c->tr_u, sizeof(float) * N * c->gstride))
    return set_error(c, NNPGPU_ERR_OOM, "train_force: device allocation failed or HBM budget exceeded");
  BatchDev B = batch_view(c, U, (const double*)c->posn.p, (const int*)c->type.p, (double*)c->energy.p, (double*)c->force.p);
  cudaMemcpyAsync(c->tr_eref.p, energy_ref, sizeof(double) * nstruc, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->tr_fref.p, force_ref, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st);
  // energy term: loss, dc/dout and the gradient written into tr_grad
  if (launch_train(B, c->nets, c->pot.ntypes, (const double*)c->tr_eref.p, loss, delta, (double*)c->tr_dcdo.p, (double*)c->tr_err.p,
                   (float*)c->tr_part.p, pstride, (double*)c->tr_grad.p, maxp, st) != 0)
    return set_error(c, NNPGPU_ERR_UNSUPPORTED, "train_force: networks too wide for the gradient kernel's shared memory");
  // force term: residual weights, loss, descriptor-space weights, then the gradient added
  launch_train_force_loss(B, (const double*)c->tr_fref.p, beta, (float4*)c->tr_t.p, (double*)c->tr_fatom.p, (double*)c->tr_fstruc.p,
                          (double*)c->tr_err.p, st);
  if (launch_tangent(B, c->P, c->ne, c->nz, (const float4*)c->tr_t.p, (float*)c->tr_u.p, st) != 0)
    return set_error(c, NNPGPU_ERR_UNSUPPORTED, "train_force: no tangent kernel instance");
  if (launch_train_force(B, c->nets, c->pot.ntypes, (const float*)c->tr_u.p, (float*)c->tr_part.p, pstride, (double*)c->tr_grad.p, maxp,
                         st) != 0)
    return set_error(c, NNPGPU_ERR_UNSUPPORTED, "train_force: networks too wide for the force-gradient kernel's shared memory");
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return cuda_fail(c, le, "train_force launch");
  cudaMemcpyAsync(error, c->tr_err.p, sizeof(double) * 3, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(grad, c->tr_grad.p, sizeof(double) * total, cudaMemcpyDeviceToHost, st);
  const cudaError_t err = cudaStreamSynchronize(st);
  if (err != cudaSuccess) return cuda_fail(c, err, "train_force");
  return NNPGPU_OK;
}

extern "C" int nnpgpu_energy_symm(nnpgpu_ctx* c, int nstruc, const int* natoms, const int* species, const double* symm, int symm_stride,
                                  int flags, double* energy) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  cudaSetDevice(c->device);
  if (nstruc < 0 || (nstruc > 0 && (!natoms || !energy))) return set_error(c, NNPGPU_ERR_INVALID, "energy_symm: invalid batch description");
  if (flags & ~(NNPGPU_BF16 | NNPGPU_NO_VACUUM))
    return set_error(c, NNPGPU_ERR_INVALID, "energy_symm: only NNPGPU_BF16 and NNPGPU_NO_VACUUM apply");
  if (symm_stride < c->max_nin) return set_error(c, NNPGPU_ERR_INVALID, "energy_symm: symm_stride below the largest input size");
  size_t total = 0;
  for (int s = 0; s < nstruc; ++s) {
    if (natoms[s] < 0) return set_error(c, NNPGPU_ERR_INVALID, "energy_symm: negative atom count");
    total += (size_t)natoms[s];
  }
  if (total > 0 && (!species || !symm)) return set_error(c, NNPGPU_ERR_INVALID, "energy_symm: species or descriptors missing");
  for (size_t a = 0; a < total; ++a)
    if (species[a] < 0 || species[a] >= c->pot.ntypes) return set_error(c, NNPGPU_ERR_INVALID, "energy_symm: species index out of range");
  if (nstruc == 0) return NNPGPU_OK;
  cudaStream_t st = c->stream;
  // no geometry: every structure is described as non-periodic, which only sets its atom range
  const std::vector<double> no_cell(9 * (size_t)nstruc, 0.0);
  Uploaded U;
  int rc = prepare(c, nstruc, natoms, no_cell.data(), 32, U, st);
  if (rc != NNPGPU_OK) return rc;
  if (!ensure(c, c->symm_in, sizeof(double) * std::max<size_t>(total, 1) * symm_stride))
    return set_error(c, NNPGPU_ERR_OOM, "energy_symm: device allocation failed or HBM budget exceeded");
  cudaMemcpyAsync(c->type.p, species, sizeof(int) * total, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(c->symm_in.p, symm, sizeof(double) * total * symm_stride, cudaMemcpyHostToDevice, st);
  BatchDev B = batch_view(c, U, (const double*)c->posn.p, (const int*)c->type.p, (double*)c->energy.p, (double*)c->force.p);
  launch_symm_load(B, c->P.nin, c->pot.ntypes, (const double*)c->symm_in.p, symm_stride, st);
  launch_type_sort(B, c->pot.ntypes, st);
  if (flags & NNPGPU_BF16) {
    const int rcode = launch_network_bf16(B, c->nets, c->tcbuf, c->pot.ntypes, st, c->tcnets ? c->tcnets->data() : nullptr, 0,
                                          c->tc_wait_limit);
    if (rcode == -1) return set_error(c, NNPGPU_ERR_UNSUPPORTED, "BF16 network path unavailable for this potential");
    if (rcode != 0) return cuda_fail(c, cudaGetLastError(), "tensor-core network set-up");
  } else {
    launch_network_fp32(B, c->nets, c->pot.ntypes, c->tune.nn_tile, st);
  }
  launch_gather(B, c->nets, !(flags & NNPGPU_NO_VACUUM), false, st);
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return cuda_fail(c, le, "energy_symm launch");
  int hstat[ST_WORDS];
  cudaMemcpyAsync(energy, c->energy.p, sizeof(double) * nstruc, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hstat, c->status.p, sizeof(hstat), cudaMemcpyDeviceToHost, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "energy_symm");
  if (hstat[ST_ERROR] & ERR_BAD_TYPE) return set_error(c, NNPGPU_ERR_INVALID, "energy_symm: species index out of range");
  return NNPGPU_OK;
}

extern "C" int nnpgpu_neighbors(nnpgpu_ctx* c, int natoms, const double* posn, const double* cell, int cap, int* count, int* index,
                                float* r, unsigned char* mn, int* shift) {
  return neighbors_impl(c, 0.0, 256, natoms, posn, cell, cap, count, index, r, mn, shift);
}

extern "C" int nnpgpu_neighbors_rc(nnpgpu_ctx* c, double rc, int natoms, const double* posn, const double* cell, int cap, int* count,
                                   int* index, float* r, unsigned char* mn, int* shift) {
  if (!(rc > 0)) return set_error(c, NNPGPU_ERR_INVALID, "cutoff must be positive");
  return neighbors_impl(c, rc, 1024, natoms, posn, cell, cap, count, index, r, mn, shift);
}
