// noalloc.cu - symmetry functions of one structure without any device allocation.
//
// Some callers cannot let a library call cudaMalloc while they run: a molecular-dynamics code
// that divides the GPU's memory among its own pools before the first step, or a service that
// reserves all device memory at start-up and forbids allocation afterwards (an allocation in
// the middle of a step could fail, or synchronise the device at a point the caller does not
// control).  nnpgpu_symm_noalloc serves them: it computes the symmetry functions of one
// structure whose inputs and outputs the caller provides in device memory, and keeps every
// intermediate (geometry, neighbour lists, status words) in one scratch array compiled into
// this library.
//
// Limits: at most NOALLOC_MAX_ATOMS atoms, NOALLOC_CAP neighbours per atom within the cutoff,
// NOALLOC_MAX_IMAGES lattice images; larger requests are rejected with a message.  The array
// (about 4.6 MB) is held by every GPU that loads the library until the process exits.  All calls
// share it: the status words and the atom->structure map are cleared at the start of each call,
// the rest is overwritten; calls whose work overlaps on the GPU (two streams, two host threads)
// race on it and must be serialised by the caller.
//
// Set-up: the first call on a context (natoms = 0 is enough) looks up the array's device address
// with the context's device current and runs the three kernels of this entry point once on a
// one-atom structure held in the array.  CUDA loads modules and kernels lazily (the default since
// CUDA 12.2), and loading places code and the array in device memory; after the set-up call the
// later calls load nothing.  Make the set-up call before reserving the device's memory and
// before any stream capture.
#include <cmath>
#include <cstring>
#include <mutex>

#include "context.h"

namespace nnpgpu {
namespace {

constexpr int NOALLOC_MAX_ATOMS = 1024;
constexpr int NOALLOC_CAP = 192;
constexpr int NOALLOC_MAX_IMAGES = 512;
constexpr int NOALLOC_WARM_NIN = 1024;  // output row of the set-up call (>= any input size)

// Layout of the scratch array (offsets in bytes, each 256-byte aligned).
struct ScratchLayout {
  size_t meta, imgs, status, atom_struc, sfrac, sfloor, nb_cnt, nb_j, nb_r, nb_code, warm_posn, warm_type, warm_symm, total;
};
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr ScratchLayout make_layout() {
  ScratchLayout L{};
  size_t o = 0;
  L.meta = o; o = align256(o + sizeof(StrucMeta));
  L.imgs = o; o = align256(o + sizeof(ImgEntry) * NOALLOC_MAX_IMAGES);
  L.status = o; o = align256(o + sizeof(int) * ST_WORDS);
  L.atom_struc = o; o = align256(o + sizeof(int) * NOALLOC_MAX_ATOMS);
  L.sfrac = o; o = align256(o + sizeof(float4) * NOALLOC_MAX_ATOMS);
  L.sfloor = o; o = align256(o + sizeof(int4) * NOALLOC_MAX_ATOMS);
  L.nb_cnt = o; o = align256(o + sizeof(int) * NOALLOC_MAX_ATOMS);
  L.nb_j = o; o = align256(o + sizeof(int) * NOALLOC_MAX_ATOMS * NOALLOC_CAP);
  L.nb_r = o; o = align256(o + sizeof(float4) * NOALLOC_MAX_ATOMS * NOALLOC_CAP);
  L.nb_code = o; o = align256(o + sizeof(int) * NOALLOC_MAX_ATOMS * NOALLOC_CAP);
  L.warm_posn = o; o = align256(o + sizeof(double) * 3);  // the set-up call's one-atom structure
  L.warm_type = o; o = align256(o + sizeof(int));
  L.warm_symm = o; o = align256(o + sizeof(float) * NOALLOC_WARM_NIN);
  L.total = o;
  return L;
}
constexpr ScratchLayout kLayout = make_layout();

// The scratch itself.  In host code this name is only a handle for cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kLayout.total];

// Device address of the scratch array, looked up once per device (first call on that device).
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};

int scratch_address(nnpgpu_ctx* c, void** out) {
  if (c->device < 0 || c->device >= kMaxDevices) return set_error(c, NNPGPU_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[c->device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // the context's device is current
    if (e != cudaSuccess || !p)
      return set_error(c, NNPGPU_ERR_CUDA, std::string("no-allocation scratch lookup failed: ") + cudaGetErrorString(e));
    g_scratch_addr[c->device] = p;
  }
  *out = g_scratch_addr[c->device];
  return NNPGPU_OK;
}

// Makes the context's device current for the call and gives the caller's device back on return.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int now = -1;
    if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
  }
};

double nrm3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// Geometry of one structure into fixed arrays: the same formulas as make_meta (Cell::init,
// src/struc/cell.cpp:45-70; lattice shells of NeighborList::build, src/struc/neighbor.cpp:67-95),
// written here without containers so that the call allocates nothing on the host either.
int fixed_meta(const double* cell, int natoms, double rc, StrucMeta& m, ImgEntry* imgs, int& nimg) {
  std::memset(&m, 0, sizeof(m));
  m.natoms = natoms;
  nimg = 0;
  double fro = 0;
  for (int k = 0; k < 9; ++k) {
    m.R[k] = cell ? cell[k] : 0.0;
    fro += m.R[k] * m.R[k];
  }
  fro = std::sqrt(fro);
  m.fro = fro;
  if (!(fro > 0)) return 0;  // non-periodic
  auto M = [&](int r, int q) { return m.R[3 * q + r]; };
  const double c00 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
  const double c01 = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
  const double c02 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
  const double det = M(0, 0) * c00 + M(0, 1) * c01 + M(0, 2) * c02;
  if (det == 0 || !std::isfinite(det)) return -1;
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
    for (int q = 0; q < 3; ++q) m.RInv[3 * q + r] = inv[r][q];
  double col[3][3];
  for (int q = 0; q < 3; ++q)
    for (int r = 0; r < 3; ++r) col[q][r] = m.R[3 * q + r];
  double dmax = nrm3(col[0]);
  for (int q = 1; q < 3; ++q) dmax = dmax < nrm3(col[q]) ? dmax : nrm3(col[q]);
  dmax *= 0.5;
  m.dMax2 = dmax * dmax;
  for (int q = 0; q < 3; ++q)
    for (int r = 0; r < 3; ++r) {
      m.shifts[6 * q + r] = col[q][r];
      m.shifts[6 * q + 3 + r] = -col[q][r];
    }
  for (int k = 0; k < 9; ++k) m.Rf[k] = (float)m.R[k];
  for (int k = 0; k < 18; ++k) m.shiftsf[k] = (float)m.shifts[k];
  m.dmax2f = (float)m.dMax2;
  m.fro2f = (float)(fro * fro);
  int perm[3] = {0, 1, 2};  // columns by decreasing norm, stable for ties
  for (int a = 1; a < 3; ++a)
    for (int b = a; b > 0 && nrm3(col[perm[b]]) > nrm3(col[perm[b - 1]]); --b) {
      const int t = perm[b];
      perm[b] = perm[b - 1];
      perm[b - 1] = t;
    }
  const double* R0 = col[perm[0]];
  const double* R1 = col[perm[1]];
  const double* R2 = col[perm[2]];
  const double cx[3] = {R0[1] * R1[2] - R0[2] * R1[1], R0[2] * R1[0] - R0[0] * R1[2], R0[0] * R1[1] - R0[1] * R1[0]};
  const double dot2 = R2[0] * cx[0] + R2[1] * cx[1] + R2[2] * cx[2];
  // shell ratios in FP64, bounded before the integer conversion (a near-flat cell gives huge ratios)
  const double ratio[3] = {2.0 * rc / nrm3(R0), 2.0 * rc / (nrm3(cx) / nrm3(R0)), 2.0 * rc / std::fabs(dot2 / (nrm3(R0) * nrm3(R1)))};
  long long want = 1;
  int shell[3];
  for (int q = 0; q < 3; ++q) {
    if (!std::isfinite(ratio[q]) || ratio[q] > (double)NOALLOC_MAX_IMAGES) return -2;
    shell[q] = (int)std::floor(ratio[q]);
    want *= 2LL * shell[q] + 1;
  }
  const double Lsum = nrm3(col[0]) + nrm3(col[1]) + nrm3(col[2]);
  m.margin = (float)(2.0 * rc * (Lsum * 1e-6 + 1e-5) + 1e-4 * rc * rc);
  if (shell[0] == 0 && shell[1] == 0 && shell[2] == 0) {
    m.mode = 2;
    return 0;
  }
  if (want > NOALLOC_MAX_IMAGES) return -2;
  m.mode = 1;
  set_image_box(m, inv, rc, shell, perm);
  for (int i = -shell[0]; i <= shell[0]; ++i)
    for (int j = -shell[1]; j <= shell[1]; ++j)
      for (int k = -shell[2]; k <= shell[2]; ++k) {
        ImgEntry& e = imgs[nimg++];
        std::memset(&e, 0, sizeof(e));
        for (int x = 0; x < 3; ++x) {
          e.v[x] = i * R0[x] + j * R1[x] + k * R2[x];
          e.vf[x] = (float)e.v[x];
        }
        e.n[perm[0]] = i;
        e.n[perm[1]] = j;
        e.n[perm[2]] = k;
      }
  m.nimg = nimg;
  return 0;
}

// Launches the entry point's kernels on one structure whose geometry is already in the scratch
// array at base (meta, images, cleared status and atom->structure words).
int run_symm(nnpgpu_ctx* c, uint8_t* S, int natoms, const double* d_posn, const int* d_species, float* d_symm, int symm_stride,
             cudaStream_t st) {
  BatchDev B;
  B.natoms = natoms;
  B.nstruc = 1;
  B.cap = NOALLOC_CAP;
  B.rc = c->pot.rc;
  B.ntypes = c->pot.ntypes;
  B.posn = d_posn;
  B.type = d_species;
  B.atom_struc = (const int*)(S + kLayout.atom_struc);
  B.meta = (const StrucMeta*)(S + kLayout.meta);
  B.imgs = (const ImgEntry*)(S + kLayout.imgs);
  B.sfrac = (float4*)(S + kLayout.sfrac);
  B.sfloor = (int4*)(S + kLayout.sfloor);
  B.nb_j = (int*)(S + kLayout.nb_j);
  B.nb_r = (float4*)(S + kLayout.nb_r);
  B.nb_code = (int*)(S + kLayout.nb_code);
  B.nb_cnt = (int*)(S + kLayout.nb_cnt);
  B.status = (int*)(S + kLayout.status);
  B.G = d_symm;
  B.gstride = symm_stride;
  launch_neighbors(B, st);
  if (launch_symm(B, c->P, c->ne, c->nz, c->tune.warps_symm, st) != 0)
    return set_error(c, NNPGPU_ERR_UNSUPPORTED, "no descriptor kernel for this potential");
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(c, NNPGPU_ERR_CUDA, std::string("nnpgpu_symm_noalloc launch: ") + cudaGetErrorString(e));
  return NNPGPU_OK;
}

// Copies one structure's geometry into the scratch array and clears the words that must start at zero.
void upload_geometry(uint8_t* S, const StrucMeta& meta, const ImgEntry* imgs, int nimg, int natoms, cudaStream_t st) {
  // pageable-source copies return once the stack buffers have been consumed
  cudaMemcpyAsync(S + kLayout.meta, &meta, sizeof(meta), cudaMemcpyHostToDevice, st);
  if (nimg > 0) cudaMemcpyAsync(S + kLayout.imgs, imgs, sizeof(ImgEntry) * nimg, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(S + kLayout.status, 0, sizeof(int) * ST_WORDS, st);
  cudaMemsetAsync(S + kLayout.atom_struc, 0, sizeof(int) * natoms, st);
}

// First call on a context: the array's device address, then one pass of the kernels over a
// single atom at the origin with no cell (species 0, output row in the array), so that every
// kernel this entry point launches for the context's potential is loaded on the device.
int setup(nnpgpu_ctx* c, uint8_t** base) {
  void* p = nullptr;
  int rc = scratch_address(c, &p);
  if (rc != NNPGPU_OK) return rc;
  *base = (uint8_t*)p;
  if (c->noalloc_ready) return NNPGPU_OK;
  if (c->max_nin > NOALLOC_WARM_NIN) return set_error(c, NNPGPU_ERR_UNSUPPORTED, "nnpgpu_symm_noalloc: input size above 1024");
  uint8_t* S = *base;
  cudaStream_t st = c->stream;
  StrucMeta meta;
  int nimg = 0;
  fixed_meta(nullptr, 1, c->pot.rc, meta, nullptr, nimg);
  upload_geometry(S, meta, nullptr, 0, 1, st);
  cudaMemsetAsync(S + kLayout.warm_posn, 0, sizeof(double) * 3, st);
  cudaMemsetAsync(S + kLayout.warm_type, 0, sizeof(int), st);
  rc = run_symm(c, S, 1, (const double*)(S + kLayout.warm_posn), (const int*)(S + kLayout.warm_type), (float*)(S + kLayout.warm_symm),
                c->max_nin, st);
  if (rc != NNPGPU_OK) return rc;
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_error(c, NNPGPU_ERR_CUDA, std::string("nnpgpu_symm_noalloc set-up: ") + cudaGetErrorString(e));
  c->noalloc_ready = true;
  return NNPGPU_OK;
}

}  // namespace
}  // namespace nnpgpu

using namespace nnpgpu;

// Symmetry functions of one structure without device allocation (see the header for the
// contract).  The first call on a context does the set-up described at the top of this file.
extern "C" int nnpgpu_symm_noalloc(nnpgpu_ctx* c, int natoms, const double* d_posn, const int* d_species, const double* cell,
                                   float* d_symm, int symm_stride, void* stream) {
  if (!c) return NNPGPU_ERR_INVALID;
  if (!c->stream) return set_error(c, NNPGPU_ERR_CUDA, "context has no device");
  if (natoms < 0 || natoms > NOALLOC_MAX_ATOMS)
    return set_error(c, NNPGPU_ERR_INVALID,
                     "nnpgpu_symm_noalloc: " + std::to_string(natoms) + " atoms, the limit is " + std::to_string(NOALLOC_MAX_ATOMS));
  if (natoms > 0 && (!d_posn || !d_species || !d_symm))
    return set_error(c, NNPGPU_ERR_INVALID, "nnpgpu_symm_noalloc: device input or output pointer missing");
  if (natoms > 0 && symm_stride < c->max_nin)
    return set_error(c, NNPGPU_ERR_INVALID, "nnpgpu_symm_noalloc: symm_stride below the largest input size");
  DeviceGuard guard(c->device);
  uint8_t* S = nullptr;
  const int rc0 = setup(c, &S);
  if (rc0 != NNPGPU_OK) return rc0;
  if (natoms == 0) return NNPGPU_OK;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;

  StrucMeta meta;
  ImgEntry imgs[NOALLOC_MAX_IMAGES];
  int nimg = 0;
  const int g = fixed_meta(cell, natoms, c->pot.rc, meta, imgs, nimg);
  if (g == -1) return set_error(c, NNPGPU_ERR_INVALID, "nnpgpu_symm_noalloc: singular or non-finite cell");
  if (g == -2)
    return set_error(c, NNPGPU_ERR_INVALID,
                     "nnpgpu_symm_noalloc: the cell needs more than " + std::to_string(NOALLOC_MAX_IMAGES) + " lattice images");
  upload_geometry(S, meta, imgs, nimg, natoms, st);
  const int rc1 = run_symm(c, S, natoms, d_posn, d_species, d_symm, symm_stride, st);
  if (rc1 != NNPGPU_OK) return rc1;
  int hstat[ST_WORDS];
  cudaMemcpyAsync(hstat, S + kLayout.status, sizeof(hstat), cudaMemcpyDeviceToHost, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_error(c, NNPGPU_ERR_CUDA, std::string("nnpgpu_symm_noalloc: ") + cudaGetErrorString(e));
  if (hstat[ST_ERROR] & ERR_BAD_POSITION) return set_error(c, NNPGPU_ERR_INVALID, "nnpgpu_symm_noalloc: non-finite atom position");
  if (hstat[ST_ERROR] & ERR_BAD_TYPE) return set_error(c, NNPGPU_ERR_INVALID, "nnpgpu_symm_noalloc: species index out of range");
  if (hstat[ST_MAXCOUNT] > NOALLOC_CAP)
    return set_error(c, NNPGPU_ERR_CAPACITY,
                     "nnpgpu_symm_noalloc: " + std::to_string(hstat[ST_MAXCOUNT]) + " neighbours within the cutoff, the limit is " +
                         std::to_string(NOALLOC_CAP));
  return NNPGPU_OK;
}
