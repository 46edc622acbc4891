// context.h - the engine context behind the C ABI (include/nnpgpu.h).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/nnpgpu.h"
#include "kernels.h"
#include "potential.h"
#include "serve.h"

namespace nnpgpu {

// A device buffer that grows on demand and counts against the context's HBM budget.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};
struct HostBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Host-side geometry of one structure (mirrors Cell::init and the shell set-up of
// NeighborList::build, src/struc/cell.cpp:45-70 and src/struc/neighbor.cpp:67-95).
void make_meta(const double* cell, int atom0, int natoms, double rc, StrucMeta& m, std::vector<ImgEntry>& imgs);

class Serving;

// A resident neighbour list (built with cutoff rc + skin) that a structure of a batch may use
// instead of searching all atoms (neighbour mode 3); j/code/cnt are device arrays, cap slots per atom.
struct SkinRef {
  const int* j = nullptr;
  const int* code = nullptr;
  const int* cnt = nullptr;
  int cap = 0;
};

// Geometry of one batch as uploaded to the device (per-structure metadata and atom offsets).
struct Uploaded {
  int natoms = 0, nstruc = 0, cap = 0, ncells = 0;
  std::vector<StrucMeta> metas;
  std::vector<int> offsets;
};

// The batch description behind the geometry currently on the device.
struct MetaCache {
  bool valid = false;
  int generation = -1, cap = 0;
  double rc = 0.0;
  std::vector<int> natoms;
  std::vector<double> cell;
  std::vector<const void*> skins;  // per structure: j, code, cnt, cap
  Uploaded U;
};

}  // namespace nnpgpu

struct nnpgpu_ctx {
  std::string err;
  std::string potfile;
  int device = 0;
  int verbose = 0;
  cudaStream_t stream = nullptr;
  nnpgpu::HPot pot;
  nnpgpu::PotParams P;
  int ne = 1, nz = 1, max_nin = 0, gstride = 0;
  nnpgpu::NetsP nets{};
  void* netbuf = nullptr;
  size_t netbytes = 0;
  void* tcbuf = nullptr;  // BF16 weights of the tensor-core path (packed operand layout)
  size_t tcbytes = 0;
  std::shared_ptr<std::vector<uint8_t>> tcnets;  // kernel parameter block of that path
  size_t budget = 0, used = 0;
  int cap_hint = 0;
  nnpgpu::TuneCfg tune;
  int tc_wait_limit = 1 << 22;  // polls of each mbarrier wait of the tensor-core networks (nnpgpu_set_wait_limit)
  // batch buffers
  nnpgpu::DevBuf posn, type, atom_struc, meta, imgs, sfrac, sfloor, nb_j, nb_r, nb_code, nb_cnt, G, dEdG, eatom, perm,
      type_count, facc, force, energy, status, nb_order, at_order, cell_of, cell_cnt, cell_start, cell_atoms, atom_cell, mom, nb_t, tr_eref,
      tr_dcdo, tr_err, tr_part, tr_grad, symm_in, tr_fref, tr_t, tr_fatom, tr_fstruc, tr_u, sfrac_c, sfloor_c;
  nnpgpu::HostBuf h_meta, h_in, h_out;  // pinned staging: geometry, inputs, outputs
  int buf_generation = 0;
  nnpgpu::MetaCache meta_cache;
  // captured launch sequences of the batched path, keyed by batch shape
  typedef std::tuple<int, int, int, int, int, int, const void*, const void*, const void*, const void*> GraphKey;
  std::map<GraphKey, cudaGraphExec_t> graphs;
  std::map<GraphKey, int> shapes_seen;
  std::unique_ptr<nnpgpu::Serving> serving;
  // stage tracing (nnpgpu_profile_*): events at stage boundaries of the batched launch sequence
  bool prof_on = false;
  cudaEvent_t prof_ev[NNPGPU_NSTAGES + 1] = {};
  double prof_ms[NNPGPU_NSTAGES] = {};
  long long prof_n[NNPGPU_NSTAGES] = {};
  // nnpgpu_symm_noalloc: set-up done on this context (scratch address known, kernels loaded)
  bool noalloc_ready = false;
};

namespace nnpgpu {
// Grow dev to at least bytes (never shrinks).  Returns false on allocation failure / budget.
bool ensure(nnpgpu_ctx* c, DevBuf& b, size_t bytes);
bool ensure_host(nnpgpu_ctx* c, HostBuf& b, size_t bytes);
// Runs the launch sequence for atoms of structures [s0, s0+ns) of the uploaded batch.
int run_pipeline(nnpgpu_ctx* c, const BatchDev& B, int flags, cudaStream_t st);
int set_error(nnpgpu_ctx* c, int code, const std::string& msg);
// Host-buffer batch evaluation with optional resident skin lists per structure (skins may be null;
// an entry with cnt == nullptr, or a structure that is not single-image at rc, builds normally).
int compute_host(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* posn, const int* species, const double* cell, int flags,
                 double* energy, double* force, float* symm, const SkinRef* skins);
// Builds the neighbour list of one structure with cutoff rc_skin into device arrays of skin_cap
// slots per atom (local atom indices).  Returns OK, or NNPGPU_ERR_CAPACITY with *max_count set.
int build_skin(nnpgpu_ctx* c, int natoms, const double* posn, const double* cell, double rc_skin, int skin_cap, int* d_j, int* d_code,
               int* d_cnt, float4* d_r, int* max_count, bool posn_on_device = false);
// Device-buffer evaluation (as nnpgpu_compute_device) with optional resident skin lists.
int compute_device_skins(nnpgpu_ctx* c, int nstruc, const int* natoms, const double* d_posn, const int* d_species, const double* cell,
                         int flags, double* d_energy, double* d_force, cudaStream_t st, const SkinRef* skins);
// Packs the BF16 weights of the tensor-core network path (network_tc.cu).
int prepare_tc_weights(nnpgpu_ctx* c);
}  // namespace nnpgpu
