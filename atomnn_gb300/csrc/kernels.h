// kernels.h - device buffers of one batch and the kernel launchers (host-side interface).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "common.cuh"

namespace nnpgpu {

// All device pointers of one batch of structures.  Atoms of a structure are contiguous;
// per-atom neighbour data uses fixed-stride slots [i*cap, i*cap+cap).
struct BatchDev {
  int natoms = 0, nstruc = 0, cap = 0;
  int a0 = 0, s0 = 0;
  int ntypes = 1;  // first atom / structure of this view (all arrays are batch-indexed)
  double rc = 0;
  // inputs
  const double* posn = nullptr;  // [natoms*3]
  const int* type = nullptr;     // [natoms]
  const int* atom_struc = nullptr;
  // [natoms] the atom each warp of the neighbour kernel takes: whole structures, those with the
  // most candidate pairs per centre first, so that no slow structure starts at the end (null:
  // batch order)
  const int* nb_order = nullptr;
  // [natoms] the atom each warp of the descriptor and chain-rule kernels takes: whole structures,
  // the densest (most neighbours per atom) first (null: batch order)
  const int* at_order = nullptr;
  const StrucMeta* meta = nullptr;
  const ImgEntry* imgs = nullptr;
  // neighbour lists
  float4* sfrac = nullptr;  // wrapped fractional coordinates
  int4* sfloor = nullptr;   // their integer floors
  int* nb_j = nullptr;
  float4* nb_r = nullptr;
  int* nb_code = nullptr;
  unsigned char* nb_t = nullptr;  // species of each slot's neighbour (null: looked up from type[])
  int* nb_cnt = nullptr;
  // cell lists of the structures in neighbour mode 4 (ncells entries, sentinels included)
  int ncells = 0;
  int* cell_cnt = nullptr;    // atoms per cell; zero between calls
  int* cell_start = nullptr;  // first slot of each cell in cell_atoms (global atom positions)
  int* cell_atoms = nullptr;  // [natoms] atoms ordered by cell
  int* atom_cell = nullptr;   // [natoms] cell of each atom
  int* cell_of = nullptr;     // [natoms] cell of each position of cell_atoms
  float4* sfrac_c = nullptr;  // [natoms] sfrac in cell_atoms order
  int4* sfloor_c = nullptr;   // [natoms] sfloor in cell_atoms order
  // descriptors and networks
  float* G = nullptr;      // [natoms*gstride]
  float* dEdG = nullptr;   // [natoms*gstride]
  float* mom = nullptr;    // [natoms*mstride] moment tensors of moment blocks (descriptor pass -> chain rule)
  int gstride = 0;
  float* eatom = nullptr;  // [natoms] network output
  int* perm = nullptr;     // [natoms] atoms grouped by type
  int* type_count = nullptr;  // [NT_MAX+1] counters (device)
  // forces
  long long* facc = nullptr;  // [natoms*3] forces in 64-bit fixed point (FORCE_SCALE units), summed by the chain rule
  double* force = nullptr; // [natoms*3] output
  double* energy = nullptr;  // [nstruc] output
  int* status = nullptr;   // [ST_WORDS]
};

// Launch shapes chosen by the autotuner (nnpgpu_autotune): centre atoms (warps) per CTA of
// the neighbour, descriptor and chain-rule kernels, and the atom tile of the FP32 networks.
struct TuneCfg {
  int warps_nbr = 4;
  int warps_symm = 4;
  int warps_force = 4;
  int nn_tile = 32;
};

// warps = centre atoms per CTA (1-4)
void launch_neighbors(const BatchDev& B, cudaStream_t st, int warps = 4);
// dynamic shared memory of the neighbour kernel when some structure uses a cell list
size_t neighbor_smem_bytes(int cap, int warps);
// descriptors (NNP::symm) and chain rule (NNP::force) ; ne/nz select the template instance
int launch_symm(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st);
int launch_force(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st);
size_t symm_smem_bytes(int cap, int ne, int warps);
size_t force_smem_bytes(int cap, int ne, int warps, bool kx, int gstride);
// Image-shell box of a mode-1 structure (StrucMeta::rinvf/hrc/shell/perm): inv is R^-1 (rows),
// shell and perm as enumerated for the image list.  Shared by the batched and no-allocation
// set-ups.
inline void set_image_box(StrucMeta& m, const double inv[3][3], double rc, const int shell[3], const int perm[3]) {
  for (int k = 0; k < 9; ++k) m.rinvf[k] = (float)m.RInv[k];
  for (int c = 0; c < 3; ++c) {
    // |(R^-1 t)_c| <= |row c of R^-1| |t|; 2e-3 in fractional units covers the FP32 evaluation
    // and the decision margin many times over
    double h2 = 0.0;
    for (int q = 0; q < 3; ++q) h2 += inv[c][q] * inv[c][q];
    m.hrc[c] = (float)(rc * std::sqrt(h2) + 2e-3);
    m.shell[c] = shell[c];
    m.perm[c] = perm[c];
  }
}

// atomic networks: FP32 SIMT path and BF16 tensor-core path
void launch_type_sort(const BatchDev& B, int ntypes, cudaStream_t st);
size_t type_sort_ints(int natoms);  // ints of the type_count buffer for a batch of natoms
void launch_network_fp32(const BatchDev& B, const NetsP& N, int ntypes, int tile, cudaStream_t st);
// stored FP64 descriptors (sstride per atom) into B.G (nin[t] values of each atom's type t)
void launch_symm_load(const BatchDev& B, const int* nin, int ntypes, const double* src, int sstride, cudaStream_t st);
// wait_limit: polls of each mbarrier wait before the kernel gives up with ERR_TIMEOUT
int launch_network_bf16(const BatchDev& B, const NetsP& N, const void* tc_weights, int ntypes, cudaStream_t st, const void* tcnets_host,
                        int want_grad, int wait_limit);
// the energy trainer's batch error and parameter gradient after a batched energy pass
int train_tiles(int natoms, int ntypes);
int launch_train(const BatchDev& B, const NetsP& N, int ntypes, const double* eref, int loss, double delta, double* dcdo, double* err,
                 float* partial, int pstride, double* grad, int max_params, cudaStream_t st);
// the force trainer: residual weights t_k = beta (F_k - F_ref,k)/N^2, the loss terms, the
// descriptor-space weights u (tangent_kernel) and the parameter gradient of the force term
// accumulated onto grad
int train_force_tiles(int natoms, int ntypes);
void launch_train_force_loss(const BatchDev& B, const double* fref, double beta, float4* tvec, double* fatom, double* fstruc, double* err,
                             cudaStream_t st);
int launch_tangent(const BatchDev& B, const PotParams& P, int ne, int nz, const float4* tvec, float* U, cudaStream_t st);
int launch_train_force(const BatchDev& B, const NetsP& N, int ntypes, const float* U, float* partial, int pstride, double* grad,
                       int max_params, cudaStream_t st);
// forces from their fixed-point sums, per-structure energy
void launch_gather(const BatchDev& B, const NetsP& N, bool add_vacuum, bool want_force, cudaStream_t st);

}  // namespace nnpgpu
