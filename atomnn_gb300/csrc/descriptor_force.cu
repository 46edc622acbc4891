// descriptor_force.cu - instances and launcher of the chain-rule kernel (descriptor.cuh) for
// GAUSS-only potentials; the general instances are in descriptor_force_gen.cu.
#include "descriptor.cuh"

namespace nnpgpu {

size_t force_smem_bytes(int cap, int ne, int warps, bool kx, int gstride) { return sizeof(float) * warp_smem_floats(cap, ne, kx, gstride) * warps; }

template <int NEK, int NZK>
static void launch_force_t(const BatchDev& B, const PotParams& P, int warps, cudaStream_t st) {
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(force_kernel<NEK, NZK, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  const size_t sm = force_smem_bytes(B.cap, NEK, warps, false, B.gstride + P.mstride);
  force_kernel<NEK, NZK, false><<<(B.natoms + warps - 1) / warps, 32 * warps, sm, st>>>(
      P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_t, B.nb_r, B.nb_cnt, B.dEdG, B.gstride, B.mom, P.mstride, B.nb_code, B.facc, B.at_order, B.status);
}

// Kernel instance covering the potential's largest block grid: (ne, nz) within (2,5), (4,5) or (4,6).
int launch_force(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st) {
  if (B.natoms == 0) return 0;
  if (P.gen) return launch_force_gen(B, P, ne, nz, warps, st);
  if (ne <= 2 && nz <= 5) launch_force_t<2, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 5) launch_force_t<4, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 6) launch_force_t<4, 6>(B, P, warps, st);
  else return -1;
  return 0;
}

}  // namespace nnpgpu
