// descriptor_symm.cu - instances and launcher of the symmetry-function kernel (descriptor.cuh).
#include "descriptor.cuh"

namespace nnpgpu {

size_t symm_smem_bytes(int cap, int ne, int warps) { return sizeof(float) * warp_smem_floats(cap, ne, false) * warps; }

template <int NEK, int NZK, bool GEN>
static void launch_symm_t(const BatchDev& B, const PotParams& P, int warps, cudaStream_t st) {
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(symm_kernel<NEK, NZK, GEN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  const size_t sm = symm_smem_bytes(B.cap, NEK, warps);
  symm_kernel<NEK, NZK, GEN><<<(B.natoms + warps - 1) / warps, 32 * warps, sm, st>>>(
      P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_t, B.nb_r, B.nb_cnt, B.G, B.gstride, B.mom, P.mstride, B.at_order);
}

// Kernel instance covering the potential's largest block grid: (ne, nz) within (2,5), (4,5) or (4,6).
int launch_symm(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st) {
  if (B.natoms == 0) return 0;
  if (ne <= 2 && nz <= 5) P.gen ? launch_symm_t<2, 5, true>(B, P, warps, st) : launch_symm_t<2, 5, false>(B, P, warps, st);
  else if (ne <= 4 && nz <= 5) P.gen ? launch_symm_t<4, 5, true>(B, P, warps, st) : launch_symm_t<4, 5, false>(B, P, warps, st);
  else if (ne <= 4 && nz <= 6) P.gen ? launch_symm_t<4, 6, true>(B, P, warps, st) : launch_symm_t<4, 6, false>(B, P, warps, st);
  else return -1;
  return 0;
}

}  // namespace nnpgpu
