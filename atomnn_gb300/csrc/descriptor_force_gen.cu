// descriptor_force_gen.cu - instances of the chain-rule kernel (descriptor.cuh) for potentials
// with a non-GAUSS angular family or blocks off the function grid.
#include "descriptor.cuh"

namespace nnpgpu {

template <int NEK, int NZK>
static void launch_force_gen_t(const BatchDev& B, const PotParams& P, int warps, cudaStream_t st) {
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(force_kernel<NEK, NZK, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  const size_t sm = force_smem_bytes(B.cap, NEK, warps, P.kx, B.gstride + P.mstride);
  force_kernel<NEK, NZK, true><<<(B.natoms + warps - 1) / warps, 32 * warps, sm, st>>>(
      P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_t, B.nb_r, B.nb_cnt, B.dEdG, B.gstride, B.mom, P.mstride, B.nb_code, B.facc, B.at_order, B.status);
}

int launch_force_gen(const BatchDev& B, const PotParams& P, int ne, int nz, int warps, cudaStream_t st) {
  if (ne <= 2 && nz <= 5) launch_force_gen_t<2, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 5) launch_force_gen_t<4, 5>(B, P, warps, st);
  else if (ne <= 4 && nz <= 6) launch_force_gen_t<4, 6>(B, P, warps, st);
  else return -1;
  return 0;
}

}  // namespace nnpgpu
