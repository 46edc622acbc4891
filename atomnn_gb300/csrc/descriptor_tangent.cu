// descriptor_tangent.cu - instances and launcher of the force trainer's tangent kernel
// (descriptor.cuh).
#include "descriptor.cuh"

namespace nnpgpu {

template <int NEK, int NZK>
static void launch_tangent_t(const BatchDev& B, const PotParams& P, const float4* tvec, float* U, cudaStream_t st) {
  static bool attr = false;
  if (!attr) attr = cudaFuncSetAttribute(tangent_kernel<NEK, NZK>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess;
  const int warps = 4;
  tangent_kernel<NEK, NZK><<<(B.natoms + warps - 1) / warps, 32 * warps, sizeof(float) * warp_smem_floats(B.cap, NEK, true) * warps, st>>>(
      P, B.a0, B.natoms, B.cap, B.type, B.nb_j, B.nb_t, B.nb_r, B.nb_code, B.nb_cnt, tvec, U, B.gstride);
}

// The kernel instance must cover every block's zeta chain: the moment blocks' zeta <= 4 (nz 3)
// included, which nz (the triplet blocks' largest) does not count.
int launch_tangent(const BatchDev& B, const PotParams& P, int ne, int nz, const float4* tvec, float* U, cudaStream_t st) {
  if (B.natoms == 0) return 0;
  nz = nz < 3 ? 3 : nz;
  if (ne <= 2 && nz <= 5) launch_tangent_t<2, 5>(B, P, tvec, U, st);
  else if (ne <= 4 && nz <= 5) launch_tangent_t<4, 5>(B, P, tvec, U, st);
  else if (ne <= 4 && nz <= 6) launch_tangent_t<4, 6>(B, P, tvec, U, st);
  else return -1;
  return 0;
}

}  // namespace nnpgpu
