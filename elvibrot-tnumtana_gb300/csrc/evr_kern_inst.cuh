// evr_kern_inst.cuh -- instantiation of one term kernel (EVR_KSLAB: slab-streaming or
// general) for one (type, G source) pair, and for the FP32 slab kernel with or without the
// tensor-core contractions (EVR_KTC); included by the evr_kern_*.cu units, which are
// compiled in parallel.
#include "evr_kernels_impl.cuh"

namespace evr {
namespace kern {

#if EVR_KSLAB
#ifndef EVR_KTC
#define EVR_KTC false
#endif
template <typename T, bool GFLY, bool TC>
cudaError_t launch_slab_kernel(int grid, size_t smem, cudaStream_t s, const ItemParams<T>& p) {
  hpsi_slab_kernel<T, GFLY, TC><<<grid, slab_threads<T>(), smem, s>>>(p);
  return cudaGetLastError();
}
template <typename T, bool GFLY, bool TC>
cudaError_t set_slab_kernel_smem(int bytes) {
  return cudaFuncSetAttribute(hpsi_slab_kernel<T, GFLY, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
template <typename T, bool GFLY, bool TC>
cudaError_t slab_kernel_static_smem(int* bytes) {
  cudaFuncAttributes a;
  const cudaError_t e = cudaFuncGetAttributes(&a, hpsi_slab_kernel<T, GFLY, TC>);
  *bytes = e == cudaSuccess ? (int)a.sharedSizeBytes : 0;
  return e;
}
template cudaError_t launch_slab_kernel<EVR_KT, EVR_KGFLY, EVR_KTC>(int, size_t, cudaStream_t,
                                                                   const ItemParams<EVR_KT>&);
template cudaError_t set_slab_kernel_smem<EVR_KT, EVR_KGFLY, EVR_KTC>(int);
template cudaError_t slab_kernel_static_smem<EVR_KT, EVR_KGFLY, EVR_KTC>(int*);
#else
template <typename T, bool GFLY>
cudaError_t launch_items_kernel(int grid, size_t smem, cudaStream_t s, const ItemParams<T>& p, int threads) {
  hpsi_items_kernel<T, GFLY><<<grid, threads, smem, s>>>(p);
  return cudaGetLastError();
}
template <typename T, bool GFLY>
cudaError_t set_items_kernel_smem(int bytes) {
  return cudaFuncSetAttribute(hpsi_items_kernel<T, GFLY>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
template <typename T, bool GFLY>
cudaError_t occupancy_items_kernel(int* per_sm, int smem_bytes) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, hpsi_items_kernel<T, GFLY>, kThreads, smem_bytes);
}
template <typename T, bool GFLY>
cudaError_t items_kernel_static_smem(int* bytes) {
  cudaFuncAttributes a;
  const cudaError_t e = cudaFuncGetAttributes(&a, hpsi_items_kernel<T, GFLY>);
  *bytes = e == cudaSuccess ? (int)a.sharedSizeBytes : 0;
  return e;
}
template cudaError_t launch_items_kernel<EVR_KT, EVR_KGFLY>(int, size_t, cudaStream_t, const ItemParams<EVR_KT>&,
                                                             int);
template cudaError_t set_items_kernel_smem<EVR_KT, EVR_KGFLY>(int);
template cudaError_t items_kernel_static_smem<EVR_KT, EVR_KGFLY>(int*);
template cudaError_t occupancy_items_kernel<EVR_KT, EVR_KGFLY>(int*, int);
#endif

}  // namespace kern
}  // namespace evr
