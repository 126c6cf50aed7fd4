// evr_tc_test.cu -- self-test of the tensor-core mode contraction (evr_tc.cuh): one CTA
// runs contract_tc on a tensor given by the caller, so that its result can be compared
// with the same contraction done on the host.  A utility with no counterpart in the
// reference (it checks the kernel building block the FP32 H.psi path uses).
#include <cstring>
#include <vector>

#include "evr_internal.h"
#include "evr_kernels_impl.cuh"
#include "evr_tc.cuh"

namespace {

using evr::kern::FastDiv;

__global__ void tc_selftest_kernel(const float* in, float* out, const float* mat, int A, int K, int M, int B, int Vt,
                                   float alpha, int acc, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ FastDiv s_da, s_dv;
  evr::tc::TcSmem* sm = reinterpret_cast<evr::tc::TcSmem*>(smem_raw);
  if (threadIdx.x == 0) {
    s_da = FastDiv::make((uint32_t)A);
    s_dv = FastDiv::make((uint32_t)Vt);
  }
  evr::tc::TcState st;
  evr::tc::tc_setup(st, sm, err);  // ends with a barrier (the divisors are visible after it)
  evr::tc::contract_tc(st, in, Vt, out, Vt, s_da, K, M, B, s_dv, mat, alpha, acc != 0);
  evr::tc::tc_teardown(st);
}

}  // namespace

extern "C" int evr_tc_selftest(int device, int A, int K, int M, int B, int Vt, const float* in, float* out,
                               const float* mat, float alpha, int acc, int threads) {
  using evr::tc::kMaxKp;
  using evr::tc::kMaxNp;
  if (A < 1 || B < 1 || Vt < 1 || K < 1 || M < 1 || K > kMaxKp || M > kMaxNp || !in || !out || !mat)
    return EVR_EINVAL;
  if (threads != 128 && threads != 256 && threads != 512) return EVR_EINVAL;
  const int64_t nin = (int64_t)A * K * B * Vt, nout = (int64_t)A * M * B * Vt;
  if (nin > (1 << 26) || nout > (1 << 26)) return EVR_EINVAL;
  const int ldm = (M + 3) & ~3;
  if (cudaSetDevice(device) != cudaSuccess) return EVR_EDEVICE;
  float *din = nullptr, *dout = nullptr, *dmat = nullptr;
  int* derr = nullptr;
  int rc = EVR_OK;
  auto ok = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == EVR_OK) rc = EVR_EDEVICE;
    return e == cudaSuccess;
  };
  if (ok(cudaMalloc((void**)&din, nin * sizeof(float))) && ok(cudaMalloc((void**)&dout, nout * sizeof(float))) &&
      ok(cudaMalloc((void**)&dmat, (size_t)ldm * K * sizeof(float))) && ok(cudaMalloc((void**)&derr, sizeof(int))) &&
      ok(cudaMemcpy(din, in, nin * sizeof(float), cudaMemcpyHostToDevice)) &&
      ok(cudaMemcpy(dout, out, nout * sizeof(float), cudaMemcpyHostToDevice)) &&
      ok(cudaMemcpy(dmat, mat, (size_t)ldm * K * sizeof(float), cudaMemcpyHostToDevice)) &&
      ok(cudaMemset(derr, 0, sizeof(int)))) {
    const int smem = (int)sizeof(evr::tc::TcSmem);
    if (ok(cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))) {
      tc_selftest_kernel<<<1, threads, smem>>>(din, dout, dmat, A, K, M, B, Vt, alpha, acc, derr);
      int herr = 0;
      if (ok(cudaGetLastError()) && ok(cudaDeviceSynchronize()) &&
          ok(cudaMemcpy(out, dout, nout * sizeof(float), cudaMemcpyDeviceToHost)) &&
          ok(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost)) && herr != 0)
        rc = EVR_ETIMEDOUT;
    }
  }
  (void)cudaGetLastError();
  cudaFree(din);
  cudaFree(dout);
  cudaFree(dmat);
  cudaFree(derr);
  return rc;
}
