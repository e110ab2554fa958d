// Instantiations of the potential-block apply for float blocks.
#include "bsl_vapply.cuh"

namespace bsl {

int launch_vapply_f32(const float* vb, dim3 g, cudaStream_t s, int nn, const double* v, const double* uk,
                     const double* rot, double* out, long long N, int mode, double* partials, unsigned int* counter,
                     double* scalars, double* hist, int j, long long dpk) {
#define BSL_CASE(K)                                                                                    \
  case K:                                                                                              \
    k_vapply<K, float><<<g, kThreads, 0, s>>>(vb, v, uk, rot, out, N, mode, partials, counter, scalars, hist, j, dpk); \
    break;
  switch (nn) {
    BSL_CASE(1)
    BSL_CASE(3)
    BSL_CASE(4)
    BSL_CASE(6)
    BSL_CASE(9)
    BSL_CASE(10)
    BSL_CASE(15)
    BSL_CASE(16)
    BSL_CASE(21)
    BSL_CASE(25)
    BSL_CASE(28)
    BSL_CASE(36)
    default:
      return fail(BSL_ERR_UNSUPPORTED, "mixed precision needs a block size with a specialised kernel");
  }
#undef BSL_CASE
  BSL_CUDA(cudaGetLastError());
  return BSL_OK;
}

}  // namespace bsl
