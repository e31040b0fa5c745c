// placeholder replaced by the tcgen05 kernels
#include "sg_internal.h"
namespace sg {
bool tc_available() { return false; }
cudaError_t tc_syrk_bf16(const void*, const void*, int64_t, int64_t, float*, float, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t tc_gemm_tf32(const float*, int64_t, const float*, int64_t, float*, cudaStream_t) { return cudaErrorNotSupported; }
}
