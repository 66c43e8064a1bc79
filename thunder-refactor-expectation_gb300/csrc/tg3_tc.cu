// tg3_tc.cu -- split-bf16 tensor-core cross term (tcgen05 / TMEM / TMA).
#include "tg3_internal.cuh"

namespace tg3 {

bool bf16x3_available() { return false; }

size_t bf16x3_scratch_bytes(int, int, int, int) { return 256; }

cudaError_t launch_gemm_nt_bf16x3(const float*, long long, int, const float*, long long, int,
                                  int, int, int, int, float*, long long, int, const float*,
                                  long long, float, void*, size_t, int*, cudaStream_t)
{
    return cudaErrorNotSupported;
}

}  // namespace tg3
