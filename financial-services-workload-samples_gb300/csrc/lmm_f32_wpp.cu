// FP32 warp-per-path LMM kernels for shapes other than NN=80/NMAT=40.
#include "lmm_device.cuh"

namespace lmm {

bool f32_wpp_supports(int, int) { return false; }
int wpp_block_threads() { return 128; }
cudaError_t wpp_blocks_per_sm(int, int, Mode, bool, int *blocks)
{
    *blocks = 0;
    return cudaErrorNotSupported;
}
cudaError_t launch_wpp_any(const DevModel &, Mode, const float *, uint64_t, int64_t, bool,
                           const Work &, float *, const double *, cudaStream_t)
{
    return cudaErrorNotSupported;
}

}  // namespace lmm
