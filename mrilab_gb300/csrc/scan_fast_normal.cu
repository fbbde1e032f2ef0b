// Instantiations of the accurate (rotating-frame) scan kernel for one tissue model.
#include "scan_launch.h"

namespace mrl {

namespace {
template <int P, int NS>
cudaError_t go(dim3 grid, size_t smem, cudaStream_t st, const FastLaunch &F) {
    auto k = scan_fast_kernel<KM_NORMAL, P, NS, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kBlock, smem, st>>>(F);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_scan_fast_normal(int P, int NS, dim3 grid, size_t smem, cudaStream_t st, const FastLaunch &F) {
    if (P == 1 && NS == 1) return go<1, 1>(grid, smem, st, F);
    if (P == 1 && NS == 2) return go<1, 2>(grid, smem, st, F);
    if (P == 1 && NS == 4) return go<1, 4>(grid, smem, st, F);
    if (P == 2 && NS == 1) return go<2, 1>(grid, smem, st, F);
    if (P == 2 && NS == 2) return go<2, 2>(grid, smem, st, F);
    if (P == 2 && NS == 4) return go<2, 4>(grid, smem, st, F);
    if (P == 3 && NS == 1) return go<3, 1>(grid, smem, st, F);
    if (P == 3 && NS == 2) return go<3, 2>(grid, smem, st, F);
    if (P == 3 && NS == 4) return go<3, 4>(grid, smem, st, F);
    return cudaErrorInvalidValue;
}

}  // namespace mrl
