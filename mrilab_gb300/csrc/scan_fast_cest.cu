// Instantiations of the accurate (rotating-frame) scan kernel for one tissue model.
#include "scan_launch.h"

namespace mrl {

namespace {
template <int P, int NS>
cudaError_t go(dim3 grid, size_t smem, cudaStream_t st, const FastLaunch &F) {
    auto k = scan_fast_kernel<KM_CEST, P, NS, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kBlock, smem, st>>>(F);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_scan_fast_cest(int P, int NS, dim3 grid, size_t smem, cudaStream_t st, const FastLaunch &F) {
    if (P == 2 && NS == 1) return go<2, 1>(grid, smem, st, F);
    if (P == 2 && NS == 2) return go<2, 2>(grid, smem, st, F);
    if (P == 2 && NS == 4) return go<2, 4>(grid, smem, st, F);
    if (P == 3 && NS == 1) return go<3, 1>(grid, smem, st, F);
    if (P == 3 && NS == 2) return go<3, 2>(grid, smem, st, F);
    if (P == 3 && NS == 4) return go<3, 4>(grid, smem, st, F);
    if (P == 4 && NS == 1) return go<4, 1>(grid, smem, st, F);
    if (P == 4 && NS == 2) return go<4, 2>(grid, smem, st, F);
    if (P == 4 && NS == 4) return go<4, 4>(grid, smem, st, F);
    if (P == 5 && NS == 1) return go<5, 1>(grid, smem, st, F);
    if (P == 5 && NS == 2) return go<5, 2>(grid, smem, st, F);
    if (P == 5 && NS == 4) return go<5, 4>(grid, smem, st, F);
    if (P == 6 && NS == 1) return go<6, 1>(grid, smem, st, F);
    if (P == 6 && NS == 2) return go<6, 2>(grid, smem, st, F);
    if (P == 6 && NS == 4) return go<6, 4>(grid, smem, st, F);
    return cudaErrorInvalidValue;
}

}  // namespace mrl
