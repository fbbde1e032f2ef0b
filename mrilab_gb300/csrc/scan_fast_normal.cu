// Instantiations of the accurate (rotating-frame) scan kernel for one tissue model.
#include "scan_launch.h"

namespace mrl {

namespace {
using Kernel = void (*)(const FastLaunch *, const int2 *, int, int *);

template <int P, int NS>
Kernel pick(bool all_free) {
    (void)all_free;
    return scan_fast_kernel<KM_NORMAL, P, NS, false>;
}

Kernel select(int P, int NS, bool all_free) {
    if (P == 1 && NS == 1) return pick<1, 1>(all_free);
    if (P == 1 && NS == 2) return pick<1, 2>(all_free);
    if (P == 1 && NS == 4) return pick<1, 4>(all_free);
    if (P == 2 && NS == 1) return pick<2, 1>(all_free);
    if (P == 2 && NS == 2) return pick<2, 2>(all_free);
    if (P == 2 && NS == 4) return pick<2, 4>(all_free);
    if (P == 3 && NS == 1) return pick<3, 1>(all_free);
    if (P == 3 && NS == 2) return pick<3, 2>(all_free);
    if (P == 3 && NS == 4) return pick<3, 4>(all_free);
    return nullptr;
}
}  // namespace

cudaError_t launch_scan_fast_normal(int P, int NS, bool all_free, dim3 grid, size_t smem, cudaStream_t st,
                                         const FastGrid &g) {
    Kernel k = select(P, NS, all_free);
    if (!k) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, kBlock, smem, st>>>(g.descs, g.items, g.n_items, g.counter);
    return cudaGetLastError();
}

int occupancy_scan_fast_normal(int P, int NS, bool all_free, size_t smem) {
    Kernel k = select(P, NS, all_free);
    int n = 0;
    if (!k || cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kBlock, smem) != cudaSuccess)
        return 0;
    return n;
}

}  // namespace mrl
