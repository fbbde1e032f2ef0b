// The exact propagator's instantiations of the accurate scan kernel for the
// general model with bound pools (TypeFlag 1) -- and the MT and CEST models,
// whose bound pool is pool 1: free pools rotate, bound
// pools are saturated on rf steps, then the relaxation-exchange step comes
// from the exact table (a bound pool without a transverse generator).  In
// their own translation unit so that they compile alongside the others.
#include "scan_launch.h"

namespace mrl {

FastKernel select_exact_bound(int P, int NS) {
    if (P == 2 && NS == 1) return scan_fast_kernel<KM_EXCH, 2, 1, false, 2>;
    if (P == 2 && NS == 2) return scan_fast_kernel<KM_EXCH, 2, 2, false, 2>;
    if (P == 2 && NS == 4) return scan_fast_kernel<KM_EXCH, 2, 4, false, 2>;
    if (P == 3 && NS == 1) return scan_fast_kernel<KM_EXCH, 3, 1, false, 2>;
    if (P == 3 && NS == 2) return scan_fast_kernel<KM_EXCH, 3, 2, false, 2>;
    // CEST with four and five pools (water, MT, and two or three CEST pools)
    if (P == 4 && NS == 1) return scan_fast_kernel<KM_EXCH, 4, 1, false, 2>;
    if (P == 5 && NS == 1) return scan_fast_kernel<KM_EXCH, 5, 1, false, 2>;
    return nullptr;
}

}  // namespace mrl
