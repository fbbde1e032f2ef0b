// Instantiations of the accurate scan kernel whose receive contraction runs
// on tcgen05 (17 to 32 coils): the exchange model (ME, and GM with free or
// bound pools) up to three pools with its coefficients computed in the
// kernel or from the split scheme's table, and the single-pool model.  The
// other instantiations keep the warp-level contraction and a smaller step
// loop.  Its own translation unit: it compiles alongside the others.
#include "scan_launch.h"

namespace mrl {

namespace {
template <int P, int NS>
FastKernel pick_exch(int co, bool all_free) {
    if (co == 1) return all_free ? scan_fast_kernel<KM_EXCH, P, NS, true, 1, true> : nullptr;
    if (co != 0) return nullptr;
    return all_free ? scan_fast_kernel<KM_EXCH, P, NS, true, 0, true> : scan_fast_kernel<KM_EXCH, P, NS, false, 0, true>;
}
}  // namespace

FastKernel select_fast_tc(int km, int co, int P, int NS, bool all_free) {
    if (km == KM_NORMAL && co == 0 && P == 1) {
        if (NS == 1) return scan_fast_kernel<KM_NORMAL, 1, 1, false, 0, true>;
        if (NS == 2) return scan_fast_kernel<KM_NORMAL, 1, 2, false, 0, true>;
        if (NS == 4) return scan_fast_kernel<KM_NORMAL, 1, 4, false, 0, true>;
        return nullptr;
    }
    if (km != KM_EXCH) return nullptr;
    if (P == 1 && NS == 1) return pick_exch<1, 1>(co, all_free);
    if (P == 1 && NS == 2) return pick_exch<1, 2>(co, all_free);
    if (P == 1 && NS == 4) return pick_exch<1, 4>(co, all_free);
    if (P == 2 && NS == 1) return pick_exch<2, 1>(co, all_free);
    if (P == 2 && NS == 2) return pick_exch<2, 2>(co, all_free);
    if (P == 2 && NS == 4) return pick_exch<2, 4>(co, all_free);
    if (P == 3 && NS == 1) return pick_exch<3, 1>(co, all_free);
    if (P == 3 && NS == 2) return pick_exch<3, 2>(co, all_free);
    if (P == 3 && NS == 4) return pick_exch<3, 4>(co, all_free);
    return nullptr;
}

}  // namespace mrl
