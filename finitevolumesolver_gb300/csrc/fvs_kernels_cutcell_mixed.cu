// fvs_kernels_cutcell_mixed.cu -- the fast FP64 (FMA contraction, refined
// reciprocals and square roots: math policy CcFast) and the
// mixed-precision (FP32 reconstruction, fluxes, wall states and CFL speeds;
// FP64 state, fractions, h-box combination and update) instantiations of the
// KBN cut-cell kernels (fvs_cutcell_kbn.cuh); the mixed flavour's FP32
// quotients and roots are the approximate ones of math policy CcFast32.
#include "fvs_cutcell.h"
#include "fvs_cutcell_kbn.cuh"

namespace fvs {

cudaError_t LaunchCutCellReferenceStatesT(int precision, const CcStateArgs& a, cudaStream_t s) {
  return precision == 2 ? cc::LaunchKbnStates<float, cc::CcFast32>(a, s)
                        : cc::LaunchKbnStates<double, cc::CcFast>(a, s);
}

cudaError_t LaunchCutCellSweepT(int precision, const CcSweepArgs& a, bool band, cudaStream_t s) {
  return precision == 2 ? cc::LaunchKbnSweep<float, cc::CcFast32>(a, band, s)
                        : cc::LaunchKbnSweep<double, cc::CcFast>(a, band, s);
}

cudaError_t LaunchCutCellStableDtT(int precision, const CcStateArgs& a,
                                   unsigned long long* smax_out, Control* ctrl, cudaStream_t s) {
  return precision == 2 ? cc::LaunchKbnStableDt<float, cc::CcFast32>(a, smax_out, ctrl, s)
                        : cc::LaunchKbnStableDt<double, cc::CcFast>(a, smax_out, ctrl, s);
}

}  // namespace fvs
