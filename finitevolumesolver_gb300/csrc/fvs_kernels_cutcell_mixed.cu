// fvs_kernels_cutcell_mixed.cu -- the fast FP64 (FMA contraction) and the
// mixed-precision (FP32 reconstruction, fluxes, wall states and CFL speeds;
// FP64 state, fractions, h-box combination and update) instantiations of the
// KBN cut-cell kernels (fvs_cutcell_kbn.cuh).
#include "fvs_cutcell.h"
#include "fvs_cutcell_kbn.cuh"

namespace fvs {

cudaError_t LaunchCutCellReferenceStatesT(int precision, const CcStateArgs& a, cudaStream_t s) {
  return precision == 2 ? cc::LaunchKbnStates<float>(a, s) : cc::LaunchKbnStates<double>(a, s);
}

cudaError_t LaunchCutCellSweepT(int precision, const CcSweepArgs& a, cudaStream_t s) {
  return precision == 2 ? cc::LaunchKbnSweep<float>(a, s) : cc::LaunchKbnSweep<double>(a, s);
}

cudaError_t LaunchCutCellStableDtT(int precision, const CcStateArgs& a,
                                   unsigned long long* smax_out, Control* ctrl, cudaStream_t s) {
  return precision == 2 ? cc::LaunchKbnStableDt<float>(a, smax_out, ctrl, s)
                        : cc::LaunchKbnStableDt<double>(a, smax_out, ctrl, s);
}

}  // namespace fvs
