// Tensor-core DChi2 engine (tcgen05); see dchi2_direct.cu for the exact
// SIMT engine used when this one does not apply.
#include "gv_internal.cuh"

namespace gv {

bool dchi2_tc_supported(const Problem& P) { return false; }

gv_status dchi2_tc(Problem& P, const float* d_img, int flag_opt, float* d_result,
                   int only_channel, int mode) {
  set_error("tensor-core DChi2 engine not available");
  return GV_ERR_UNSUPPORTED;
}

}  // namespace gv
