// Aux-bit transfer-matrix cores: DNNI (one carried bit) and diagonal BNNNI
// (two carried bits).
#include "tm_internal.h"

namespace ltm {

void build_aux(Op& op) { fail(TM_ERR_UNSUPPORTED, "operator family not available yet"); }

template <class T>
double matvec_aux(const Op& op, const T* x, T* y, bool scaled, cudaStream_t s) {
  fail(TM_ERR_UNSUPPORTED, "operator family not available yet");
}

template double matvec_aux<float>(const Op&, const float*, float*, bool, cudaStream_t);
template double matvec_aux<double>(const Op&, const double*, double*, bool, cudaStream_t);

}  // namespace ltm
