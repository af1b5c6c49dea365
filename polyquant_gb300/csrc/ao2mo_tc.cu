// Split-precision AO->MO transform on tcgen05 tensor cores (see ao2mo.cu for
// the half-transform structure).
#include "pq_internal.h"

namespace pq {
pq_status ao2mo_tc(const double *, int, int64_t, const double *, int64_t, int64_t, int, double *, cudaStream_t) {
  set_error("pq_ao2mo: split-precision tensor-core modes are not built yet");
  return PQ_ERR_ARG;
}
}  // namespace pq
