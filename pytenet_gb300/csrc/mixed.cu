// Mixed-precision (split-BF16 on tcgen05) form of the site / bond operators.
// Placeholder until the tensor-core path lands: every entry reports
// PTN_UNSUPPORTED so that callers fail loudly instead of computing in FP64.
#include "ptn_common.cuh"

namespace ptn {

size_t heff_workspace_bytes_mixed(int, int, int, int, int) { return 0; }
size_t bond_workspace_bytes_mixed(int, int, int) { return 0; }

static ptn_status unsupported() {
  set_error("mixed precision path is not built into this library");
  return PTN_UNSUPPORTED;
}

ptn_status heff_prepare_mixed(const double2*, const double2*, const double2*, int, int, int, int,
                              int, void*, size_t, cudaStream_t) { return unsupported(); }
ptn_status heff_apply_mixed(const double2*, double2*, const double2*, int, int, int, int, int,
                            void*, size_t, const int*, cudaStream_t) { return unsupported(); }
ptn_status bond_prepare_mixed(const double2*, const double2*, int, int, int, void*, size_t,
                              cudaStream_t) { return unsupported(); }
ptn_status bond_apply_mixed(const double2*, double2*, int, int, int, void*, size_t, const int*,
                            cudaStream_t) { return unsupported(); }
ptn_status heff_apply_mixed_entry(const double2*, const double2*, const double2*, const double2*,
                                  double2*, int, int, int, int, int, void*, size_t, cudaStream_t) {
  return unsupported();
}
ptn_status bond_apply_mixed_entry(const double2*, const double2*, const double2*, double2*, int,
                                  int, int, void*, size_t, cudaStream_t) { return unsupported(); }

}  // namespace ptn
