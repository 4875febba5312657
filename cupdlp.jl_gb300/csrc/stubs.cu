// stubs.cu — entry points not implemented yet: they fail loudly with NOT_SUPPORTED.
#include "problem.h"

extern "C" {
gpdhg_status gpdhg_problem_create_unscaled(const gpdhg_lp_desc*, const gpdhg_params*, gpdhg_problem** out) {
  if (out) *out = nullptr;
  return GPDHG_ERR_NOT_SUPPORTED;
}
gpdhg_status gpdhg_get_rescaling(const gpdhg_problem*, double*, double*) { return GPDHG_ERR_NOT_SUPPORTED; }
}
