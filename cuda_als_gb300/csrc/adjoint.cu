// adjoint.cu — reverse mode of the user half-sweep (placeholder until the kernel lands).
#include "internal.h"
#include "tc.h"

als_status run_adjoint(als_handle *, const als_coo_view *, double *, float *, double *) {
    return als::set_global_error(ALS_ERR_UNSUPPORTED, "adjoint not built");
}
