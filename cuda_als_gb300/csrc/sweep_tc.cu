// sweep_tc.cu — tensor-core half-sweep (placeholder until the tcgen05 kernel lands).
#include "internal.h"
#include "tc.h"

bool tc_path_supported(int f) { (void)f; return false; }
als_status tc_prepare(als_handle *, std::string *why) { *why = "tensor-core path not built"; return ALS_ERR_UNSUPPORTED; }
void tc_release(als_handle *) {}
void tc_invalidate_graphs(als_handle *) {}
als_status tc_values_changed(als_handle *) { return ALS_OK; }
als_status tc_half_sweep(als_handle *, int, int *, std::string *why) { *why = "tensor-core path not built"; return ALS_ERR_UNSUPPORTED; }
als_status tc_get_plan(const als_handle *, int, int32_t *, int32_t *, int32_t *, int32_t *nb) { *nb = 0; return ALS_ERR_UNSUPPORTED; }
