// tc.h — tensor-core (tcgen05) half-sweep and adjoint entry points used by sweep.cpp.
#pragma once

#include <string>

#include "handle.h"

bool tc_path_supported(int f);
als_status tc_prepare(als_handle *h, std::string *why);
void tc_release(als_handle *h);
void tc_invalidate_graphs(als_handle *h);
als_status tc_values_changed(als_handle *h);
als_status tc_quantise(als_handle *h, int side, int *launches, std::string *why);
cudaError_t tc_launch_bucket(const als_handle *h, int side, int32_t lo, int32_t hi, int solve,
                             int slot, int *launches);
als_status run_adjoint(als_handle *h, const als_coo_view *heldout, double *loss, float *dLdY,
                       double *dLdlambda);
als_status run_adjoint_f64(als_handle *h, const als_coo_view *heldout, const double *Y,
                           double lambda, double *loss, double *dLdY, double *dLdlambda);
