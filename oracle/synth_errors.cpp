// The error recorder synth.cpp calls, for the oracle-side build of the workload generator
// (oracle/build.py build_synth): the message is kept per thread and the status returned, as the
// library's own recorder does.  TEST INFRASTRUCTURE ONLY.
#include <string>

#include "../include/als_gb300.h"

namespace als {

thread_local std::string g_synth_error;

als_status set_global_error(als_status s, const std::string &msg) {
    g_synth_error = msg;
    return s;
}

}  // namespace als

extern "C" const char *oracle_synth_last_error(void) { return als::g_synth_error.c_str(); }
