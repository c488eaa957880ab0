// als_error.hpp — the exception thrown by the header-only C++ faces (als_model.hpp,
// als_logger.hpp) for a non-OK als_status; what() is "<STATUS NAME>: <library message>".
#pragma once

#include <stdexcept>
#include <string>

#include "als_gb300.h"

class als_gb300_error : public std::runtime_error {
public:
    als_gb300_error(als_status s, const std::string &what)
        : std::runtime_error(std::string(als_status_string(s)) + ": " + what), status(s) {}
    als_status status;
};

namespace als_gb300_detail {
inline void check(als_status s, const als_handle *h = nullptr) {
    if (s != ALS_OK) throw als_gb300_error(s, als_last_error(h));
}
}  // namespace als_gb300_detail
