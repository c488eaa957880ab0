// The reference's include name for its logger (logger.h), satisfied by this library's C++ face:
// a source written against the reference's logger compiles unchanged with this directory and
// include/ on the include path and -lals_gb300 on the link line.
#pragma once

#include "als_logger.hpp"
