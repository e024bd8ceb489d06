// dr_guard.h - no C++ exception crosses the C ABI.
//
// Every entry point that returns a dr_status has a function-try-block whose handler calls
// dr_internal_exception: an allocation failure (std::bad_alloc, e.g. from a file that declares huge
// sizes) becomes DR_E_NOMEM, any other exception DR_E_STATE, with the message in dr_last_error().
#pragma once
#include "../../include/dr_api.h"

// Call only inside a catch handler.  Records "<where>: <what>" for dr_last_error() on this thread.
dr_status dr_internal_exception(const char *where) noexcept;
