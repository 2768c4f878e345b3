// Internal helpers shared by the translation units of libqbcuda.
#pragma once

#include "qbcuda.h"

namespace qbc {

// Record a message for qbc_last_error() and return `code`.
int fail(int code, const char* fmt, ...);
void clear_error();

// True when every cube coordinate of the view's traversal is exactly
// representable, so a child shift can be undone exactly on the way up.
bool cube_shift_exact(const qbc_view& v);

}  // namespace qbc
