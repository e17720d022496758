// ginf/core.h -- the model layer of the API (src/include/core.h).
#ifndef GINF_GB300_CORE_H
#define GINF_GB300_CORE_H

#include "grid.h"
#include "matrix.h"
#include "utils.h"

namespace ginf {
// Status (a ginf_status value) of the last solver call on this thread, and
// its message.  The void entry points below never exit the process; they
// report failures here and on stderr, leaving the result matrix unchanged.
int lastStatus();
const char *lastError();
}  // namespace ginf

#endif
