// Thread-local error message behind afar_last_error().
#include <cstdarg>
#include <cstdio>

#include "afar_internal.h"

namespace afar {

static thread_local char g_error[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_error, sizeof(g_error), fmt, ap);
  va_end(ap);
}

}  // namespace afar

extern "C" const char* afar_last_error(void) { return afar::g_error; }
