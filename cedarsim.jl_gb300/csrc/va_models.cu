// The Verilog-A models' evaluation, compiled once and device-linked into the
// engine kernels.  Built only when the library is built in separate mode
// (large generated model code, e.g. BSIM-CMG); otherwise every kernel
// translation unit carries its own copy of the dispatch.
#define CEDAR_VA_DEFINE
#include "va_models.gen.h"
