// application.h -- include name of the reference framework (gpro/application.h); the GPU
// build's declarations all live in gpro/gpro.h.
#include "gpro/gpro.h"
