// computeLayer.h -- include name of the reference header; the load estimator is
// declared in gpro/load.h.
#include "gpro/load.h"
