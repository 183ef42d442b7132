// mfdOperator.h -- include name of the reference operator header; the GPU operators
// are declared in gpro/operators.h.
#include "gpro/operators.h"
