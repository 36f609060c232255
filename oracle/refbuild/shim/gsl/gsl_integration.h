/* Oracle-build shim: see gsl_shim_common.h. */
#include "gsl/gsl_shim_common.h"
