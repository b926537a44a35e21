/* oracle/shim/gsl/gsl_blas.h -- forwards to the oracle's GSL subset (test infrastructure only). */
#include "pa_gsl_shim.h"
