/* GSL header stand-in for the oracle reference build: see ../gsl_shim_common.h */
#include "../gsl_shim_common.h"
