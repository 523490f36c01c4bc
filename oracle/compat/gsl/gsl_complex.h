/* Project-written GSL API subset (test infrastructure only), see ../compat_gsl.h */
#include "../compat_gsl.h"
