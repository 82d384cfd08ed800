/* Stand-in for mkl_lapacke.h: everything the reference needs is declared in mkl.h. */
#include "mkl.h"
