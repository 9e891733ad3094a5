/* matrix.h of the test stand-in: everything is declared in mex.h */
#include "mex.h"
