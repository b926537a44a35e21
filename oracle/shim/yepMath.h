/* oracle/shim/yepMath.h -- see yepLibrary.h (test infrastructure only). */
#include "yepLibrary.h"
