/* oracle/shim/yepCore.h -- see yepLibrary.h (test infrastructure only). */
#include "yepLibrary.h"
