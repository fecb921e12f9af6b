/* Shim: forwards the reference's general/common/memorycheck.h to the oracle build's common shim. */
#include "general/common/common.h"
