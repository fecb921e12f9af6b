/* Shim: forwards the reference's general/common/consoleinput.h to the oracle build's common shim. */
#include "general/common/common.h"
