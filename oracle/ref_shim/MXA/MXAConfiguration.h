/* Stand-in for the cmake-generated MXA/MXAConfiguration.h (same content as MXA/MXA.h). */
#include "MXA/MXA.h"
