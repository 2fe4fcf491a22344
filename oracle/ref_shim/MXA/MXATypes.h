/* Stand-in for the cmake-generated MXA/MXATypes.h: fixed-width integer types. */
#ifndef REF_SHIM_MXA_TYPES_H
#define REF_SHIM_MXA_TYPES_H
#include "ref_config.h"
#endif
