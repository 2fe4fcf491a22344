/* Stand-in for the cmake-generated MBIRLib/MBIRLib.h (template MBIRLibConfiguration.h.in):
 * static library, parallel algorithms on (the reference needs its TBB branch: its serial branch
 * does not compile).  Test infrastructure only. */
#ifndef _MBIRLib_H_
#define _MBIRLib_H_
#ifndef OpenMBIR_USE_PARALLEL_ALGORITHMS
#define OpenMBIR_USE_PARALLEL_ALGORITHMS 1
#endif
#include "ref_config.h"
#include "MBIRLib/Common/MBIRLibDLLExport.h"
#endif
