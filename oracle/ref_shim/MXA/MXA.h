/* Stand-in for the cmake-generated MXA/MXA.h (template MXAConfiguration.h.in): no HDF5, TIFF
 * or XML support, 64-bit file reader and writer classes.  Test infrastructure only. */
#ifndef _MXA_CONFIGURATION_H_
#define _MXA_CONFIGURATION_H_
#define MXA_HDF5_SUPPORT 0
#define MXA_TIFF_SUPPORT 0
#define MXA_XML_SUPPORT 0
#define HDF5_VTK_BRIDGE 0
#define MXADATAMODEL_SYSTEM "Linux"
#define MXAFILEREADER_CLASS_NAME MXAFileReader64
#define MXAFILEWRITER_CLASS_NAME MXAFileWriter64
#include "ref_config.h"
#include "MXA/MXADLLExport.h"
#endif
