/* Stand-in for the cmake-generated version header (template cmpVersion.h.in). */
#ifndef REF_SHIM_MBIRLIB_VERSION_H
#define REF_SHIM_MBIRLIB_VERSION_H
#include <string>
namespace MBIRLib {
namespace Version {
inline std::string Complete() { return "reference-built-from-source"; }
inline std::string Major() { return "0"; }
inline std::string Minor() { return "0"; }
inline std::string Patch() { return "0"; }
}
}
#endif
