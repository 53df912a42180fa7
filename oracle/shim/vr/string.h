/* String helpers for the vr shim (test infrastructure only); nothing on the
 * grid path uses them, the header only has to exist. */
#ifndef GRIDRT_SHIM_VR_STRING_H
#define GRIDRT_SHIM_VR_STRING_H
#include <string>
namespace vr { typedef std::string String; }
#endif
