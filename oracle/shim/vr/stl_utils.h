/* STL helpers for the vr shim (test infrastructure only). */
#ifndef GRIDRT_SHIM_VR_STL_UTILS_H
#define GRIDRT_SHIM_VR_STL_UTILS_H
#include <vector>
namespace vr {
template <typename T> inline void vectorFreeMemory(std::vector<T>& v) { std::vector<T>().swap(v); }
}
#endif
