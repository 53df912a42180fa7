/*
 * Minimal stand-in for the `vr` math/utility library (vrbase), which the
 * reference (potato3d/grid-rt) links against but does not ship.  Only the
 * symbols used by the uniform-grid build / 3D-DDA trace files are provided.
 *
 * TEST INFRASTRUCTURE ONLY: this shim exists so that the reference's own CPU
 * sources can be compiled unmodified into oracle/_ref for parity checks.
 *
 * Semantics chosen where vrbase is unknown (written once, used by both the
 * compiled reference and the C restatement in oracle/oracle.c):
 *   sign(x)      = -1 if x < 0, +1 if x > 0, 0 if x == 0
 *   signBit(x)   = IEEE sign bit (1 for -0.0f)
 *   abs(x)       = x < 0 ? -x : x
 *   min/max      = a < b ? a : b  /  a > b ? a : b
 *   MAX_VALUE    = FLT_MAX
 *   vec3 dot     = (x*x' + y*y') + z*z'   (left to right)
 */
#ifndef GRIDRT_SHIM_VR_COMMON_H
#define GRIDRT_SHIM_VR_COMMON_H

#include <cstdint>
#include <cstdio>
#include <climits>
#include <cfloat>
#include <cmath>
#include <vector>

namespace vr {
typedef std::int8_t int8;
typedef std::int16_t int16;
typedef std::int32_t int32;
typedef std::int64_t int64;
typedef std::uint8_t uint8;
typedef std::uint16_t uint16;
typedef std::uint32_t uint32;
typedef std::uint64_t uint64;

template <typename T> inline T abs(T x) { return x < T(0) ? -x : x; }
template <typename T> inline T min(T a, T b) { return a < b ? a : b; }
template <typename T> inline T max(T a, T b) { return a > b ? a : b; }
template <typename T> inline T clampTo(T v, T lo, T hi) { return v < lo ? lo : (v > hi ? hi : v); }
template <typename T> inline T clampAbove(T v, T lo) { return v < lo ? lo : v; }
template <typename T> inline T clampBelow(T v, T hi) { return v > hi ? hi : v; }
template <typename T> inline T sign(T x) { return x < T(0) ? T(-1) : (x > T(0) ? T(1) : T(0)); }
inline int signBit(float x) { return std::signbit(x) ? 1 : 0; }
inline bool isInvalidNumber(float x) { return std::isnan(x) || std::isinf(x); }
inline float toRadians(float deg) { return deg * 0.017453292519943295f; }

template <typename T> struct Math {
    static constexpr T MAX_VALUE = FLT_MAX;
    static constexpr T ZERO_TOLERANCE = T(1e-6);
};
typedef Math<float> Mathf;
}  // namespace vr

#define USING_VR_INTEGER_TYPES   \
    using vr::int8;              \
    using vr::int16;             \
    using vr::int32;             \
    using vr::int64;             \
    using vr::uint8;             \
    using vr::uint16;            \
    using vr::uint32;            \
    using vr::uint64;

#endif
