/*
 * Stub definitions for the three rt::Context members that the reference's
 * IAccStruct::traceNearestInstance references (src/rtcore/IAccStruct.cpp:31-45).
 * The parity harness never calls traceNearestInstance; these only satisfy the
 * linker so the base class (and its brute-force traceNearestGeometry,
 * src/rtcore/IAccStruct.cpp:74-106) can be compiled unmodified.
 * TEST INFRASTRUCTURE ONLY.
 */
#include <rt/Context.h>

namespace rt {
Context* Context::current() { return nullptr; }
float Context::getRayEpsilon() const { return 2e-4f; }
IEnvironment* Context::getEnvironment() const { return nullptr; }
}  // namespace rt
