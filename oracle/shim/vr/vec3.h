/* vec3f for the vr shim (test infrastructure only; see vr/common.h). */
#ifndef GRIDRT_SHIM_VR_VEC3_H
#define GRIDRT_SHIM_VR_VEC3_H

#include <vr/common.h>

namespace vr {

struct vec3f {
    float x, y, z;
    vec3f() : x(0.f), y(0.f), z(0.f) {}
    vec3f(float a, float b, float c) : x(a), y(b), z(c) {}
    void set(float a, float b, float c) { x = a; y = b; z = c; }
    float& operator[](unsigned i) { return (&x)[i]; }
    const float& operator[](unsigned i) const { return (&x)[i]; }
    vec3f operator+(const vec3f& o) const { return vec3f(x + o.x, y + o.y, z + o.z); }
    vec3f operator-(const vec3f& o) const { return vec3f(x - o.x, y - o.y, z - o.z); }
    vec3f operator*(const vec3f& o) const { return vec3f(x * o.x, y * o.y, z * o.z); }
    vec3f operator*(float s) const { return vec3f(x * s, y * s, z * s); }
    vec3f operator/(float s) const { return vec3f(x / s, y / s, z / s); }
    vec3f operator-() const { return vec3f(-x, -y, -z); }
    vec3f& operator+=(const vec3f& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3f& operator-=(const vec3f& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3f& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3f& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
    bool operator==(const vec3f& o) const { return x == o.x && y == o.y && z == o.z; }
    bool operator!=(const vec3f& o) const { return !(*this == o); }
    float dot(const vec3f& o) const { return x * o.x + y * o.y + z * o.z; }
    vec3f cross(const vec3f& o) const {
        return vec3f(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
    }
    float length() const { return std::sqrt(dot(*this)); }
    float normalize() {
        float l = length();
        if (l > 0.f) { float inv = 1.0f / l; x *= inv; y *= inv; z *= inv; }
        return l;
    }
    static vec3f UNIT_X() { return vec3f(1.f, 0.f, 0.f); }
    static vec3f UNIT_Y() { return vec3f(0.f, 1.f, 0.f); }
    static vec3f UNIT_Z() { return vec3f(0.f, 0.f, 1.f); }
    static vec3f ZERO() { return vec3f(0.f, 0.f, 0.f); }
};

inline vec3f operator*(float s, const vec3f& v) { return v * s; }

}  // namespace vr

#endif
