/* mat4f for the vr shim (test infrastructure only; see vr/common.h).
 * Row-major 4x4; transform() treats the vector as a point (w = 1),
 * transform3x3() as a direction (w = 0).  The parity harness only ever
 * uses identity instances, for which both are exact. */
#ifndef GRIDRT_SHIM_VR_MAT4_H
#define GRIDRT_SHIM_VR_MAT4_H

#include <vr/vec3.h>

namespace vr {

struct mat4f {
    float m[4][4];
    mat4f() { makeIdentity(); }
    void makeIdentity() {
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) m[r][c] = (r == c) ? 1.f : 0.f;
    }
    void transpose() {
        for (int r = 0; r < 4; ++r)
            for (int c = r + 1; c < 4; ++c) { float t = m[r][c]; m[r][c] = m[c][r]; m[c][r] = t; }
    }
    bool isIdentity() const {
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c)
                if (m[r][c] != ((r == c) ? 1.f : 0.f)) return false;
        return true;
    }
    /* Gauss-Jordan inverse in double; identity stays bit-exact identity. */
    bool invert() {
        if (isIdentity()) return true;
        double a[4][8];
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? m[r][c] : (c - 4 == r ? 1.0 : 0.0);
        for (int col = 0; col < 4; ++col) {
            int piv = col;
            for (int r = col + 1; r < 4; ++r)
                if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
            if (a[piv][col] == 0.0) return false;
            if (piv != col)
                for (int c = 0; c < 8; ++c) { double t = a[col][c]; a[col][c] = a[piv][c]; a[piv][c] = t; }
            double inv = 1.0 / a[col][col];
            for (int c = 0; c < 8; ++c) a[col][c] *= inv;
            for (int r = 0; r < 4; ++r)
                if (r != col) {
                    double f = a[r][col];
                    for (int c = 0; c < 8; ++c) a[r][c] -= f * a[col][c];
                }
        }
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) m[r][c] = (float)a[r][c + 4];
        return true;
    }
    void transform(vec3f& v) const {
        float x = m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z + m[0][3];
        float y = m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z + m[1][3];
        float z = m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z + m[2][3];
        v.set(x, y, z);
    }
    void transform3x3(vec3f& v) const {
        float x = m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z;
        float y = m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z;
        float z = m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z;
        v.set(x, y, z);
    }
};

}  // namespace vr

#endif
