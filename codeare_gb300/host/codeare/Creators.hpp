// Creators.hpp -- the 2-D Shepp-Logan phantom used by the CGSENSE test case
// (reference: src/matrix/Creators.hpp:369-395 ellipse and :453-490 phantom:
// Shepp & Logan, IEEE TNS 21, 1974).  The ellipse table is the published one;
// the rasterisation follows the reference's float arithmetic so both produce
// the same pixels.
#pragma once

#include <cmath>

#include "Matrix.hpp"

template <class T> inline Matrix<T> phantom(const size_t &n)
{
    static const float p[10][5] = {
        {.69f, .92f, .0f, .0f, .0f},        {.6624f, .874f, .0f, -.0184f, .0f},
        {.11f, .31f, -.22f, .0f, -.3f},     {.16f, .41f, .22f, .0f, .3f},
        {.21f, .25f, .0f, .35f, .0f},       {.046f, .046f, .00f, .1f, .0f},
        {.046f, .046f, .0f, -.1f, .0f},     {.046f, .023f, .08f, -.605f, .0f},
        {.023f, .023f, .0f, -.606f, .0f},   {.023f, .046f, -.06f, -.605f, .0f}};
    static const float v[10] = {1.f, -.8f, -.2f, -.2f, .1f, .1f, .1f, .1f, .1f, .1f};
    Matrix<T> res(n);
    const float fn = float(n);
    for (int e = 0; e < 10; ++e) {
        const float a0 = p[e][0] * fn / 2.0f, a1 = p[e][1] * fn / 2.0f;
        const float m0 = (1.0f - p[e][2]) * fn / 2.0f, m1 = (1.0f - p[e][3]) * fn / 2.0f;
        const float cp = std::cos(p[e][4]), sp = std::sin(p[e][4]);
        for (size_t r = 0; r < n; ++r)
            for (size_t c = 0; c < n; ++c) {
                const float x = (((float)c - m1) * cp + ((float)r - m0) * sp) / a1;
                const float y = (((float)r - m0) * cp - ((float)c - m1) * sp) / a0;
                if (x * x + y * y <= 1.0f) res(c, r) += T(v[e]);
            }
    }
    return res;
}
