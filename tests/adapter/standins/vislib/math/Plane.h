// Stand-in for vislib::math::Plane (vislib/include/vislib/math/Plane.h), for building the MegaMol adapter where
// the MegaMol tree is absent: a plane through a point with a unit normal.
#pragma once

#include <cmath>

namespace vislib::math {

template<class T>
class Plane {
public:
    struct Vec {
        T x = 0, y = 0, z = 0;
        T X() const { return x; }
        T Y() const { return y; }
        T Z() const { return z; }
    };
    Plane() = default;
    Plane(T px, T py, T pz, T nx, T ny, T nz) {
        const T l = std::sqrt(nx * nx + ny * ny + nz * nz);
        p_ = {px, py, pz};
        n_ = {nx / l, ny / l, nz / l};
    }
    Vec Normal() const { return n_; }
    Vec Point() const { return p_; }

private:
    Vec p_, n_;
};

}  // namespace vislib::math
