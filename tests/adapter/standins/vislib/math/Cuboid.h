// Stand-in for vislib::math::Cuboid (vislib/include/vislib/math/Cuboid.h), for building the MegaMol adapter where
// the MegaMol tree is absent: an axis-aligned box given by its six faces.
#pragma once

namespace vislib::math {

template<class T>
class Cuboid {
public:
    Cuboid() = default;
    Cuboid(T l, T b, T k, T r, T t, T f) : l_(l), b_(b), k_(k), r_(r), t_(t), f_(f) {}
    void Set(T l, T b, T k, T r, T t, T f) {
        l_ = l, b_ = b, k_ = k, r_ = r, t_ = t, f_ = f;
    }
    T Left() const { return l_; }
    T Bottom() const { return b_; }
    T Back() const { return k_; }
    T Right() const { return r_; }
    T Top() const { return t_; }
    T Front() const { return f_; }
    T Width() const { return r_ - l_; }
    T Height() const { return t_ - b_; }
    T Depth() const { return f_ - k_; }

private:
    T l_ = 0, b_ = 0, k_ = 0, r_ = 0, t_ = 0, f_ = 0;
};

}  // namespace vislib::math
