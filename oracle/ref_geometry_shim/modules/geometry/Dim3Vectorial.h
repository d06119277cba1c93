// Stand-in for the reference's modules/geometry/Dim3Vectorial.h (TEST
// INFRASTRUCTURE, used only by oracle/build_ref.sh to compile the
// reference's geometry reader with gcc): the three-component counterpart of
// the Dim2Vectorial stand-in beside it, members named through this->.
#pragma once

#include "modules/geometry/Dim3.h"

template <typename T>
struct Dim3Vectorial : public Dim3<T> {
    Dim3Vectorial(T const &a, T const &b, T const &c) : Dim3<T>(a, b, c) {}
    virtual ~Dim3Vectorial() = default;

    Dim3Vectorial &operator+=(Dim3Vectorial const &o) {
        this->x += o.x;
        this->y += o.y;
        this->z += o.z;
        return *this;
    }
    Dim3Vectorial &operator-=(Dim3Vectorial const &o) {
        this->x -= o.x;
        this->y -= o.y;
        this->z -= o.z;
        return *this;
    }
    friend Dim3Vectorial operator+(Dim3Vectorial a, Dim3Vectorial const &b) { return a += b; }
    friend Dim3Vectorial operator-(Dim3Vectorial a, Dim3Vectorial const &b) { return a -= b; }
};
