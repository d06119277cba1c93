// Stand-in for the reference's modules/geometry/Dim2Vectorial.h (TEST
// INFRASTRUCTURE, used only by oracle/build_ref.sh to compile the
// reference's geometry reader with gcc).  Same interface: a Dim2<T> with
// component-wise += and -= and the binary + and -.  The reference's version
// names the dependent base's members without this->, which MSVC accepts and
// gcc's two-phase lookup rejects; here they are named through this->.
#pragma once

#include "modules/geometry/Dim2.h"

template <typename T>
struct Dim2Vectorial : public Dim2<T> {
    Dim2Vectorial(T const &a, T const &b) : Dim2<T>(a, b) {}
    virtual ~Dim2Vectorial() = default;

    Dim2Vectorial &operator+=(Dim2Vectorial const &o) {
        this->x += o.x;
        this->y += o.y;
        return *this;
    }
    Dim2Vectorial &operator-=(Dim2Vectorial const &o) {
        this->x -= o.x;
        this->y -= o.y;
        return *this;
    }
    friend Dim2Vectorial operator+(Dim2Vectorial a, Dim2Vectorial const &b) { return a += b; }
    friend Dim2Vectorial operator-(Dim2Vectorial a, Dim2Vectorial const &b) { return a -= b; }
};
