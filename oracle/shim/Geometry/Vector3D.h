// Test-infrastructure shim (oracle only; never linked into the product).
//
// FasterCap includes "Geometry/Vector3D.h" from the FastFieldSolvers "Geometry"
// package, which is not part of the reference tree and has no pinned version.
// This header restates only the interface the reference's Solver/*.cpp use
// (members x,y,z, pos(), [], +, -, unary -, scalar * and /, compound
// assignment, Mod(), Normalize(), Invert(), free Mod/DotProd/CrossProd and the
// C3D_CROSSPROD / C3D_DOTPROD macros).
//
// Arithmetic semantics chosen here (the upstream semantics are unpinned):
//  * an operation between two vectors of the same element type is done in
//    that type (float - float stays float);
//  * mixed float/double vector operations and vector-by-scalar operations
//    follow the C++ usual arithmetic conversions component-wise, and the
//    result vector has the promoted element type;
//  * Mod(), DotProd(), CrossProd() and the member Mod() always work in double
//    (a float vector is widened first);
//  * compound assignment computes in the promoted type and rounds on store.
// The product's host builder and the C oracle restate exactly these rules.
#ifndef FCG_SHIM_VECTOR3D_H
#define FCG_SHIM_VECTOR3D_H

#include <math.h>
#include <type_traits>

#ifndef _ASSERT
#define _ASSERT(x) ((void)0)
#endif

template <class T> class C3DVecT {
public:
    T x, y, z;
    C3DVecT() : x(0), y(0), z(0) {}
    C3DVecT(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class U>
    C3DVecT(const C3DVecT<U> &o) : x((T)o.x), y((T)o.y), z((T)o.z) {}

    void pos(T a, T b, T c) { x = a; y = b; z = c; }
    T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }

    C3DVecT operator-() const { return C3DVecT(-x, -y, -z); }

    template <class U> C3DVecT &operator+=(const C3DVecT<U> &o) {
        x = (T)(x + o.x); y = (T)(y + o.y); z = (T)(z + o.z); return *this;
    }
    template <class U> C3DVecT &operator-=(const C3DVecT<U> &o) {
        x = (T)(x - o.x); y = (T)(y - o.y); z = (T)(z - o.z); return *this;
    }
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    C3DVecT &operator*=(S s) { x = (T)(x * s); y = (T)(y * s); z = (T)(z * s); return *this; }
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    C3DVecT &operator/=(S s) { x = (T)(x / s); y = (T)(y / s); z = (T)(z / s); return *this; }

    double Mod() const {
        double a = x, b = y, c = z;
        return sqrt(a * a + b * b + c * c);
    }
    void Normalize() {
        double m = Mod();
        x = (T)(x / m); y = (T)(y / m); z = (T)(z / m);
    }
    void Invert() { x = -x; y = -y; z = -z; }
};

typedef C3DVecT<double> C3DVector;
typedef C3DVecT<float> C3DVector_float;

template <class A, class B>
inline C3DVecT<typename std::common_type<A, B>::type> operator+(const C3DVecT<A> &a, const C3DVecT<B> &b) {
    return C3DVecT<typename std::common_type<A, B>::type>(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <class A, class B>
inline C3DVecT<typename std::common_type<A, B>::type> operator-(const C3DVecT<A> &a, const C3DVecT<B> &b) {
    return C3DVecT<typename std::common_type<A, B>::type>(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <class A, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline C3DVecT<typename std::common_type<A, S>::type> operator*(const C3DVecT<A> &a, S s) {
    return C3DVecT<typename std::common_type<A, S>::type>(a.x * s, a.y * s, a.z * s);
}
template <class A, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline C3DVecT<typename std::common_type<A, S>::type> operator*(S s, const C3DVecT<A> &a) {
    return C3DVecT<typename std::common_type<A, S>::type>(a.x * s, a.y * s, a.z * s);
}
template <class A, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline C3DVecT<typename std::common_type<A, S>::type> operator/(const C3DVecT<A> &a, S s) {
    return C3DVecT<typename std::common_type<A, S>::type>(a.x / s, a.y / s, a.z / s);
}
template <class A, class B>
inline bool operator==(const C3DVecT<A> &a, const C3DVecT<B> &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

inline double Mod(const C3DVector &a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline double Mod2(const C3DVector &a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline double DotProd(const C3DVector &a, const C3DVector &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline C3DVector CrossProd(const C3DVector &a, const C3DVector &b) {
    return C3DVector(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

#define C3D_CROSSPROD(res, a, b) \
    { (res).x = (a).y * (b).z - (a).z * (b).y; (res).y = (a).z * (b).x - (a).x * (b).z; (res).z = (a).x * (b).y - (a).y * (b).x; }
#define C3D_DOTPROD(a, b) ((a).x * (b).x + (a).y * (b).y + (a).z * (b).z)

#endif
