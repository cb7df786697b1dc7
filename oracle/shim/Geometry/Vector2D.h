// Test-infrastructure shim (oracle only). Restates the 2D vector interface of
// the FastFieldSolvers "Geometry" package as used by the reference's 2D code,
// which is compiled into the oracle only because Autorefine.cpp references it.
// Same arithmetic rules as the 3D shim.
#ifndef FCG_SHIM_VECTOR2D_H
#define FCG_SHIM_VECTOR2D_H

#include <math.h>
#include <type_traits>

template <class T> class C2DVecT {
public:
    T x, y;
    C2DVecT() : x(0), y(0) {}
    C2DVecT(T a, T b) : x(a), y(b) {}
    template <class U>
    C2DVecT(const C2DVecT<U> &o) : x((T)o.x), y((T)o.y) {}

    void pos(T a, T b) { x = a; y = b; }
    T &operator[](int i) { return i == 0 ? x : y; }
    const T &operator[](int i) const { return i == 0 ? x : y; }
    C2DVecT operator-() const { return C2DVecT(-x, -y); }

    template <class U> C2DVecT &operator+=(const C2DVecT<U> &o) { x = (T)(x + o.x); y = (T)(y + o.y); return *this; }
    template <class U> C2DVecT &operator-=(const C2DVecT<U> &o) { x = (T)(x - o.x); y = (T)(y - o.y); return *this; }
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    C2DVecT &operator*=(S s) { x = (T)(x * s); y = (T)(y * s); return *this; }
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    C2DVecT &operator/=(S s) { x = (T)(x / s); y = (T)(y / s); return *this; }

    double Mod() const { double a = x, b = y; return sqrt(a * a + b * b); }
    void Normalize() { double m = Mod(); x = (T)(x / m); y = (T)(y / m); }
    void Invert() { x = -x; y = -y; }
};

typedef C2DVecT<double> C2DVector;
typedef C2DVecT<float> C2DVector_float;
typedef C2DVecT<double> C2DVertex;

template <class A, class B>
inline C2DVecT<typename std::common_type<A, B>::type> operator+(const C2DVecT<A> &a, const C2DVecT<B> &b) {
    return C2DVecT<typename std::common_type<A, B>::type>(a.x + b.x, a.y + b.y);
}
template <class A, class B>
inline C2DVecT<typename std::common_type<A, B>::type> operator-(const C2DVecT<A> &a, const C2DVecT<B> &b) {
    return C2DVecT<typename std::common_type<A, B>::type>(a.x - b.x, a.y - b.y);
}
template <class A, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline C2DVecT<typename std::common_type<A, S>::type> operator*(const C2DVecT<A> &a, S s) {
    return C2DVecT<typename std::common_type<A, S>::type>(a.x * s, a.y * s);
}
template <class A, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline C2DVecT<typename std::common_type<A, S>::type> operator*(S s, const C2DVecT<A> &a) {
    return C2DVecT<typename std::common_type<A, S>::type>(a.x * s, a.y * s);
}
template <class A, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
inline C2DVecT<typename std::common_type<A, S>::type> operator/(const C2DVecT<A> &a, S s) {
    return C2DVecT<typename std::common_type<A, S>::type>(a.x / s, a.y / s);
}

inline double Mod(const C2DVector &a) { return sqrt(a.x * a.x + a.y * a.y); }
inline double DotProd(const C2DVector &a, const C2DVector &b) { return a.x * b.x + a.y * b.y; }
inline double CrossProd(const C2DVector &a, const C2DVector &b) { return a.x * b.y - a.y * b.x; }

#endif
