// Test-infrastructure shim (oracle only). Restates the part of the
// FastFieldSolvers "LinAlgebra" package the reference uses: CLin_Vector (a
// resizable double vector), CLin_Range (an aliasing view: assigning a vector to
// a range makes the range refer to that vector's storage, which the
// reference's matrix-vector product relies on to write its output), mod()
// (2-norm), dot_prod() and the ASSERT macro (compiled out).
#ifndef FCG_SHIM_VECT_H
#define FCG_SHIM_VECT_H

#include <math.h>
#include <stddef.h>
#include <vector>

#ifndef ASSERT
#define ASSERT(x) ((void)0)
#endif

typedef long CLin_subscript;

class CLin_Vector {
public:
    std::vector<double> m_v;
    CLin_Vector() {}
    explicit CLin_Vector(CLin_subscript n) : m_v((size_t)n, 0.0) {}
    CLin_Vector(CLin_subscript n, double val) : m_v((size_t)n, val) {}
    bool newsize(CLin_subscript n) { m_v.assign((size_t)n, 0.0); return true; }
    void destroy() { std::vector<double>().swap(m_v); }
    CLin_subscript size() const { return (CLin_subscript)m_v.size(); }
    CLin_subscript dim() const { return size(); }
    double &operator[](CLin_subscript i) { return m_v[(size_t)i]; }
    const double &operator[](CLin_subscript i) const { return m_v[(size_t)i]; }
    CLin_Vector &operator=(double val) { for (size_t i = 0; i < m_v.size(); i++) m_v[i] = val; return *this; }
    double *data() { return m_v.data(); }
};

class CLin_Range {
public:
    double *m_p;
    CLin_subscript m_n;
    CLin_Range() : m_p(NULL), m_n(0) {}
    CLin_Range(CLin_Vector &v) : m_p(v.data()), m_n(v.size()) {}
    // view of elements [first, last] (inclusive)
    CLin_Range(CLin_Vector &v, CLin_subscript first, CLin_subscript last) : m_p(v.data() + first), m_n(last - first + 1) {}
    CLin_Range &operator=(CLin_Vector &v) { m_p = v.data(); m_n = v.size(); return *this; }
    double &operator[](CLin_subscript i) { return m_p[i]; }
    CLin_subscript size() const { return m_n; }
};

inline CLin_Vector operator-(const CLin_Vector &a, const CLin_Vector &b) {
    CLin_Vector r(a.size());
    for (CLin_subscript i = 0; i < a.size(); i++) r[i] = a[i] - b[i];
    return r;
}

inline CLin_Vector operator+(const CLin_Vector &a, const CLin_Vector &b) {
    CLin_Vector r(a.size());
    for (CLin_subscript i = 0; i < a.size(); i++) r[i] = a[i] + b[i];
    return r;
}

inline CLin_Vector operator/(const CLin_Vector &a, double d) {
    CLin_Vector r(a.size());
    for (CLin_subscript i = 0; i < a.size(); i++) r[i] = a[i] / d;
    return r;
}

inline double mod(const CLin_Vector &v) {
    double s = 0.0;
    for (CLin_subscript i = 0; i < v.size(); i++) s += v[i] * v[i];
    return sqrt(s);
}

inline double dot_prod(const CLin_Vector &a, const CLin_Vector &b) {
    double s = 0.0;
    for (CLin_subscript i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
}

#endif
