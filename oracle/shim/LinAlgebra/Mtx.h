// Test-infrastructure shim (oracle only). CLin_Matrix restated from the
// reference's usage: newsize(rows, cols), [i][j], num_rows/num_cols, dim(1|2),
// fill by scalar assignment, difference, and the Frobenius norms FNorm(M) and
// FNorm(Re, Im).
#ifndef FCG_SHIM_MTX_H
#define FCG_SHIM_MTX_H

#include "Vect.h"

class CLin_Matrix {
public:
    std::vector<double> m_a;
    CLin_subscript m_r, m_c;
    CLin_Matrix() : m_r(0), m_c(0) {}
    CLin_Matrix(CLin_subscript r, CLin_subscript c) : m_a((size_t)(r * c), 0.0), m_r(r), m_c(c) {}
    bool newsize(CLin_subscript r, CLin_subscript c) { m_r = r; m_c = c; m_a.assign((size_t)(r * c), 0.0); return true; }
    void destroy() { std::vector<double>().swap(m_a); m_r = m_c = 0; }
    double *operator[](CLin_subscript i) { return &m_a[(size_t)(i * m_c)]; }
    const double *operator[](CLin_subscript i) const { return &m_a[(size_t)(i * m_c)]; }
    CLin_subscript num_rows() const { return m_r; }
    CLin_subscript num_cols() const { return m_c; }
    CLin_subscript dim(int d) const { return d == 1 ? m_r : m_c; }
    CLin_Matrix &operator=(double v) { for (size_t i = 0; i < m_a.size(); i++) m_a[i] = v; return *this; }
};

inline CLin_Matrix operator-(const CLin_Matrix &a, const CLin_Matrix &b) {
    CLin_Matrix r(a.m_r, a.m_c);
    for (size_t i = 0; i < r.m_a.size(); i++) r.m_a[i] = a.m_a[i] - b.m_a[i];
    return r;
}

inline double FNorm(const CLin_Matrix &a) {
    double s = 0.0;
    for (size_t i = 0; i < a.m_a.size(); i++) s += a.m_a[i] * a.m_a[i];
    return sqrt(s);
}

inline double FNorm(const CLin_Matrix &re, const CLin_Matrix &im) {
    double s = 0.0;
    for (size_t i = 0; i < re.m_a.size(); i++) s += re.m_a[i] * re.m_a[i] + im.m_a[i] * im.m_a[i];
    return sqrt(s);
}

#endif
