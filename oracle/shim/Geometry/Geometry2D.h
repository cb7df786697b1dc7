// Test-infrastructure shim (oracle only): 2D bounding box of the
// FastFieldSolvers "Geometry" package, as used by the reference's 2D parser.
#ifndef FCG_SHIM_GEOMETRY2D_H
#define FCG_SHIM_GEOMETRY2D_H

#include "Vector2D.h"

class C2DBBox {
public:
    C2DVector min_point, max_point;
    bool m_bEmpty;
    C2DBBox() : m_bEmpty(true) {}
    void Clear() { m_bEmpty = true; min_point = C2DVector(); max_point = C2DVector(); }
    C2DBBox &operator+=(const C2DVector &p) {
        if (m_bEmpty) { min_point = p; max_point = p; m_bEmpty = false; return *this; }
        for (int i = 0; i < 2; i++) {
            if (p[i] < min_point[i]) min_point[i] = p[i];
            if (p[i] > max_point[i]) max_point[i] = p[i];
        }
        return *this;
    }
};

#endif
