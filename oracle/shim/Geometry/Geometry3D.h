// Test-infrastructure shim (oracle only). Restates the bounding box, plane and
// list types of the FastFieldSolvers "Geometry" package as the reference uses
// them (C3DBBox +=, MaxSide, min_point/max_point, Clear; C3DPlane normal and
// Point3Dfrom2D; C3DList as a std::list).
#ifndef FCG_SHIM_GEOMETRY3D_H
#define FCG_SHIM_GEOMETRY3D_H

#include <list>
#include "Vector3D.h"
#include "Vector2D.h"

// Axis-aligned bounding box of points, kept in double.
class C3DBBox {
public:
    C3DVector min_point, max_point;
    bool m_bEmpty;
    C3DBBox() : m_bEmpty(true) {}
    void Clear() { m_bEmpty = true; min_point = C3DVector(); max_point = C3DVector(); }
    C3DBBox &operator+=(const C3DVector &p) {
        if (m_bEmpty) { min_point = p; max_point = p; m_bEmpty = false; return *this; }
        for (int i = 0; i < 3; i++) {
            if (p[i] < min_point[i]) min_point[i] = p[i];
            if (p[i] > max_point[i]) max_point[i] = p[i];
        }
        return *this;
    }
    // 2D points are added with z = 0
    C3DBBox &operator+=(const C2DVector &p) { return (*this) += C3DVector(p.x, p.y, 0.0); }
    // index of the longest extent; ties resolve to the lower index
    unsigned char MaxSide() const {
        double dx = max_point.x - min_point.x, dy = max_point.y - min_point.y, dz = max_point.z - min_point.z;
        if (dx >= dy && dx >= dz) return 0;
        if (dy >= dz) return 1;
        return 2;
    }
};

// Plane n.p + d = 0 with unit normal n.
class C3DPlane {
public:
    C3DVector m_vecNormal;
    double m_dD;
    C3DPlane() : m_dD(0.0) {}
    // lift a 2D point of the projection plane (c1, c2) back onto the plane
    C3DVector Point3Dfrom2D(const C2DVector &p, char c1, char c2, char c3) const {
        C3DVector r;
        r[c1] = p.x;
        r[c2] = p.y;
        r[c3] = -(m_dD + m_vecNormal[c1] * p.x + m_vecNormal[c2] * p.y) / m_vecNormal[c3];
        return r;
    }
};

template <class T> class C3DList : public std::list<T> {};

#endif
