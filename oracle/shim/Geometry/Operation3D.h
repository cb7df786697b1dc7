// Test-infrastructure shim (oracle only). Restates the three C3DOperation
// calls the reference parser makes on quadrilateral panels:
// PlaneFromPolygon (Newell normal, unit-normalised, plane through the vertex
// average), PointPlaneDist (signed distance) and FindProjPlane (drop the axis
// of the largest normal component).
#ifndef FCG_SHIM_OPERATION3D_H
#define FCG_SHIM_OPERATION3D_H

#include "Geometry3D.h"

#define C3D_OK 0
#define C3D_POINTS_ARE_COLLINEAR 1
#define C3D_DIR_X 0
#define C3D_DIR_Y 1
#define C3D_DIR_Z 2

class C3DOperation {
public:
    int PlaneFromPolygon(C3DPlane &plane, double &mod, const C3DVector *pts, int n) {
        C3DVector nrm, avg;
        for (int i = 0; i < n; i++) {
            int j = (i + 1) % n;
            nrm.x += (pts[i].y - pts[j].y) * (pts[i].z + pts[j].z);
            nrm.y += (pts[i].z - pts[j].z) * (pts[i].x + pts[j].x);
            nrm.z += (pts[i].x - pts[j].x) * (pts[i].y + pts[j].y);
            avg += pts[i];
        }
        mod = Mod(nrm);
        if (mod < 1e-300) return C3D_POINTS_ARE_COLLINEAR;
        nrm = nrm / mod;
        avg = avg / (double)n;
        plane.m_vecNormal = nrm;
        plane.m_dD = -DotProd(nrm, avg);
        return C3D_OK;
    }
    double PointPlaneDist(const C3DVector &p, const C3DPlane &plane) {
        return DotProd(plane.m_vecNormal, p) + plane.m_dD;
    }
    char FindProjPlane(char *c1, char *c2, const C3DVector &normal) {
        double ax = fabs(normal.x), ay = fabs(normal.y), az = fabs(normal.z);
        char c3;
        if (ax >= ay && ax >= az) c3 = C3D_DIR_X;
        else if (ay >= az) c3 = C3D_DIR_Y;
        else c3 = C3D_DIR_Z;
        *c1 = (char)((c3 + 1) % 3);
        *c2 = (char)((c3 + 2) % 3);
        return c3;
    }
};

#endif
