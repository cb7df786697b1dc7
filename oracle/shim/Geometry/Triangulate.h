// Test-infrastructure shim (oracle only). The reference uses a constrained
// Delaunay triangulator only for planar quadrilaterals that are not close to
// rectangles. That code is not available, so this stand-in produces no
// triangles and reports it on stderr; inputs used by the tests never reach it.
#ifndef FCG_SHIM_TRIANGULATE_H
#define FCG_SHIM_TRIANGULATE_H

#include <vector>
#include <stdio.h>
#include "Vector2D.h"

class C2DTriangulate {
public:
    std::vector<C2DVector> vertexes;
    void Triangulate() { fprintf(stderr, "oracle shim: quality triangulation of a non-rectangular quadrilateral is not available\n"); }
    void InsertConstrEdge(const C2DVector &, const C2DVector &) {}
    void DeleteCWEdges(const C2DVector &, const C2DVector &) {}
    void Refine(double) {}
    void GenerateTriangles() {}
    long GetTriangleNum() { return 0; }
    void GetTriangleCoords(long, C2DVector *, C2DVector *, C2DVector *) {}
};

#endif
