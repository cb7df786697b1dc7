// Test helper: evaluates the reference-order analytic triangle potential
// (fcg_potential_opt) and the reduced-cost device form (fcg_potential_opt_fast)
// on the same inputs, for tests/test_potential_forms.py.
#include "../../fastercap_gb300/csrc/fc_potential.h"

extern "C" void pot_pair(int64_t n, const float *tri, const double *pts, double *ref, double *fast) {
    for (int64_t i = 0; i < n; i++) {
        const float *v = tri + 9 * i;
        fcg_d3 r = fcg_mk(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
        fcg_tri64 t;
        fcg_tri64_make(v, t);
        ref[i] = fcg_potential_opt(r, v);
        fast[i] = fcg_potential_opt_fast(r, v, t);
    }
}

// FP32 near-field form at float offsets from the source centroid: value (as
// double) and whether the FP32 evaluation decided every guard; the FP64
// formula at the same float point for comparison.
extern "C" void pot32_pair(int64_t n, const float *tri, const float *pts, double *ref, double *f32, int *ok) {
    for (int64_t i = 0; i < n; i++) {
        const float *v = tri + 9 * i;
        float c[3];
        for (int k = 0; k < 3; k++) c[k] = (float)(((double)v[k] + (double)v[3 + k] + (double)v[6 + k]) / 3.0);
        fcg_tri32 t;
        fcg_tri32_make(v, c, t);
        const float *p = pts + 3 * i;
        float off[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
        fcg_d3 r = fcg_mk(c[0], c[1], c[2]);
        r = fcg_mk(r.x + off[0], r.y + off[1], r.z + off[2]);
        ref[i] = fcg_potential_opt(r, v);
        float o = 0.0f;
        ok[i] = fcg_potential32(off[0], off[1], off[2], t, &o) ? 1 : 0;
        f32[i] = o;
    }
}
