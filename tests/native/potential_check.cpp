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
