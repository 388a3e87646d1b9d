/* Oracle harness (test infrastructure only): C entry points to the
 * reference's generated polynomial evaluators and their coefficient tables
 * (platforms/reference/src/poly-2b-v6x.cpp, poly-3b-v2x.cpp,
 * mbpol_2body_constants.h:52-1210, mbpol_3body_constants.h:22-1188).
 * Compiled twice: -DPOLY3B selects the three-body variant. */
#ifdef POLY3B
#include "mbpol_3body_constants.h"
#include "poly-3b-v2x.h"
extern "C" double ref_poly3b_eval(const double* x, double* g) { return poly_3b_v2x::eval(thefit, x, g); }
extern "C" int ref_poly3b_coeffs(double* out) {
    for (int i = 0; i < 1163; ++i) out[i] = thefit[i];
    return 1163;
}
#else
#include "mbpol_2body_constants.h"
#include "poly-2b-v6x.h"
extern "C" double ref_poly2b_eval(const double* x, double* g) { return poly_2b_v6x_eval(thefit, x, g); }
extern "C" int ref_poly2b_coeffs(double* out) {
    for (int i = 0; i < 1153; ++i) out[i] = thefit[i];
    return 1153;
}
#endif
