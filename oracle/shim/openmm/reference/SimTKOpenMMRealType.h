/* Oracle shim: RealOpenMM is double and the math macros map to <cmath>. */
#ifndef MBPOL_SHIM_REALTYPE_H
#define MBPOL_SHIM_REALTYPE_H
#include <cmath>
typedef double RealOpenMM;
#define SQRT(x) std::sqrt(x)
#define EXP(x) std::exp(x)
#define POW(x, y) std::pow(x, y)
#define FLOOR(x) std::floor(x)
#define COS(x) std::cos(x)
#define SIN(x) std::sin(x)
#define FABS(x) std::fabs(x)
#define LOG(x) std::log(x)
#endif
