/* Oracle shim: Vec3 is the same value type as RealVec here. */
#ifndef MBPOL_SHIM_VEC3_H
#define MBPOL_SHIM_VEC3_H
#include "openmm/reference/RealVec.h"
#endif
