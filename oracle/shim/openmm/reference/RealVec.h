/* Oracle shim: minimal stand-in for OpenMM's RealVec/Vec3 value type, just
 * enough for the MB-pol Reference-platform sources to compile unmodified.
 * Test infrastructure only; never linked into the product library. */
#ifndef MBPOL_SHIM_REALVEC_H
#define MBPOL_SHIM_REALVEC_H
#include <cmath>
#include <ostream>
#include "openmm/reference/SimTKOpenMMRealType.h"
namespace OpenMM {
class RealVec {
public:
    RealVec() { d[0] = d[1] = d[2] = 0.0; }
    RealVec(double x, double y, double z) { d[0] = x; d[1] = y; d[2] = z; }
    double operator[](int i) const { return d[i]; }
    double& operator[](int i) { return d[i]; }
    RealVec operator+() const { return *this; }
    RealVec operator-() const { return RealVec(-d[0], -d[1], -d[2]); }
    RealVec operator+(const RealVec& o) const { return RealVec(d[0]+o.d[0], d[1]+o.d[1], d[2]+o.d[2]); }
    RealVec operator-(const RealVec& o) const { return RealVec(d[0]-o.d[0], d[1]-o.d[1], d[2]-o.d[2]); }
    RealVec operator*(double s) const { return RealVec(d[0]*s, d[1]*s, d[2]*s); }
    RealVec operator/(double s) const { return RealVec(d[0]/s, d[1]/s, d[2]/s); }
    RealVec& operator+=(const RealVec& o) { d[0]+=o.d[0]; d[1]+=o.d[1]; d[2]+=o.d[2]; return *this; }
    RealVec& operator-=(const RealVec& o) { d[0]-=o.d[0]; d[1]-=o.d[1]; d[2]-=o.d[2]; return *this; }
    RealVec& operator*=(double s) { d[0]*=s; d[1]*=s; d[2]*=s; return *this; }
    RealVec& operator/=(double s) { d[0]/=s; d[1]/=s; d[2]/=s; return *this; }
    double dot(const RealVec& o) const { return d[0]*o.d[0] + d[1]*o.d[1] + d[2]*o.d[2]; }
    RealVec cross(const RealVec& o) const {
        return RealVec(d[1]*o.d[2]-d[2]*o.d[1], d[2]*o.d[0]-d[0]*o.d[2], d[0]*o.d[1]-d[1]*o.d[0]);
    }
private:
    double d[3];
};
typedef RealVec Vec3;
}
#endif
