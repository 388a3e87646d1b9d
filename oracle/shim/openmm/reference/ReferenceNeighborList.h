/* Oracle shim: pair-list types. The harness fills NeighborList itself
 * (brute-force minimum-image half list, d <= cutoff inclusive). */
#ifndef MBPOL_SHIM_NEIGHBORLIST_H
#define MBPOL_SHIM_NEIGHBORLIST_H
#include <vector>
#include <utility>
#include "openmm/reference/RealVec.h"
namespace OpenMM {
typedef unsigned int AtomIndex;
typedef std::pair<AtomIndex, AtomIndex> AtomPair;
typedef std::vector<AtomPair> NeighborList;
typedef std::vector<RealVec> AtomLocationList;
}
#endif
