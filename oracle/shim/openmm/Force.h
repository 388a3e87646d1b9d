/* Oracle shim: just enough of OpenMM::Force for the MB-pol API headers. */
#ifndef MBPOL_SHIM_FORCE_H
#define MBPOL_SHIM_FORCE_H
namespace OpenMM {
class ForceImpl;
class Context;
class Force {
public:
    virtual ~Force() {}
protected:
    virtual ForceImpl* createImpl() const = 0;
};
}
#endif
