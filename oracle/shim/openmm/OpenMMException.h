/* Oracle shim: exception type thrown by the Reference code. */
#ifndef MBPOL_SHIM_EXCEPTION_H
#define MBPOL_SHIM_EXCEPTION_H
#include <stdexcept>
#include <string>
namespace OpenMM {
class OpenMMException : public std::runtime_error {
public:
    explicit OpenMMException(const std::string& m) : std::runtime_error(m) {}
};
}
#endif
