/* Oracle shim: erfc comes from <cmath> on this platform. */
#include <cmath>
