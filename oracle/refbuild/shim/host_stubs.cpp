// Host-side symbols that the reference normally takes from its Python binding
// (src_python/common_Py.cpp:29-33) or from a vendored file that is missing
// from the source tree (external/cubature/clencurt.h, needed by pcubature.c).
// The oracle drives the reference from C++, so Ctrl-C polling is a no-op, and
// the p-adaptive cubature (only used when the global flag use_pcubature is
// set) reports failure instead of integrating.
#include <cstddef>
#include <stdexcept>

void check_signals() {}

extern "C" {
typedef int (*integrand_v)(unsigned, size_t, const double*, void*, unsigned, double*);
int pcubature_v(unsigned, integrand_v, void*, unsigned, const double*, const double*, size_t,
                double, double, int, double*, double*) {
  throw std::runtime_error("p-adaptive cubature is not available in the oracle build");
}
}
