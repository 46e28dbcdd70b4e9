// Kokkos math subset used by the reference hot path -- TEST INFRASTRUCTURE ONLY.
// fabs and fmax are exact IEEE operations; they forward to <cmath>.
#pragma once
#include <cmath>

namespace Kokkos {
using std::fabs;
using std::fmax;
using std::fmin;
using std::sqrt;
}  // namespace Kokkos
