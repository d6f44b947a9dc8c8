// Atomics live in Kokkos_Core.hpp in this stand-in (see there).
#include "Kokkos_Core.hpp"
