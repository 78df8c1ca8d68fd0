// Forwards to the single-header Kokkos stand-in used for the pin tests.
#include "Kokkos_Core.hpp"
