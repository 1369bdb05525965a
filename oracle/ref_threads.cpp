// ref_threads.cpp -- thread count of the Kokkos stand-in's parallel_for in
// the reference build (oracle/_ref/libxtref.so).  TEST INFRASTRUCTURE ONLY.
#include "kokkos_shim/Kokkos_Core.hpp"

extern "C" void xtref_set_threads(int n) { Kokkos::shim_threads() = n > 0 ? n : 1; }
