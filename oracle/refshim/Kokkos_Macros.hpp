// Kokkos_Macros.hpp — host-only stand-in for the Kokkos function-qualifier
// macros the reference's kernel headers use.  TEST INFRASTRUCTURE ONLY.
#ifndef FST_KOKKOS_SHIM_MACROS_HPP
#define FST_KOKKOS_SHIM_MACROS_HPP
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#endif
