// ref_driver_pouliquen.cpp -- TEST INFRASTRUCTURE.  The same host driver as
// ref_driver.cpp, around the reference's own kernels compiled with the
// Pouliquen friction law: Constantes.hxx:17 defines COULOMB, which selects
// the Coulomb law at Arista_kernel.cu:8; including Constantes.hxx first and
// undefining the macro before the kernel sources are read makes the
// unmodified sources take their #else branch (Arista_kernel.cu:20-58), as a
// build of the reference with line 17 removed would.  Constantes.hxx's
// include guard keeps the macro undefined when the kernels include it again,
// so it is included here the way Matriz.cu:4-6 includes it (with the GPU
// constants and texture declarations).
//
// Built by oracle/build_ref.sh into oracle/_ref/liblsh_ref_pouliquen.so.
#include "ref_shim.h"

#define CONSTANTES_GPU
#include "Constantes.hxx"
#undef CONSTANTES_GPU
#undef COULOMB

#include "ref_driver.cpp"
