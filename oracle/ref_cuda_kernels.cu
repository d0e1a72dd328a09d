// ref_cuda_kernels.cu -- TEST INFRASTRUCTURE.  The reference's own device
// code, compiled where it lies (read-only) into a sm_103a cubin by
// oracle/build_ref.sh: the edge, volume, eta-max and initial-dt kernels
// (Volumen_kernel.cu, which includes Arista_kernel.cu, Matriz.cu and
// Constantes.hxx) and the dt min-reduction (Reduccion_kernel.cu), through
// ref_cuda_shim.h.  Nothing from the reference is copied here; the cubin
// goes to oracle/_ref/ only (git-ignored) and is loaded by
// ref_cuda_driver.cpp.
#include "ref_cuda_shim.h"

#include "Volumen_kernel.cu"
#include "Reduccion_kernel.cu"
