// Instantiates the FMM kernels for one precision form (compiled as its own
// translation unit so the forms build in parallel).
#include "fmm_impl.cuh"
#include "adjoint_impl.cuh"

int nb_fmm_forces_mixed(nbody_ctx* c, int integ, bool want_pot) {
    return nbfmm::fmm_dispatch<NBODY_PREC_MIXED>(c, integ, want_pot);
}

int nb_fmm_vjp_mixed(nbody_ctx* c, double coef) { return nbfmm::vjp_dispatch<NBODY_PREC_MIXED>(c, coef); }

NB_DBG_ACCESSOR(fmm_mixed)
