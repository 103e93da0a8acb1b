// Instantiates the FMM kernels for one precision form (compiled as its own
// translation unit so the forms build in parallel).
#include "fmm_impl.cuh"
#include "adjoint_impl.cuh"

int nb_fmm_forces_fp32(nbody_ctx* c, int integ, bool want_pot) {
    return nbfmm::fmm_dispatch<NBODY_PREC_FP32>(c, integ, want_pot);
}

int nb_fmm_vjp_fp32(nbody_ctx* c, double coef) { return nbfmm::vjp_dispatch<NBODY_PREC_FP32>(c, coef); }

extern "C" int64_t nbody_flops_per_m2l(int order) {
    return order >= 1 && order <= NB_PMAX ? (int64_t)nb_m2l_flops_tab[order] : 0;
}

extern "C" int64_t nbody_flops_per_p2p(void) { return 20; }
