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

namespace {

// The far-field kernel's bounded wait on an mbarrier that expects bytes no copy will deliver: the
// wait runs out after `limit` cycles and raises NB_ERRBIT_ASYNC, as k_m2l does (nothing was issued,
// so nothing is in flight when the kernel returns)
__global__ void k_copy_wait_selftest(int32_t* info, long long limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        nbfmm::mbar_init(&bar, 1);
        nbfmm::fence_mbar_init();
    }
    __syncwarp();
    if (threadIdx.x == 0) nbfmm::mbar_expect_tx(&bar, 16);
    __syncwarp();
    if (!nbfmm::mbar_wait_warp(&bar, 0, limit) && threadIdx.x == 0)
        atomicOr((unsigned int*)&info[INFO_ERR], NB_ERRBIT_ASYNC);
}

}  // namespace

int nb_copy_wait_selftest(nbody_ctx* c) {
    NB_CU(c, cudaMemsetAsync(c->info.p, 0, sizeof(int32_t), c->st));
    k_copy_wait_selftest<<<1, 32, 0, c->st>>>(DP<int32_t>(c->info), c->copy_cycles);
    NB_LAUNCHED(c, "copy wait self-test");
    NB_CU(c, cudaMemcpyAsync(c->h_info, c->info.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    return nb_check_async(c);
}

NB_DBG_ACCESSOR(fmm_fp32)
