// Individual (block) time steps on top of the fused step.  The reference integrates with one fixed
// dt and lists a variable time step among its goals (its TODO); this is the hierarchical form:
// each particle takes dt_i = dt_max / 2^k_i, with k_i the smallest level whose step is no longer
// than eta sqrt(length / |a_i|) (the adaptive criterion of nbody_set_timestep_control, per
// particle), clamped to 0 .. K.  One base step of dt_max runs 2^K substeps of dt_max / 2^K:
//   t0:        every particle takes its level from a(t0) and an opening half kick;
//   each substep s = 1 .. 2^K: every particle drifts by dt_max / 2^K, the forces are evaluated, and
//              each particle whose step ends at s (s a multiple of 2^(K - k_i)) takes its closing
//              half kick; if s < 2^K it then takes a new level from the new acceleration (no coarser
//              than the substep grid allows at s: k >= K - trailing_zeros(s)) and an opening half
//              kick for its next step.
// At the end of the base step every particle has closed its step, so positions and velocities are
// synchronous again.  With K = 0 this is the kick-drift-kick leapfrog of one fixed step.  A substep
// at which some particle's step ends evaluates the whole tree, with the near field and L2P only for
// the leaves holding such a particle; a substep at which none ends only drifts.  The kicks are per
// particle, deterministic.
#include "nbody_internal.cuh"

namespace {

constexpr int TB = 256;
inline unsigned nblk(int64_t n) { return (unsigned)((n + TB - 1) / TB); }

// level of a particle with |a|^2 = a2: smallest k in 0 .. K with dt_max 2^-k <= eta sqrt(len / |a|)
__device__ __forceinline__ int block_level(double a2, double eta, double len, double dt_max, int K) {
    if (!(a2 > 0.0)) return 0;
    const double want = eta * sqrt(len / sqrt(a2));
    int k = 0;
    while (k < K && ldexp(dt_max, -k) > want) ++k;
    return k;
}

// s = 0: levels and opening kicks of every particle; s >= 1: closing (and new opening) kicks of the
// particles whose step ends at substep s.  ended[k] counts the closed steps of level k; ended[30]
// (set to ~0 before the launch) receives the earliest substep after s at which a step ends.  Both
// are gathered per block in shared memory first: one global atomic per level and block, not one
// per particle on the same word.
template <typename R>
__global__ void __launch_bounds__(TB) k_block_kick(int64_t n, R* __restrict__ vx, R* __restrict__ vy,
                                                    R* __restrict__ vz, const R* __restrict__ ax,
                                                    const R* __restrict__ ay, const R* __restrict__ az,
                                                    const uint32_t* __restrict__ id, uint8_t* __restrict__ level,
                                                    double dt_max, int K, int s, double eta, double len,
                                                    unsigned int* __restrict__ ended) {
    __shared__ unsigned int s_ended[32];
    __shared__ unsigned int s_next;
    if (threadIdx.x < 32) s_ended[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_next = ~0u;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    unsigned int next = ~0u;                           // substep at which this particle's step ends
    if (i < n) {
        const uint32_t p = id[i];
        const R a0 = ax[i], a1 = ay[i], a2 = az[i];
        R v0 = vx[i], v1 = vy[i], v2 = vz[i];
        bool opens = true;
        if (s > 0) {
            const int k = level[p];
            const int span = 1 << (K - k);
            if (s & (span - 1)) {                      // its step does not end at this substep
                next = (unsigned int)((s / span + 1) * span);
                opens = false;
            } else {
                const R h = (R)ldexp(dt_max, -(k + 1));
                v0 += h * a0; v1 += h * a1; v2 += h * a2;
                atomicAdd(&s_ended[k], 1u);
                if (s == (1 << K)) {                   // end of the base step: synchronous again
                    vx[i] = v0; vy[i] = v1; vz[i] = v2;
                    opens = false;
                }
            }
        }
        if (opens) {
            const double am2 = (double)a0 * (double)a0 + (double)a1 * (double)a1 + (double)a2 * (double)a2;
            int k = block_level(am2, eta, len, dt_max, K);
            if (s > 0) k = max(k, K - (__ffs(s) - 1));    // a new step must start on its own grid
            level[p] = (uint8_t)k;
            next = (unsigned int)(s + (1 << (K - k)));
            const R h = (R)ldexp(dt_max, -(k + 1));
            v0 += h * a0; v1 += h * a1; v2 += h * a2;
            vx[i] = v0; vy[i] = v1; vz[i] = v2;
        }
    }
    next = __reduce_min_sync(0xffffffffu, next);
    if ((threadIdx.x & 31) == 0 && next != ~0u) atomicMin(&s_next, next);
    __syncthreads();
    if (threadIdx.x <= (unsigned)K && s_ended[threadIdx.x]) atomicAdd(&ended[threadIdx.x], s_ended[threadIdx.x]);
    if (threadIdx.x == 0 && s_next != ~0u) atomicMin(&ended[30], s_next);
}

// per leaf (near-field order), one warp each: does one of its particles close its step at substep
// s?  32 particles' levels per load round; the active leaves are counted per block, then globally.
__global__ void __launch_bounds__(TB) k_block_active(int64_t nleaves, const uint32_t* __restrict__ leaves,
                                                      const NodeRec* __restrict__ nodes,
                                                      const uint32_t* __restrict__ id,
                                                      const uint8_t* __restrict__ level, int K, int s,
                                                      uint8_t* __restrict__ active, unsigned int* __restrict__ count) {
    __shared__ unsigned int s_count;
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    const int64_t li = (int64_t)blockIdx.x * (TB / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (li < nleaves) {                                // warp-uniform
        const NodeRec nd = nodes[leaves[li]];
        bool a = false;
        for (uint32_t b = 0; b < nd.count && !a; b += 32) {
            bool mine = false;
            if (b + lane < nd.count) {
                const int k = level[id[nd.begin + b + lane]];
                mine = (s & ((1 << (K - k)) - 1)) == 0;
            }
            a = __any_sync(0xffffffffu, mine);
        }
        if (lane == 0) {
            active[li] = a;
            if (a) atomicAdd(&s_count, 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_count) atomicAdd(count, s_count);
}

template <typename R>
int block_kick(nbody_ctx* c, int s) {
    const int k = c->cur;
    const double len = c->dt_len > 0.0 ? c->dt_len : c->prm.eps;
    NB_CU(c, cudaMemsetAsync(DP<unsigned int>(c->blk_count) + 30, 0xff, sizeof(unsigned int), c->st));
    k_block_kick<R><<<nblk(c->n), TB, 0, c->st>>>(c->n, DP<R>(c->vx[k]), DP<R>(c->vy[k]), DP<R>(c->vz[k]),
                                                  DP<R>(c->ax[k]), DP<R>(c->ay[k]), DP<R>(c->az[k]),
                                                  DP<uint32_t>(c->id[k]), DP<uint8_t>(c->blk_level), c->dt_max,
                                                  c->blk_K, s, c->dt_eta, len, DP<unsigned int>(c->blk_count));
    NB_LAUNCHED(c, "block kick");
    return NBODY_OK;
}

}  // namespace

int nb_block_active_leaves(nbody_ctx* c) {
    NB_TRY(nb_grow(c, c->blk_active, (size_t)c->nleaves + 1));
    const unsigned grid = (unsigned)((c->nleaves + TB / 32 - 1) / (TB / 32));     // a warp per leaf
    k_block_active<<<grid, TB, 0, c->st>>>(c->nleaves, DP<uint32_t>(c->leaves), DP<NodeRec>(c->nodes),
                                           DP<uint32_t>(c->id[c->cur]), DP<uint8_t>(c->blk_level), c->blk_K,
                                           c->blk_s, DP<uint8_t>(c->blk_active), DP<unsigned int>(c->blk_count) + 31);
    NB_LAUNCHED(c, "block active leaves");
    c->launches += 1;
    c->blk_leaves += c->nleaves;
    return NBODY_OK;
}

int nb_block_step(nbody_ctx* c) {
    NB_TRY(nb_grow(c, c->blk_level, (size_t)c->n));
    NB_TRY(nb_grow(c, c->blk_count, sizeof(unsigned int) * 32));
    NB_CU(c, cudaMemsetAsync(c->blk_count.p, 0, sizeof(unsigned int) * 32, c->st));
    if (!c->have_acc) {
        NB_TRY(nb_evaluate(c, 0, NB_INTEG_NONE, false));
        c->have_acc = true;
    }
    c->blk_dt = ldexp(c->dt_max, -c->blk_K);
    NB_TRY(c->rsz == 4 ? block_kick<float>(c, 0) : block_kick<double>(c, 0));
    const int S = 1 << c->blk_K;
    c->blk_leaves = 0;
    c->blk_evals = 0;
    int next = 0;
    for (int s = 1; s <= S; ++s) {
        if (s > next) {
            // the earliest substep at which a step ends, from the last kick (at most S: every step
            // ends by the end of the base step)
            NB_CU(c, cudaMemcpyAsync(&c->h_blk_count[30], DP<unsigned int>(c->blk_count) + 30,
                                     sizeof(unsigned int), cudaMemcpyDeviceToHost, c->st));
            NB_CU(c, cudaStreamSynchronize(c->st));
            next = (int)c->h_blk_count[30];
            if (next < s || next > S) return nb_fail(c, NBODY_ERR_STATE, "block step: bad next substep");
        }
        if (s < next) {
            NB_TRY(nb_drift(c, c->blk_dt));          // no particle's step ends here: drift only
            continue;
        }
        // drift of every particle + forces; near field and L2P only for leaves holding a particle whose
        // step ends at s (the others' accelerations are not used at this substep)
        c->blk_s = s;
        const int rc = nb_evaluate(c, 2, NB_INTEG_NONE, false);
        c->blk_s = 0;
        NB_TRY(rc);
        ++c->blk_evals;
        NB_TRY(c->rsz == 4 ? block_kick<float>(c, s) : block_kick<double>(c, s));
    }
    NB_CU(c, cudaMemcpyAsync(c->h_blk_count, c->blk_count.p, sizeof(unsigned int) * 32, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    c->blk_active_leaves = c->h_blk_count[31];
    return NBODY_OK;
}

extern "C" int nbody_get_levels(nbody_ctx* c, int32_t* levels) {
    if (!c || !levels) return NBODY_ERR_INVALID;
    if (c->dt_mode != NBODY_DT_BLOCK || c->blk_level.bytes < (size_t)c->n || c->n == 0)
        return nb_fail(c, NBODY_ERR_STATE, "no block step taken");
    NB_CU(c, cudaSetDevice(c->device));
    std::vector<uint8_t> lv((size_t)c->n);
    NB_CU(c, cudaMemcpyAsync(lv.data(), c->blk_level.p, (size_t)c->n, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    for (int64_t i = 0; i < c->n; ++i) levels[i] = lv[i];
    return NBODY_OK;
}
