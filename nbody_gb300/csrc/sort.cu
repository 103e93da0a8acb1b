// Device-wide exclusive scan (uint32) and stable LSD radix sort (uint64 keys,
// uint32 values).  Used for the Morton ordering of the particles, the
// breadth-first ordering of the octree nodes and every compaction of the step.
// Both are deterministic: no result depends on scheduling.
#include "nbody_internal.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

constexpr int RADIX_THREADS = 256;
constexpr int RADIX_ROUNDS = 16;
constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ROUNDS;

// exclusive block scan of one value per thread; returns the block total in *total
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t block_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint32_t inc = warp_incl_scan(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < nwarps ? warp_sums[lane] : 0u;
        uint32_t si = warp_incl_scan(s);
        if (lane < nwarps) warp_sums[lane] = si - s;
        if (lane == nwarps - 1) block_total = si;
    }
    __syncthreads();
    uint32_t r = warp_sums[warp] + inc - v;
    if (total) *total = block_total;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ in, int64_t n,
                                                                uint32_t* __restrict__ part) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_partials(uint32_t* part, int64_t nb, uint32_t* total) {
    uint32_t run = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
        int64_t i = b0 + threadIdx.x;
        uint32_t v = i < nb ? part[i] : 0u;
        uint32_t tot;
        uint32_t e = block_excl_scan(v, &tot);
        if (i < nb) part[i] = run + e;
        run += tot;
    }
    if (threadIdx.x == 0 && total) *total = run;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                              int64_t n, const uint32_t* __restrict__ part) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = base + k < n ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t e = block_excl_scan(s, nullptr) + part[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < n) out[base + k] = e;
        e += v[k];
    }
}

// the same three phases over K arrays at once (one launch per phase for all of them)
struct ScanK {
    const uint32_t* in[3];         // null: array unused
    uint32_t* out[3];
    uint32_t* total[3];
    const uint32_t* n_dev;         // non-null: scan only the first *n_dev entries (<= n)
};

__device__ __forceinline__ int64_t scan_len(const ScanK& A, int64_t n) {
    if (!A.n_dev) return n;
    const int64_t m = (int64_t)*A.n_dev;
    return m < n ? m : n;
}

template <int K>
__global__ void __launch_bounds__(SCAN_THREADS) k_scank_reduce(ScanK A, int64_t n, uint32_t* __restrict__ part,
                                                                 int64_t nb) {
    n = scan_len(A, n);
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    if ((int64_t)blockIdx.x * SCAN_TILE >= n) {
        if (threadIdx.x < K) part[threadIdx.x * nb + blockIdx.x] = 0;
        return;
    }
#pragma unroll
    for (int a = 0; a < K; ++a) {
        if (!A.in[a]) continue;
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k)
            if (base + k < n) s += A.in[a][base + k];
        uint32_t tot;
        block_excl_scan(s, &tot);
        if (threadIdx.x == 0) part[a * nb + blockIdx.x] = tot;
    }
}

template <int K>
__global__ void __launch_bounds__(1024) k_scank_partials(ScanK A, uint32_t* part, int64_t nb) {
#pragma unroll
    for (int a = 0; a < K; ++a) {
        if (!A.in[a]) continue;
        uint32_t run = 0;
        for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
            const int64_t i = b0 + threadIdx.x;
            const uint32_t v = i < nb ? part[a * nb + i] : 0u;
            uint32_t tot;
            const uint32_t e = block_excl_scan(v, &tot);
            if (i < nb) part[a * nb + i] = run + e;
            run += tot;
        }
        if (threadIdx.x == 0 && A.total[a]) *A.total[a] = run;
    }
}

template <int K>
__global__ void __launch_bounds__(SCAN_THREADS) k_scank_down(ScanK A, int64_t n, const uint32_t* __restrict__ part,
                                                               int64_t nb) {
    n = scan_len(A, n);
    if ((int64_t)blockIdx.x * SCAN_TILE >= n) return;
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
#pragma unroll
    for (int a = 0; a < K; ++a) {
        if (!A.in[a]) continue;
        uint32_t v[SCAN_ITEMS];
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            v[k] = base + k < n ? A.in[a][base + k] : 0u;
            s += v[k];
        }
        uint32_t e = block_excl_scan(s, nullptr) + part[a * nb + blockIdx.x];
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            if (base + k < n) A.out[a][base + k] = e;
            e += v[k];
        }
    }
}

__global__ void __launch_bounds__(RADIX_THREADS) k_radix_hist(const uint64_t* __restrict__ keys, int64_t n, int shift,
                                                                uint32_t mask, uint32_t* __restrict__ hist, int nblocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        int64_t i = base + r * RADIX_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(RADIX_THREADS) k_radix_scatter(const uint64_t* __restrict__ kin,
                                                                   const uint32_t* __restrict__ vin,
                                                                   uint64_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                                   int64_t n, int shift, uint32_t mask,
                                                                   const uint32_t* __restrict__ offs, int nblocks) {
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_run[256];
    __shared__ uint32_t s_w[RADIX_THREADS / 32][256];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    s_base[tid] = offs[(int64_t)tid * nblocks + blockIdx.x];
    s_run[tid] = 0;
    int64_t base = (int64_t)blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        if (base + r * RADIX_THREADS >= n) break;
#pragma unroll
        for (int w = 0; w < RADIX_THREADS / 32; ++w) s_w[w][tid] = 0;
        __syncthreads();
        int64_t i = base + r * RADIX_THREADS + tid;
        bool valid = i < n;
        uint64_t key = valid ? kin[i] : 0ull;
        uint32_t digit = valid ? ((uint32_t)(key >> shift) & mask) : 0x10000u;
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) s_w[warp][digit] = __popc(peers);
        __syncthreads();
        {
            uint32_t acc = s_run[tid];
#pragma unroll
            for (int w = 0; w < RADIX_THREADS / 32; ++w) {
                uint32_t cnt = s_w[w][tid];
                s_w[w][tid] = acc;
                acc += cnt;
            }
            s_run[tid] = acc;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = s_base[digit] + s_w[warp][digit] + rank;
            kout[pos] = key;
            vout[pos] = vin[i];
        }
        __syncthreads();
    }
}

}  // namespace

int nb_scan_u32(nbody_ctx* c, const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev) {
    if (n <= 0) {
        if (total_dev) NB_CU(c, cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), c->st));
        return NBODY_OK;
    }
    int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    NB_TRY(nb_grow(c, c->scan_part, sizeof(uint32_t) * (size_t)(nb + 1)));
    uint32_t* part = DP<uint32_t>(c->scan_part);
    k_scan_reduce<<<(unsigned)nb, SCAN_THREADS, 0, c->st>>>(in, n, part);
    k_scan_partials<<<1, 1024, 0, c->st>>>(part, nb, total_dev);
    k_scan_down<<<(unsigned)nb, SCAN_THREADS, 0, c->st>>>(in, out, n, part);
    NB_LAUNCHED(c, "scan");
    c->launches += 3;
    return NBODY_OK;
}

int nb_scan3_u32(nbody_ctx* c, const uint32_t* const in[3], uint32_t* const out[3], int64_t n,
                 uint32_t* const total_dev[3], const uint32_t* n_dev) {
    if (n <= 0) {
        for (int a = 0; a < 3; ++a)
            if (total_dev[a]) NB_CU(c, cudaMemsetAsync(total_dev[a], 0, sizeof(uint32_t), c->st));
        return NBODY_OK;
    }
    const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    NB_TRY(nb_grow(c, c->scan_part, sizeof(uint32_t) * (size_t)(3 * nb + 1)));
    uint32_t* part = DP<uint32_t>(c->scan_part);
    ScanK A;
    for (int a = 0; a < 3; ++a) { A.in[a] = in[a]; A.out[a] = out[a]; A.total[a] = total_dev[a]; }
    A.n_dev = n_dev;
    k_scank_reduce<3><<<(unsigned)nb, SCAN_THREADS, 0, c->st>>>(A, n, part, nb);
    k_scank_partials<3><<<1, 1024, 0, c->st>>>(A, part, nb);
    k_scank_down<3><<<(unsigned)nb, SCAN_THREADS, 0, c->st>>>(A, n, part, nb);
    NB_LAUNCHED(c, "scan3");
    c->launches += 3;
    return NBODY_OK;
}

int nb_radix_sort(nbody_ctx* c, int64_t n, uint64_t* k0, uint32_t* v0, uint64_t* k1, uint32_t* v1, int begin_bit,
                  int end_bit, int* result_in_first) {
    *result_in_first = 1;
    if (n <= 1) return NBODY_OK;
    int nblocks = (int)((n + RADIX_TILE - 1) / RADIX_TILE);
    size_t hbytes = sizeof(uint32_t) * (size_t)256 * nblocks;
    NB_TRY(nb_grow(c, c->hist, hbytes));
    NB_TRY(nb_grow(c, c->hist_scan, hbytes));
    uint64_t *ki = k0, *ko = k1;
    uint32_t *vi = v0, *vo = v1;
    for (int sh = begin_bit; sh < end_bit; sh += 8) {
        int bits = end_bit - sh < 8 ? end_bit - sh : 8;
        uint32_t mask = (1u << bits) - 1u;
        k_radix_hist<<<nblocks, RADIX_THREADS, 0, c->st>>>(ki, n, sh, mask, DP<uint32_t>(c->hist), nblocks);
        NB_LAUNCHED(c, "radix_hist");
        NB_TRY(nb_scan_u32(c, DP<uint32_t>(c->hist), DP<uint32_t>(c->hist_scan), (int64_t)256 * nblocks, nullptr));
        k_radix_scatter<<<nblocks, RADIX_THREADS, 0, c->st>>>(ki, vi, ko, vo, n, sh, mask, DP<uint32_t>(c->hist_scan),
                                                               nblocks);
        NB_LAUNCHED(c, "radix_scatter");
        c->launches += 2;
        uint64_t* tk = ki; ki = ko; ko = tk;
        uint32_t* tv = vi; vi = vo; vo = tv;
        *result_in_first = !*result_in_first;
    }
    return NBODY_OK;
}
