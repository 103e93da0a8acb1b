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
constexpr int RADIX_ROUNDS = 4;           // 1,024-key tiles: enough blocks to fill the GPU at 262k keys
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

// Single-pass exclusive scan over up to three arrays (decoupled look-back).  Each block takes
// its tile from a ticket counter, so every tile it waits on belongs to a block that is already
// running (the block that draws the last ticket puts the counter back to zero for the next
// launch); it publishes its tile's sum, then walks back over the status words of the tiles
// before it (one warp per array, 32 tiles per step) until it meets an inclusive prefix.  A
// status word packs the call's epoch, a flag (1: tile sum, 2: inclusive prefix) and the value
// in one 64-bit store, so words left by earlier calls never match and no reset is needed.  The
// sums are integer, so the result does not depend on which words a block happened to see.
constexpr uint32_t SCAN_EPOCH_SHIFT = 34;
constexpr uint64_t SCAN_FLAG_SUM = 1ull << 32, SCAN_FLAG_INCL = 2ull << 32;

struct ScanK {
    const uint32_t* in[3];         // null: array unused
    uint32_t* out[3];
    uint32_t* total[3];
    const uint32_t* n_dev;         // non-null: scan only the first *n_dev entries (<= n)
    unsigned long long* state;     // [0] ticket counter, [1 + a * nb + t] status of tile t of array a
    int64_t nb;                    // blocks of this launch (tiles of n entries)
    uint64_t epoch;
    int32_t* info;                 // INFO_SCAN_ERR is raised when a look-back gives up
    int64_t spin_limit;            // polls of one status word before giving up
};

__device__ __forceinline__ int64_t scan_len(const ScanK& A, int64_t n) {
    if (!A.n_dev) return n;
    const int64_t m = (int64_t)*A.n_dev;
    return m < n ? m : n;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// one warp: publishes tile t's sum `agg`, returns the sum of all tiles before t (every lane)
__device__ uint32_t scan_lookback(unsigned long long* st, int64_t t, uint32_t agg, uint64_t epoch, int32_t* info,
                                  int64_t spin_limit) {
    const int lane = lane_id();
    const unsigned long long tag = epoch << SCAN_EPOCH_SHIFT;
    if (t == 0) {
        if (lane == 0) st_relaxed_u64(st, tag | SCAN_FLAG_INCL | agg);
        return 0;
    }
    if (lane == 0) st_relaxed_u64(st + t, tag | SCAN_FLAG_SUM | agg);
    uint32_t prefix = 0;
    bool gave_up = false;
    for (int64_t j = t - 1;; j -= 32) {
        const int64_t my = j - lane;
        // positions before tile 0 read as an inclusive zero; tile 0 itself is always inclusive
        uint64_t flag = SCAN_FLAG_INCL;
        uint32_t val = 0;
        if (my >= 0) {
            unsigned long long w = ld_relaxed_u64(st + my);
            int64_t spins = 0;
            while ((w >> SCAN_EPOCH_SHIFT) != epoch && ++spins < spin_limit) {
                __nanosleep(64);
                w = ld_relaxed_u64(st + my);
            }
            if ((w >> SCAN_EPOCH_SHIFT) == epoch) {
                flag = w & (3ull << 32);
                val = (uint32_t)w;
            } else {
                gave_up = true;
            }
        }
        const unsigned incl = __ballot_sync(0xffffffffu, flag == SCAN_FLAG_INCL);
        const int stop = incl ? __ffs(incl) - 1 : 31;
        uint32_t s = lane <= stop ? val : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        prefix += s;
        if (incl) break;
    }
    if (__any_sync(0xffffffffu, gave_up) && lane == 0) atomicOr((unsigned int*)&info[INFO_SCAN_ERR], 1u);
    if (lane == 0) st_relaxed_u64(st + t, tag | SCAN_FLAG_INCL | (uint32_t)(prefix + agg));
    return prefix;
}

template <int K>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan(ScanK A, int64_t n) {
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_prefix[K];
    n = scan_len(A, n);
    const int64_t last = n > 0 ? (n - 1) / SCAN_TILE : 0;     // the tile that writes the totals
    if ((int64_t)blockIdx.x > last) return;                    // only last + 1 blocks draw tickets
    if (threadIdx.x == 0) {
        const unsigned long long tk = atomicAdd(A.state, 1ull);
        if (tk == (unsigned long long)last) atomicExch(A.state, 0ull);
        if (tk > (unsigned long long)last) atomicOr((unsigned int*)&A.info[INFO_SCAN_ERR], 2u);
        s_tile = tk > (unsigned long long)last ? 0xffffffffu : (uint32_t)tk;
    }
    __syncthreads();
    if (s_tile == 0xffffffffu) return;                         // counter left over by a failed launch
    const int64_t t = s_tile;
    const int64_t base = t * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    uint32_t v[K][SCAN_ITEMS], ex[K], agg[K];
#pragma unroll
    for (int a = 0; a < K; ++a) {
        ex[a] = agg[a] = 0;
        if (!A.in[a]) continue;
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            v[a][k] = base + k < n ? A.in[a][base + k] : 0u;
            s += v[a][k];
        }
        ex[a] = block_excl_scan(s, &agg[a]);
    }
    const int warp = threadIdx.x >> 5;
#pragma unroll
    for (int a = 0; a < K; ++a)
        if (warp == a && A.in[a]) {
            const uint32_t pre = scan_lookback(A.state + 1 + a * A.nb, t, agg[a], A.epoch, A.info, A.spin_limit);
            if (lane_id() == 0) s_prefix[a] = pre;
        }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < K; ++a) {
        if (!A.in[a]) continue;
        uint32_t e = s_prefix[a] + ex[a];
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            if (base + k < n) A.out[a][base + k] = e;
            e += v[a][k];
        }
        if (t == last && threadIdx.x == 0 && A.total[a]) *A.total[a] = s_prefix[a] + agg[a];
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
            uint32_t pos = NB_IDX(s_base[digit] + s_w[warp][digit] + rank, n, NB_SITE_SORT);
            kout[pos] = key;
            vout[pos] = vin[i];
        }
        __syncthreads();
    }
}

// the look-back's wait on a status word that nothing publishes (word 0 of `st` holds epoch 0, which
// no scan uses): tile 1 polls it until the limit runs out and raises INFO_SCAN_ERR
__global__ void k_scan_wait_selftest(unsigned long long* st, int32_t* info, int64_t spin_limit) {
    scan_lookback(st, 1, 1u, 1u, info, spin_limit);
}

}  // namespace

namespace {

// launches the single-pass scan over the arrays of `in` (null entries skipped)
template <int K>
int scan_launch(nbody_ctx* c, const uint32_t* const* in, uint32_t* const* out, int64_t n, uint32_t* const* total,
                const uint32_t* n_dev) {
    const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    const size_t bytes = sizeof(unsigned long long) * (size_t)(1 + K * nb);
    if (c->scan_part.bytes < bytes) {
        NB_TRY(nb_grow(c, c->scan_part, bytes));
        NB_CU(c, cudaMemsetAsync(c->scan_part.p, 0, c->scan_part.bytes, c->st));
    }
    ScanK A;
    for (int a = 0; a < 3; ++a) {
        A.in[a] = a < K ? in[a] : nullptr;
        A.out[a] = a < K ? out[a] : nullptr;
        A.total[a] = a < K ? total[a] : nullptr;
    }
    A.n_dev = n_dev;
    A.state = DP<unsigned long long>(c->scan_part);
    A.nb = nb;
    c->scan_epoch = c->scan_epoch % ((1ull << 30) - 1) + 1;     // 1 .. 2^30 - 1; 0 marks a cleared word
    A.epoch = c->scan_epoch;
    A.info = DP<int32_t>(c->info);
    A.spin_limit = c->scan_polls;
    k_scan<K><<<(unsigned)nb, SCAN_THREADS, 0, c->st>>>(A, n);
    NB_LAUNCHED(c, "scan");
    c->launches += 1;
    return NBODY_OK;
}

}  // namespace

int nb_scan_u32(nbody_ctx* c, const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev) {
    if (n <= 0) {
        if (total_dev) NB_CU(c, cudaMemsetAsync(total_dev, 0, sizeof(uint32_t), c->st));
        return NBODY_OK;
    }
    return scan_launch<1>(c, &in, &out, n, &total_dev, nullptr);
}

int nb_scan3_u32(nbody_ctx* c, const uint32_t* const in[3], uint32_t* const out[3], int64_t n,
                 uint32_t* const total_dev[3], const uint32_t* n_dev) {
    if (n <= 0) {
        for (int a = 0; a < 3; ++a)
            if (total_dev[a]) NB_CU(c, cudaMemsetAsync(total_dev[a], 0, sizeof(uint32_t), c->st));
        return NBODY_OK;
    }
    if (!in[2]) return scan_launch<2>(c, in, out, n, total_dev, n_dev);
    return scan_launch<3>(c, in, out, n, total_dev, n_dev);
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

int nb_scan_wait_selftest(nbody_ctx* c) {
    NB_TRY(nb_grow(c, c->wait_probe, 2 * sizeof(unsigned long long)));
    NB_CU(c, cudaMemsetAsync(c->wait_probe.p, 0, 2 * sizeof(unsigned long long), c->st));
    k_scan_wait_selftest<<<1, 32, 0, c->st>>>(DP<unsigned long long>(c->wait_probe), DP<int32_t>(c->info),
                                              c->scan_polls);
    NB_LAUNCHED(c, "scan wait self-test");
    NB_CU(c, cudaMemcpyAsync(c->h_info, c->info.p, sizeof(int32_t) * INFO_WORDS, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    if (c->h_info[INFO_SCAN_ERR]) return nb_fail(c, NBODY_ERR_CUDA, "a device scan did not complete in time");
    return NBODY_OK;
}

NB_DBG_ACCESSOR(sort)
