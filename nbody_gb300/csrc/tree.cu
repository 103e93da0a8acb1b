// Morton keys, re-sort and octree construction on the device.
//
// The reference rebuilds a host octree every step through an external
// library and uploads it (src/open_cl_simulation.cpp:43-47,120-135).  Here
// the tree is built from scratch on the GPU each step, in a fixed number of
// launches independent of the depth:
//   1. opening kick + drift of the previous step's state, root box;
//   2. 63-bit Morton keys (21 bits per axis) and a stable radix sort;
//   3. the leaf level of every particle, from a sliding window over the
//      sorted keys: the cell of level l around particle i holds more than C
//      particles iff some window [a, a+C] containing i has keys that agree
//      on their first l octal digits, so
//        leaf_level(i) = 1 + max_{a in [i-C, i]} cpl(key[a], key[a+C]);
//   4. the nodes starting at position i are the chain of cells of levels
//      cpl(key[i-1], key[i]) + 1 .. leaf_level(i); their counts are scanned
//      (depth-first pre-order) and the chains emitted;
//   5. a stable one-digit radix pass on the level gives breadth-first order
//      (Morton order within a level, children contiguous);
//   6. each node finds its particle count, parent and children by binary
//      search, and links itself (bottom-up: every node links to the level
//      above and below without any per-level launch).
#include "nbody_internal.cuh"

namespace {

constexpr int TB = 256;

template <typename R>
struct StatePtrs {
    R *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *m, *q;
    uint32_t* id;
};

template <typename R>
StatePtrs<R> state(nbody_ctx* c, int k) {
    return StatePtrs<R>{DP<R>(c->x[k]),  DP<R>(c->y[k]),  DP<R>(c->z[k]),  DP<R>(c->vx[k]),
                        DP<R>(c->vy[k]), DP<R>(c->vz[k]), DP<R>(c->ax[k]), DP<R>(c->ay[k]),
                        DP<R>(c->az[k]), DP<R>(c->m[k]),  DP<R>(c->q[k]),  DP<uint32_t>(c->id[k])};
}

__device__ __forceinline__ unsigned long long ord_key(double v) {
    long long b = __double_as_longlong(v);
    return b >= 0 ? ((unsigned long long)b ^ 0x8000000000000000ull) : ~(unsigned long long)b;
}
__device__ __forceinline__ double ord_val(unsigned long long k) {
    long long b = (k & 0x8000000000000000ull) ? (long long)(k ^ 0x8000000000000000ull) : (long long)(~k);
    return __longlong_as_double(b);
}

// opening kick + drift (leapfrog) and the bounding box of the new positions.  The box is reduced on
// order-preserving integer keys of the finite coordinates (integer min/max instead of the FP64 pipe);
// a non-finite coordinate raises NB_ERRBIT_NONFINITE and stays out of the bounds.
template <typename R>
__global__ void __launch_bounds__(TB) k_kick_drift_bbox(int64_t n, StatePtrs<R> s, double hdt, double dt, int kdk,
                                                         unsigned long long* bbox, int32_t* info) {
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0ull, 0ull, 0ull};
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x; i < n; i += (int64_t)gridDim.x * TB) {
        R x = s.x[i], y = s.y[i], z = s.z[i];
        if (kdk == 1) {
            R vx = s.vx[i] + (R)hdt * s.ax[i], vy = s.vy[i] + (R)hdt * s.ay[i], vz = s.vz[i] + (R)hdt * s.az[i];
            x += (R)dt * vx; y += (R)dt * vy; z += (R)dt * vz;
            s.vx[i] = vx; s.vy[i] = vy; s.vz[i] = vz;
            s.x[i] = x; s.y[i] = y; s.z[i] = z;
        } else if (kdk == 2) {             // drift only (block steps: the kicks are per particle)
            x += (R)dt * s.vx[i]; y += (R)dt * s.vy[i]; z += (R)dt * s.vz[i];
            s.x[i] = x; s.y[i] = y; s.z[i] = z;
        }
        const double p[3] = {(double)x, (double)y, (double)z};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const unsigned long long bits = (unsigned long long)__double_as_longlong(p[d]);
            const bool nonfinite = (bits & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
            bad |= nonfinite;
            if (nonfinite) continue;          // the bounds cover the finite coordinates only
            const unsigned long long k = ord_key(p[d]);
            mn[d] = k < mn[d] ? k : mn[d];
            mx[d] = k > mx[d] ? k : mx[d];
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long a = __shfl_xor_sync(0xffffffffu, mn[d], o);
            const unsigned long long b = __shfl_xor_sync(0xffffffffu, mx[d], o);
            mn[d] = a < mn[d] ? a : mn[d];
            mx[d] = b > mx[d] ? b : mx[d];
        }
    // block reduction, then one atomic per bound per block (per-warp atomics on six words serialise)
    __shared__ unsigned long long s_mn[TB / 32][3], s_mx[TB / 32][3];
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int d = 0; d < 3; ++d) { s_mn[warp][d] = mn[d]; s_mx[warp][d] = mx[d]; }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        unsigned long long a = s_mn[0][d], b = s_mx[0][d];
        for (int w = 1; w < TB / 32; ++w) {
            a = s_mn[w][d] < a ? s_mn[w][d] : a;
            b = s_mx[w][d] > b ? s_mx[w][d] : b;
        }
        atomicMin(&bbox[d], a);
        atomicMax(&bbox[3 + d], b);
    }
    if (bad) atomicOr((unsigned int*)&info[INFO_ERR], NB_ERRBIT_NONFINITE);
}

// Root box of a fixed-box run that a particle has left (escape policy NBODY_ESCAPE_GROW): the
// smallest box of side fside * 2^j whose cells of level j include the fixed box itself, with origin
// f - a * fside per axis (a >= 0 integer), that covers [lo, hi].  Inside the fixed box the cells
// below level j are the fixed box's own cells, so particles there are binned as before (the keys
// lose their j lowest levels).  false if no such box is representable.
__device__ bool grown_box(const double* lo, const double* hi, const double* f, double fside, double* o,
                          double* side) {
    double a[3];
    for (int d = 0; d < 3; ++d) {
        a[d] = lo[d] < f[d] ? ceil((f[d] - lo[d]) / fside) : 0.0;
        // rounding of the quotient: step until the origin is at or below the lowest coordinate
        for (int it = 0; it < 4 && f[d] - a[d] * fside > lo[d]; ++it) a[d] += 1.0;
        o[d] = f[d] - a[d] * fside;
        if (!(o[d] <= lo[d])) return false;
    }
    double s = fside;
    for (int j = 0; j <= 1100 && isfinite(s); ++j) {
        bool ok = true;
        for (int d = 0; d < 3; ++d) ok = ok && (a[d] * fside < s) && (o[d] + s > hi[d]);
        if (ok) {
            *side = s;
            return true;
        }
        s *= 2.0;
    }
    return false;
}

// root box: fixed (the reference's [0, bounds)) or the power-of-two data cube.  A particle outside
// a fixed box raises NB_ERRBIT_ESCAPE; with grow = 1 the step takes grown_box instead, with
// grow = 0 the box stays (the host then fails the step with NBODY_ERR_RANGE).
__global__ void k_box(const unsigned long long* bbox, int fixed, int grow, double fx, double fy, double fz,
                      double fside, BoxDev* box, int32_t* info) {
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = ord_val(bbox[d]);
        hi[d] = ord_val(bbox[3 + d]);
    }
    BoxDev b;
    // no finite coordinate on some axis (every particle non-finite, already flagged): a unit box
    // keeps the rest of the step well defined until the host reports the error
    const bool finite = isfinite(lo[0]) && isfinite(lo[1]) && isfinite(lo[2]) && isfinite(hi[0]) &&
                        isfinite(hi[1]) && isfinite(hi[2]) && lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2];
    if (!finite) {
        atomicOr((unsigned int*)&info[INFO_ERR], NB_ERRBIT_NONFINITE);
        b.ox = 0.0; b.oy = 0.0; b.oz = 0.0; b.side = 1.0;
    } else if (fixed) {
        b.ox = fx; b.oy = fy; b.oz = fz; b.side = fside;
        if (lo[0] < fx || lo[1] < fy || lo[2] < fz || hi[0] >= fx + fside || hi[1] >= fy + fside ||
            hi[2] >= fz + fside) {
            atomicOr((unsigned int*)&info[INFO_ERR], NB_ERRBIT_ESCAPE);
            const double f[3] = {fx, fy, fz};
            double o[3], side;
            if (grow && grown_box(lo, hi, f, fside, o, &side)) {
                b.ox = o[0]; b.oy = o[1]; b.oz = o[2]; b.side = side;
            } else if (grow) {
                atomicOr((unsigned int*)&info[INFO_ERR], NB_ERRBIT_RANGE);
            }
        }
    } else {
        double ext = fmax(fmax(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]) * (1.0 + 0x1p-20);
        double side = 1.0;
        while (side < ext) side *= 2.0;
        while (side * 0.5 >= ext && ext > 0) side *= 0.5;
        double o[3] = {0.0, 0.0, 0.0};
        // finite bounds fit after a few doublings; the limit (the whole double range) only guards
        // the loop against a box that cannot be represented
        bool ok = false;
        for (int it = 0; it < 2200 && !ok && isfinite(side); ++it) {
            double half = side * 0.5;
            ok = true;
            for (int d = 0; d < 3; ++d) {
                o[d] = floor(lo[d] / half) * half;
                ok = ok && (o[d] + side > hi[d]);
            }
            if (!ok) side *= 2.0;
        }
        if (!ok) {
            atomicOr((unsigned int*)&info[INFO_ERR], NB_ERRBIT_RANGE);
            o[0] = o[1] = o[2] = 0.0;
            side = 1.0;
        }
        b.ox = o[0]; b.oy = o[1]; b.oz = o[2]; b.side = side;
    }
    b.scale = 2097152.0 / b.side;
    b.unit = b.side / 4194304.0;
    *box = b;
}

__device__ __forceinline__ uint32_t quantize(double x, double o, double scale) {
    double qv = (x - o) * scale;
    if (!(qv >= 0.0)) return 0u;
    if (qv >= 2097151.0) return 2097151u;
    return (uint32_t)qv;
}

template <typename R>
__global__ void __launch_bounds__(TB) k_keys(int64_t n, const R* __restrict__ x, const R* __restrict__ y,
                                              const R* __restrict__ z, const BoxDev* __restrict__ box,
                                              uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    BoxDev b = *box;
    uint32_t ix = quantize((double)x[i], b.ox, b.scale), iy = quantize((double)y[i], b.oy, b.scale),
             iz = quantize((double)z[i], b.oz, b.scale);
    keys[i] = nb_spread3(ix) | (nb_spread3(iy) << 1) | (nb_spread3(iz) << 2);
    vals[i] = (uint32_t)i;
}

template <typename R>
__global__ void __launch_bounds__(TB) k_gather(int64_t n, const uint32_t* __restrict__ perm, StatePtrs<R> a,
                                                StatePtrs<R> b) {
    int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    uint32_t j = NB_IDX(perm[i], n, NB_SITE_GATHER);
    b.x[i] = a.x[j]; b.y[i] = a.y[j]; b.z[i] = a.z[j];
    b.vx[i] = a.vx[j]; b.vy[i] = a.vy[j]; b.vz[i] = a.vz[j];
    b.ax[i] = a.ax[j]; b.ay[i] = a.ay[j]; b.az[i] = a.az[j];
    b.m[i] = a.m[j]; b.q[i] = a.q[j]; b.id[i] = a.id[j];
}

// common prefix of two keys in octal digits (0..21)
__device__ __forceinline__ int cpl_digits(uint64_t a, uint64_t b) {
    if (a == b) return NB_LEVELS;
    return (__clzll((long long)(a ^ b)) - 1) / 3;
}

__global__ void __launch_bounds__(TB) k_tree_cpl(int64_t n, int C, const uint64_t* __restrict__ keys,
                                                  int32_t* __restrict__ cpl, int32_t* __restrict__ wnd) {
    int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    uint64_t k = keys[i];
    cpl[i] = i == 0 ? -1 : cpl_digits(keys[i - 1], k);
    if (i + C < n) wnd[i] = cpl_digits(k, keys[i + C]);
}

__global__ void __launch_bounds__(TB) k_tree_chain(int64_t n, int C, int maxlevel, const int32_t* __restrict__ cpl,
                                                    const int32_t* __restrict__ wnd, uint32_t* __restrict__ nc,
                                                    int32_t* info) {
    __shared__ int hist[NB_LEVELS + 1];
    __shared__ int sdepth, sleaves;
    if (threadIdx.x <= NB_LEVELS) hist[threadIdx.x] = 0;
    if (threadIdx.x == 0) { sdepth = 0; sleaves = 0; }
    __syncthreads();
    int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i < n) {
        int64_t lo = i - C > 0 ? i - C : 0;
        int64_t hi = i < n - 1 - C ? i : n - 1 - C;
        int mx = -1;
        for (int64_t a = lo; a <= hi; ++a) mx = max(mx, wnd[a]);
        int L = min(maxlevel, mx + 1);
        int c0 = cpl[i];
        uint32_t cnt = L > c0 ? (uint32_t)(L - c0) : 0u;
        nc[i] = cnt;
        for (int l = c0 + 1; l <= L; ++l) atomicAdd(&hist[l], 1);
        if (cnt) {
            atomicMax(&sdepth, L);
            atomicAdd(&sleaves, 1);
        }
    }
    __syncthreads();
    if (threadIdx.x <= NB_LEVELS && hist[threadIdx.x]) atomicAdd(&info[INFO_HIST + threadIdx.x], hist[threadIdx.x]);
    if (threadIdx.x == 0) {
        atomicMax(&info[INFO_DEPTH], sdepth);
        atomicAdd(&info[INFO_NLEAVES], sleaves);
    }
}

__global__ void __launch_bounds__(TB) k_tree_seeds(int64_t n, const int32_t* __restrict__ cpl,
                                                    const uint32_t* __restrict__ nc, const uint32_t* __restrict__ pfx,
                                                    uint64_t* __restrict__ sk, uint32_t* __restrict__ sv) {
    int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    uint32_t cnt = nc[i], o = pfx[i];
    int l0 = cpl[i] + 1;
    for (uint32_t j = 0; j < cnt; ++j) {
        sk[o + j] = (uint64_t)(l0 + (int)j);
        sv[o + j] = (uint32_t)i;
    }
}

struct LevelStarts {
    int s[NB_LEVELS + 3];
};

__device__ __forceinline__ int64_t lower_bound_u32(const uint32_t* a, int64_t lo, int64_t hi, uint32_t v) {
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ int64_t lower_bound_u64(const uint64_t* a, int64_t lo, int64_t hi, uint64_t v) {
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(TB) k_tree_nodes(int64_t nnodes, int64_t n, int depth,
                                                    const uint64_t* __restrict__ keys, const uint64_t* __restrict__ sk,
                                                    const uint32_t* __restrict__ sv, LevelStarts ls,
                                                    NodeRec* __restrict__ nodes, uint32_t* __restrict__ leafflag) {
    int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (k >= nnodes) return;
    int l = (int)sk[k];
    uint32_t b = NB_IDX(sv[k], n, NB_SITE_TREE);
    NodeRec nd;
    nd.level = (uint8_t)l;
    nd.begin = b;
    nd.pad = 0;
    nd.child_mask = 0;
    if (l == 0) {
        nd.count = (uint32_t)n;
        nd.ix = nd.iy = nd.iz = 0;
        nd.parent = -1;
    } else {
        int sh = 3 * (NB_LEVELS - l);
        uint64_t pre = keys[b] >> sh;
        int64_t e = lower_bound_u64(keys, (int64_t)b + 1, n, (pre + 1) << sh);
        nd.count = (uint32_t)(e - b);
        nd.ix = nb_compact3(pre);
        nd.iy = nb_compact3(pre >> 1);
        nd.iz = nb_compact3(pre >> 2);
        // parent: last node of level l-1 whose range starts at or before b
        int64_t j = lower_bound_u32(sv, ls.s[l - 1], ls.s[l], b + 1) - 1;
        nd.parent = (int32_t)j;
    }
    nd.child_begin = -1;
    nd.nchild = 0;
    if (l < depth) {
        int64_t lo = lower_bound_u32(sv, ls.s[l + 1], ls.s[l + 2], b);
        int64_t hi = lower_bound_u32(sv, lo, ls.s[l + 2], b + nd.count);
        if (hi > lo) {
            nd.child_begin = (int32_t)lo;
            nd.nchild = (uint8_t)(hi - lo);
            const int csh = 3 * (NB_LEVELS - l - 1);
            uint32_t mask = 0;
            for (int64_t c = lo; c < hi; ++c) mask |= 1u << ((keys[sv[c]] >> csh) & 7u);
            nd.child_mask = (uint8_t)mask;
        }
    }
    nodes[k] = nd;
    leafflag[k] = nd.nchild == 0 ? 1u : 0u;
}

__global__ void __launch_bounds__(TB) k_tree_leaves(int64_t nnodes, const uint32_t* __restrict__ flag,
                                                     const uint32_t* __restrict__ pfx, uint32_t* __restrict__ leaves) {
    int64_t k = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (k >= nnodes) return;
    if (flag[k]) leaves[pfx[k]] = (uint32_t)k;
}

inline unsigned nblk(int64_t n) { return (unsigned)((n + TB - 1) / TB); }

template <typename R>
int begin_step_t(nbody_ctx* c, int kdk) {
    const int64_t n = c->n;
    unsigned long long* bb = DP<unsigned long long>(c->bbox);
    NB_CU(c, cudaMemsetAsync(c->info.p, 0, sizeof(int32_t), c->st));   // INFO_ERR
    NB_CU(c, cudaMemsetAsync(bb, 0xff, 3 * sizeof(unsigned long long), c->st));
    NB_CU(c, cudaMemsetAsync(bb + 3, 0x00, 3 * sizeof(unsigned long long), c->st));
    unsigned g = nblk(n);
    if (g > 152 * 8) g = 152 * 8;
    if (g == 0) g = 1;
    const double dt = kdk == 2 ? c->blk_dt : c->prm.dt;
    k_kick_drift_bbox<R><<<g, TB, 0, c->st>>>(n, state<R>(c, c->cur), 0.5 * dt, dt, kdk, bb,
                                              DP<int32_t>(c->info));
    k_box<<<1, 1, 0, c->st>>>(bb, c->prm.fixed_box, c->escape_policy == NBODY_ESCAPE_GROW, c->prm.box_min[0],
                              c->prm.box_min[1], c->prm.box_min[2], c->prm.box_size, DP<BoxDev>(c->box),
                              DP<int32_t>(c->info));
    k_keys<R><<<nblk(n), TB, 0, c->st>>>(n, DP<R>(c->x[c->cur]), DP<R>(c->y[c->cur]), DP<R>(c->z[c->cur]),
                                         DP<BoxDev>(c->box), DP<uint64_t>(c->keys[0]), DP<uint32_t>(c->vals[0]));
    NB_LAUNCHED(c, "kick_drift_keys");
    c->launches += 3;
    return NBODY_OK;
}

template <typename R>
int gather_t(nbody_ctx* c) {
    k_gather<R><<<nblk(c->n), TB, 0, c->st>>>(c->n, DP<uint32_t>(c->vals[0]), state<R>(c, c->cur),
                                              state<R>(c, 1 - c->cur));
    NB_LAUNCHED(c, "gather");
    c->launches += 1;
    c->cur = 1 - c->cur;
    return NBODY_OK;
}

}  // namespace

int nb_begin_step(nbody_ctx* c, int kdk) {
    return c->rsz == 4 ? begin_step_t<float>(c, kdk) : begin_step_t<double>(c, kdk);
}

// opening kick + drift of the current state buffer, nothing else (the frozen-structure replay)
int nb_kick_drift(nbody_ctx* c) {
    unsigned g = nblk(c->n);
    if (g > 152 * 8) g = 152 * 8;
    if (g == 0) g = 1;
    unsigned long long* bb = DP<unsigned long long>(c->bbox);
    if (c->rsz == 4)
        k_kick_drift_bbox<float><<<g, TB, 0, c->st>>>(c->n, state<float>(c, c->cur), 0.5 * c->prm.dt, c->prm.dt, 1,
                                                      bb, DP<int32_t>(c->info));
    else
        k_kick_drift_bbox<double><<<g, TB, 0, c->st>>>(c->n, state<double>(c, c->cur), 0.5 * c->prm.dt, c->prm.dt,
                                                       1, bb, DP<int32_t>(c->info));
    NB_LAUNCHED(c, "kick_drift");
    return NBODY_OK;
}

// drift of the current state buffer by dt, nothing else (block steps: substeps without a kick)
int nb_drift(nbody_ctx* c, double dt) {
    unsigned g = nblk(c->n);
    if (g > 152 * 8) g = 152 * 8;
    if (g == 0) g = 1;
    unsigned long long* bb = DP<unsigned long long>(c->bbox);
    if (c->rsz == 4)
        k_kick_drift_bbox<float><<<g, TB, 0, c->st>>>(c->n, state<float>(c, c->cur), 0.5 * dt, dt, 2, bb,
                                                      DP<int32_t>(c->info));
    else
        k_kick_drift_bbox<double><<<g, TB, 0, c->st>>>(c->n, state<double>(c, c->cur), 0.5 * dt, dt, 2, bb,
                                                       DP<int32_t>(c->info));
    NB_LAUNCHED(c, "drift");
    c->launches += 1;
    return NBODY_OK;
}

int nb_sort_and_gather(nbody_ctx* c) {
    int first = 1;
    NB_TRY(nb_radix_sort(c, c->n, DP<uint64_t>(c->keys[0]), DP<uint32_t>(c->vals[0]), DP<uint64_t>(c->keys[1]),
                         DP<uint32_t>(c->vals[1]), 0, 3 * NB_LEVELS, &first));
    if (!first) {
        std::swap(c->keys[0], c->keys[1]);
        std::swap(c->vals[0], c->vals[1]);
    }
    return c->rsz == 4 ? gather_t<float>(c) : gather_t<double>(c);
}

int nb_build_tree(nbody_ctx* c) {
    const int64_t n = c->n;
    const int C = c->prm.leaf_capacity;
    int32_t* info = DP<int32_t>(c->info);
    NB_CU(c, cudaMemsetAsync(info + INFO_DEPTH, 0, sizeof(int32_t) * (INFO_SCAN_ERR - INFO_DEPTH), c->st));
    k_tree_cpl<<<nblk(n), TB, 0, c->st>>>(n, C, DP<uint64_t>(c->keys[0]), DP<int32_t>(c->cpl), DP<int32_t>(c->wnd));
    k_tree_chain<<<nblk(n), TB, 0, c->st>>>(n, C, c->prm.max_level, DP<int32_t>(c->cpl), DP<int32_t>(c->wnd),
                                            DP<uint32_t>(c->nc), info);
    NB_LAUNCHED(c, "tree_chain");
    c->launches += 2;
    NB_TRY(nb_scan_u32(c, DP<uint32_t>(c->nc), DP<uint32_t>(c->pfx), n, (uint32_t*)(info + INFO_NNODES)));
    NB_CU(c, cudaMemcpyAsync(c->h_info, info, sizeof(int32_t) * INFO_WORDS, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaMemcpyAsync(c->h_box, c->box.p, sizeof(BoxDev), cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    c->box_side = c->h_box->side;
    if (c->h_info[INFO_SCAN_ERR]) return nb_fail(c, NBODY_ERR_CUDA, "a device scan did not complete in time");
    const uint32_t err = (uint32_t)c->h_info[INFO_ERR];
    if (err & NB_ERRBIT_NONFINITE) return nb_fail(c, NBODY_ERR_STATE, "non-finite particle position");
    if (err & NB_ERRBIT_ESCAPE) {
        if (c->escape_policy == NBODY_ESCAPE_ERROR)
            return nb_fail(c, NBODY_ERR_RANGE, "a particle left the fixed root box");
        ++c->escapes;
    }
    if (err & NB_ERRBIT_RANGE) return nb_fail(c, NBODY_ERR_RANGE, "no representable root box covers the particles");
    c->nnodes = (uint32_t)c->h_info[INFO_NNODES];
    c->nleaves = c->h_info[INFO_NLEAVES];
    c->depth = c->h_info[INFO_DEPTH];
    c->level_start[0] = 0;
    for (int l = 0; l <= NB_LEVELS + 1; ++l)
        c->level_start[l + 1] = c->level_start[l] + (l <= NB_LEVELS ? c->h_info[INFO_HIST + l] : 0);
    if (c->level_start[NB_LEVELS + 2] != c->nnodes)
        return nb_fail(c, NBODY_ERR_STATE, "octree level histogram does not match the node count");

    const int64_t nn = c->nnodes;
    NB_TRY(nb_grow(c, c->seedk[0], sizeof(uint64_t) * nn));
    NB_TRY(nb_grow(c, c->seedk[1], sizeof(uint64_t) * nn));
    NB_TRY(nb_grow(c, c->seedv[0], sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->seedv[1], sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->nodes, sizeof(NodeRec) * nn));
    NB_TRY(nb_grow(c, c->leafflag, sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->leafpfx, sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->leaves, sizeof(uint32_t) * (c->nleaves + 1)));

    k_tree_seeds<<<nblk(n), TB, 0, c->st>>>(n, DP<int32_t>(c->cpl), DP<uint32_t>(c->nc), DP<uint32_t>(c->pfx),
                                            DP<uint64_t>(c->seedk[0]), DP<uint32_t>(c->seedv[0]));
    NB_LAUNCHED(c, "tree_seeds");
    c->launches += 1;
    int first = 1;
    NB_TRY(nb_radix_sort(c, nn, DP<uint64_t>(c->seedk[0]), DP<uint32_t>(c->seedv[0]), DP<uint64_t>(c->seedk[1]),
                         DP<uint32_t>(c->seedv[1]), 0, 8, &first));
    int si = first ? 0 : 1;
    LevelStarts ls;
    for (int l = 0; l < NB_LEVELS + 3; ++l) ls.s[l] = c->level_start[l];
    k_tree_nodes<<<nblk(nn), TB, 0, c->st>>>(nn, n, c->depth, DP<uint64_t>(c->keys[0]), DP<uint64_t>(c->seedk[si]),
                                             DP<uint32_t>(c->seedv[si]), ls, DP<NodeRec>(c->nodes),
                                             DP<uint32_t>(c->leafflag));
    NB_LAUNCHED(c, "tree_nodes");
    c->launches += 1;
    NB_TRY(nb_scan_u32(c, DP<uint32_t>(c->leafflag), DP<uint32_t>(c->leafpfx), nn, nullptr));
    k_tree_leaves<<<nblk(nn), TB, 0, c->st>>>(nn, DP<uint32_t>(c->leafflag), DP<uint32_t>(c->leafpfx),
                                              DP<uint32_t>(c->leaves));
    NB_LAUNCHED(c, "tree_leaves");
    c->launches += 1;
    return NBODY_OK;
}

NB_DBG_ACCESSOR(tree)
