// FMM kernels of the step, templated on the precision form and the order.
//
// Replaces the reference kernels of src/moment.cl (P2M/M2M),
// src/interaction.cl (interaction finding), src/field.cl (pair and node
// fields) and src/force.cl (field -> force), plus the host integration loop
// of src/open_cl_simulation.cpp:572-616, with:
//   k_p2m       multipoles of every leaf about its geometric centre, and each
//               particle's offset from its leaf centre (packed with its charge);
//   k_m2m       one tree level per launch, children shifted to the parent
//               centre (translation offsets exact, in the shift precision);
//   (lists.cu)  the far-field and near-field lists of every cell
//               (src/interaction.cl:10-100 MAC and split rules);
//   k_m2l       every cell's far-field list at once (M2L into per-lane
//               partial expansions, fixed-order reduction);
//   k_l2l       one level per launch, parent's local expansion shifted down;
//   k_p2p       a warp per leaf: near-field sums over its partner leaves with
//               source tiles staged in shared memory, the local expansion
//               evaluated at each particle (L2P), and the integrator update as
//               the epilogue.
// Every per-target sum runs in a fixed order, so results are bitwise
// reproducible run to run.
#pragma once

#include <algorithm>
#include <cmath>
#include <type_traits>

#include "nbody_internal.cuh"
#include "fmm_ops.inc"

namespace nbfmm {

struct __align__(32) D4 {
    double x, y, z, w;
};

template <int MODE> struct Prec;
template <> struct Prec<NBODY_PREC_FP32> {
    typedef float R;   // state
    typedef float S;   // bulk arithmetic (P2P, M2L, P2M, L2P)
    typedef float H;   // expansions and shifts (M2M, L2L)
    typedef float4 S4;
    static constexpr bool kahan = false;
    static constexpr bool lane_smem = false;
};
template <> struct Prec<NBODY_PREC_MIXED> {
    typedef double R;
    typedef float S;
    typedef float H;   // FP32 shifts of offsets formed from the FP64 cell centres (the FP64 pipe is 1/64 rate)
    typedef float4 S4;
    static constexpr bool kahan = true;
    static constexpr bool lane_smem = false;
};
template <> struct Prec<NBODY_PREC_FP64> {
    typedef double R;
    typedef double S;
    typedef double H;
    typedef D4 S4;
    static constexpr bool kahan = false;
    static constexpr bool lane_smem = true;   // per-lane M2L arrays live in shared memory
};

// exact centre displacement (a - b) in box units
__device__ __forceinline__ void disp(const NodeRec& a, const NodeRec& b, double unit, double& dx, double& dy,
                                     double& dz) {
    long long ax, ay, az, bx, by, bz;
    nb_centre_fine(a, ax, ay, az);
    nb_centre_fine(b, bx, by, bz);
    dx = (double)(ax - bx) * unit;
    dy = (double)(ay - by) * unit;
    dz = (double)(az - bz) * unit;
}

__device__ __forceinline__ double centre_coord(uint32_t i, int level, double origin, double side) {
    return origin + ((double)i + 0.5) * (side / (double)(1u << level));
}

template <typename T>
__device__ __forceinline__ T shfl_xor_t(T v, int o) {
    return __shfl_xor_sync(0xffffffffu, v, o);
}

// centre displacement (a - b) in the bulk precision: the fine-unit difference is an integer below
// 2^23 and the fine unit a power of two, so the FP32 product equals the rounded FP64 one exactly
template <typename S>
__device__ __forceinline__ void disp_s(const NodeRec& a, const NodeRec& b, double unit, S& dx, S& dy, S& dz) {
    int ax, ay, az, bx, by, bz;
    centre_fine32(a, ax, ay, az);
    centre_fine32(b, bx, by, bz);
    const S u = (S)unit;
    dx = (S)(ax - bx) * u;
    dy = (S)(ay - by) * u;
    dz = (S)(az - bz) * u;
}

// Sum of a compensated pair (value = hi - comp) over the lane groups o = CT .. 16 of a butterfly,
// returned in the state precision.  Mixed form: the pairs are added in FP32 with an error-free
// two-sum, converted to FP64 once; otherwise the sum runs in R.
template <int MODE>
__device__ __forceinline__ typename Prec<MODE>::R group_sum(typename Prec<MODE>::S hi, typename Prec<MODE>::S comp,
                                                            int CT) {
    typedef typename Prec<MODE>::R R;
    if constexpr (Prec<MODE>::kahan) {
        float h = hi, l = -comp;
        for (int o = CT; o < 32; o <<= 1) {
            const float h2 = __shfl_xor_sync(0xffffffffu, h, o), l2 = __shfl_xor_sync(0xffffffffu, l, o);
            const float sum = h + h2, bb = sum - h;
            const float e = (h - (sum - bb)) + (h2 - bb);
            h = sum;
            l = l + l2 + e;
        }
        return (R)h + (R)l;
    } else {
        R v = (R)hi - (R)comp;
        for (int o = CT; o < 32; o <<= 1) v += shfl_xor_t(v, o);
        return v;
    }
}

// ---------------------------------------------------------------------------
// P2M at leaves + particle offsets
// ---------------------------------------------------------------------------
template <int MODE, int P>
__global__ void __launch_bounds__(128) k_p2m(int64_t nleaves, const uint32_t* __restrict__ leaves,
                                             const NodeRec* __restrict__ nodes, const BoxDev* __restrict__ boxp,
                                             const typename Prec<MODE>::R* __restrict__ x,
                                             const typename Prec<MODE>::R* __restrict__ y,
                                             const typename Prec<MODE>::R* __restrict__ z,
                                             const typename Prec<MODE>::R* __restrict__ q,
                                             typename Prec<MODE>::S4* __restrict__ src,
                                             typename Prec<MODE>::H* __restrict__ M) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    constexpr int T = nb_terms<P>::value;
    constexpr int TM = nb_tm<P>::value;
    __shared__ S pw[4][32][3][P + 1];
    __shared__ S qq[4][32];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * 4 + wib;
    if (w >= nleaves) return;
    const uint32_t k = leaves[w];
    const NodeRec nd = nodes[k];
    const BoxDev b = *boxp;
    const R cx = (R)centre_coord(nd.ix, nd.level, b.ox, b.side);
    const R cy = (R)centre_coord(nd.iy, nd.level, b.oy, b.side);
    const R cz = (R)centre_coord(nd.iz, nd.level, b.oz, b.side);
    constexpr int NPL = (T + 31) / 32;   // coefficients per lane
    int ex[NPL][3];
    S acc[NPL];
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        acc[j] = S(0);
        int a = lane + 32 * j;
        int aa = a < T ? a : 0;
        ex[j][0] = nb_mi[aa][0]; ex[j][1] = nb_mi[aa][1]; ex[j][2] = nb_mi[aa][2];
    }
    const uint32_t end = nd.begin + nd.count;
    for (uint32_t base = nd.begin; base < end; base += 32) {
        uint32_t i = base + lane;
        if (i < end) {
            S yx = (S)(x[i] - cx), yy = (S)(y[i] - cy), yz = (S)(z[i] - cz), qi = (S)q[i];
            typename Prec<MODE>::S4 o;
            o.x = yx; o.y = yy; o.z = yz; o.w = qi;
            src[i] = o;
            S v[3] = {yx, yy, yz};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                S p = S(1);
#pragma unroll
                for (int e = 0; e <= P; ++e) { pw[wib][lane][d][e] = p; p *= v[d]; }
            }
            qq[wib][lane] = qi;
        }
        __syncwarp();
        int cnt = end - base < 32 ? (int)(end - base) : 32;
        for (int jj = 0; jj < cnt; ++jj) {
            S qj = qq[wib][jj];
#pragma unroll
            for (int j = 0; j < NPL; ++j)
                acc[j] = nb_fma(qj, pw[wib][jj][0][ex[j][0]] * pw[wib][jj][1][ex[j][1]] * pw[wib][jj][2][ex[j][2]],
                                acc[j]);
        }
        __syncwarp();
    }
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        int a = lane + 32 * j;
        if (a < T) {
            H v = (H)acc[j] * (H)nb_invfact[a];
            M[(int64_t)k * TM + a] = v;
        }
    }
}

// ---------------------------------------------------------------------------
// M2M: one level, warp per internal node.  The children are shifted CB at a time: their multipoles
// and shift monomials are staged together, and each lane runs CB independent accumulation chains
// (one per child) over its coefficients' term pairs, then adds them to its sum in child order.
// ---------------------------------------------------------------------------
template <int MODE, int P>
__global__ void __launch_bounds__(128) k_m2m(int lo, int hi, const NodeRec* __restrict__ nodes,
                                             const BoxDev* __restrict__ boxp, typename Prec<MODE>::H* __restrict__ M) {
    typedef typename Prec<MODE>::H H;
    constexpr int T = nb_terms<P>::value;
    constexpr int TM = nb_tm<P>::value;
    constexpr int CB = sizeof(H) == 8 ? 4 : 8;      // children per round (shared memory below 48 KB)
    __shared__ H sM[4][CB][T];
    __shared__ H sY[4][CB][T];
    __shared__ H spw[4][CB][3][P + 1];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int k = lo + blockIdx.x * 4 + wib;
    if (k >= hi) return;
    const NodeRec nd = nodes[k];
    if (nd.nchild == 0) return;
    const double unit = boxp->unit;
    const unsigned short* st = Tabs<P>::m2m_start();
    const unsigned short* pr = Tabs<P>::m2m_pairs();
    constexpr int NPL = (T + 31) / 32;
    H acc[NPL];
#pragma unroll
    for (int j = 0; j < NPL; ++j) acc[j] = H(0);
    for (int c0 = 0; c0 < nd.nchild; c0 += CB) {
        const int nc = min(CB, (int)nd.nchild - c0);
        // powers of each child's offset, one lane per (child, axis); absent children shift by zero
        if (lane < 3 * CB) {
            const int c = lane / 3, ax = lane - 3 * c;
            H d = H(0), p = H(1);
            if (c < nc) {
                const NodeRec cn = nodes[nd.child_begin + c0 + c];
                double dx, dy, dz;
                disp(cn, nd, unit, dx, dy, dz);
                d = (H)(ax == 0 ? dx : ax == 1 ? dy : dz);
            }
            for (int e = 0; e <= P; ++e) { spw[wib][c][ax][e] = p; p *= d; }
        }
        for (int idx = lane; idx < CB * T; idx += 32) {
            const int c = idx / T, a = idx - c * T;
            sM[wib][c][a] = c < nc ? M[(int64_t)(nd.child_begin + c0 + c) * TM + a] : H(0);
        }
        __syncwarp();
        for (int idx = lane; idx < CB * T; idx += 32) {
            const int c = idx / T, a = idx - c * T;
            sY[wib][c][a] = spw[wib][c][0][nb_mi[a][0]] * spw[wib][c][1][nb_mi[a][1]] * spw[wib][c][2][nb_mi[a][2]] *
                            (H)nb_invfact[a];
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            const int a = lane + 32 * j;
            if (a < T) {
                H sc[CB];
#pragma unroll
                for (int c = 0; c < CB; ++c) sc[c] = H(0);
                for (int u = st[a]; u < st[a + 1]; ++u) {
                    const int pm = pr[2 * u], py = pr[2 * u + 1];
#pragma unroll
                    for (int c = 0; c < CB; ++c) sc[c] = nb_fma(sM[wib][c][pm], sY[wib][c][py], sc[c]);
                }
                H s = acc[j];
#pragma unroll
                for (int c = 0; c < CB; ++c) s += sc[c];
                acc[j] = s;
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        int a = lane + 32 * j;
        if (a < T) {
            M[(int64_t)k * TM + a] = acc[j];
        }
    }
}

// ---------------------------------------------------------------------------
// far field, part 2: M2L over every cell at once
//
// A warp per target; lanes take 32 list entries at a time, each computing the
// derivative tensor of its own displacement and contracting it with its
// source's multipoles into a per-lane partial local expansion; the partials
// are reduced in a fixed butterfly order.  The 32 multipole rows of a batch
// are brought into shared memory by TMA bulk copies (one cp.async.bulk per
// lane, completing on the stage's mbarrier) while the previous batch is
// being computed: two stages, every wait bounded in time.  Row stride in
// shared memory makes the per-lane 16-byte reads conflict free.
// Displacements are exact: 32-bit fine-unit offsets times the fine unit.
// ---------------------------------------------------------------------------
struct M2LArgs {
    const NodeRec* nodes;
    const BoxDev* box;
    const void* Mm2l;        // S*: multipoles read by M2L, row stride nb_tm<P>
    void* L;                 // H*: receives the M2L sum of each target
    const uint32_t *m2l_off, *m2l_cnt, *m2l_list;
    int32_t* info;
    double eps2;
    int64_t nnodes;
    long long wait_cycles;   // bound of each wait for this warp's bulk copies (SM clock cycles)
    const void* dtab;        // S*: derivative table (FP64 form; rows of stride nb_tm<P>), null: none
    int dt_R, dt_levels;     // its offset range and levels
};

// ---------------------------------------------------------------------------
// far field, part 1b (FP64 form): the derivative tensor D(r) of the M2L operator, tabulated.  Two
// cells of one level are an integer number of cells apart, and cells one level apart an odd number
// of half cells of the finer level, so at a given root box the pairs of the far-field lists take
// few distinct displacements (at theta = 0.5: same-level offsets within +-7 cells).  Per level l
// the table holds, in rows of nb_tm<P> entries:
//   [0, W^3)              t and s at level l, cell offset o = i_t - i_s in [-R, R]^3   (W = 2R+1)
//   [W^3, W^3 + V^3)      t at l, s at l+1, half-cell offset h = 2(2 i_t + 1) - (2 i_s + 1)
//   [W^3 + V^3, W^3+2V^3) t at l+1, s at l, h = (2 i_t + 1) - 2(2 i_s + 1)
//                         (h odd, |h| <= 2R+1: V = 2R+2 values per axis)
// Each row is derivs() of the same exact displacement (fine units x fine unit) that the M2L kernel
// forms for such a pair.  Pairs outside the table (cells two or more levels apart, offsets beyond
// R) compute D in place.  The FP64 form's D costs ~300 FP64 operations per pair at 1/64 of the
// FP32 rate, so a 448-byte row from L2 is cheaper; the FP32 bulk forms compute D per pair (a table
// row is one more stream from L2 beside the multipole rows, which measured slower there).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ int dtab_rows_per_level(int R) {
    const int W = 2 * R + 1, V = 2 * R + 2;
    return W * W * W + 2 * V * V * V;
}

// row of the pair (target t, source s), or -1
__device__ __forceinline__ int dtab_row(const NodeRec& t, const NodeRec& s, int R, int levels) {
    const int lt = t.level, ls = s.level;
    const int W = 2 * R + 1, V = 2 * R + 2, Q = dtab_rows_per_level(R);
    if (lt == ls) {
        if (lt >= levels) return -1;
        const int ox = (int)t.ix - (int)s.ix, oy = (int)t.iy - (int)s.iy, oz = (int)t.iz - (int)s.iz;
        if (ox < -R || ox > R || oy < -R || oy > R || oz < -R || oz > R) return -1;
        return lt * Q + ((ox + R) * W + (oy + R)) * W + (oz + R);
    }
    int hx, hy, hz, l, blk;
    if (ls == lt + 1) {
        hx = 2 * (2 * (int)t.ix + 1) - (2 * (int)s.ix + 1);
        hy = 2 * (2 * (int)t.iy + 1) - (2 * (int)s.iy + 1);
        hz = 2 * (2 * (int)t.iz + 1) - (2 * (int)s.iz + 1);
        l = lt;
        blk = W * W * W;
    } else if (lt == ls + 1) {
        hx = (2 * (int)t.ix + 1) - 2 * (2 * (int)s.ix + 1);
        hy = (2 * (int)t.iy + 1) - 2 * (2 * (int)s.iy + 1);
        hz = (2 * (int)t.iz + 1) - 2 * (2 * (int)s.iz + 1);
        l = ls;
        blk = W * W * W + V * V * V;
    } else {
        return -1;
    }
    const int H = 2 * R + 1;
    if (l + 1 >= levels || hx < -H || hx > H || hy < -H || hy > H || hz < -H || hz > H) return -1;
    return l * Q + blk + (((hx + H) >> 1) * V + ((hy + H) >> 1)) * V + ((hz + H) >> 1);
}

template <typename S, int P>
__global__ void __launch_bounds__(128) k_dtab(int levels, int R, const BoxDev* __restrict__ boxp, double eps2d,
                                              S* __restrict__ tab) {
    constexpr int T = nb_terms<P>::value;
    constexpr int TM = nb_tm<P>::value;
    const int Q = dtab_rows_per_level(R);
    const int64_t row = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (row >= (int64_t)levels * Q) return;
    const int l = (int)(row / Q), j = (int)(row % Q);
    const int W = 2 * R + 1, V = 2 * R + 2, H = 2 * R + 1;
    int fx, fy, fz;                  // displacement t - s in fine units (side / 2^22)
    bool used = true;
    if (j < W * W * W) {
        const int ox = j / (W * W) - R, oy = (j / W) % W - R, oz = j % W - R;
        const int u = 1 << (NB_LEVELS + 1 - l);
        fx = ox * u; fy = oy * u; fz = oz * u;
    } else {
        const int k = (j - W * W * W) % (V * V * V);
        const int hx = 2 * (k / (V * V)) - H, hy = 2 * ((k / V) % V) - H, hz = 2 * (k % V) - H;
        used = l + 1 <= NB_LEVELS;
        const int u = used ? 1 << (NB_LEVELS - 1 - l) : 0;
        fx = hx * u; fy = hy * u; fz = hz * u;
    }
    S* out = tab + row * TM;
    if (!used) {
        for (int a = 0; a < TM; ++a) out[a] = S(0);
        return;
    }
    const S unit = (S)boxp->unit;
    const S dx = (S)fx * unit, dy = (S)fy * unit, dz = (S)fz * unit;
    S D[T];
    Ops<S, P>::template derivs<1>(dx, dy, dz, (S)eps2d, D);
    for (int a = 0; a < T; ++a) out[a] = D[a];
    for (int a = T; a < TM; ++a) out[a] = S(0);
}

template <int MODE, int P>
struct M2LSmem {
    typedef typename Prec<MODE>::S S;
    static constexpr int T = nb_terms<P>::value;
    static constexpr int TM = nb_tm<P>::value;
    // Up to order 5 in FP32 the kernel fits 128 registers, and five 3-warp blocks (15 warps) fit an
    // SM's shared memory only with unpadded rows (2-way bank conflicts on the 16-byte row reads, a
    // few cycles per 462 FMAs); above that, rows with an odd number of 16-byte chunks (the 8 lanes of
    // a quarter warp then read 8 distinct bank groups) and 4-warp blocks.
    static constexpr bool dense = sizeof(S) == 4 && P <= 5;
    static constexpr int SST = dense ? TM : sizeof(S) == 4 ? ((TM / 4) % 2 ? TM : TM + 4) : TM + 2;
    static constexpr int warps = Prec<MODE>::lane_smem ? 1 : dense ? 3 : 4;
    static constexpr int min_blocks = dense ? 5 : 1;
    static constexpr size_t rows = (size_t)2 * 32 * SST * sizeof(S);
    static constexpr size_t lane_arrays = Prec<MODE>::lane_smem ? (size_t)2 * 32 * T * sizeof(S) : 0;
    static constexpr size_t per_warp = (16 + rows + lane_arrays + 127) / 128 * 128;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// warp-uniform bounded wait of at most `limit` SM clock cycles; false on timeout
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    bool ok = false;
    for (;;) {
        ok = ok || mbar_try_wait(bar, parity);
        if (__all_sync(0xffffffffu, ok)) return true;
        const long long dt = __shfl_sync(0xffffffffu, clock64() - t0, 0);
        if (dt > limit) return false;
    }
}

template <int MODE, int P>
__global__ void __launch_bounds__(32 * M2LSmem<MODE, P>::warps, M2LSmem<MODE, P>::min_blocks) k_m2l(M2LArgs A) {
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    constexpr int T = nb_terms<P>::value;
    constexpr int TM = nb_tm<P>::value;
    constexpr int SST = M2LSmem<MODE, P>::SST;
    constexpr bool LS = Prec<MODE>::lane_smem;
    constexpr int W = M2LSmem<MODE, P>::warps;
    constexpr uint32_t ROWB = TM * sizeof(S);
    extern __shared__ __align__(256) unsigned char smem_raw[];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * W + wib;
    if (t >= A.nnodes) return;
    unsigned char* ws = smem_raw + (size_t)wib * M2LSmem<MODE, P>::per_warp;
    uint64_t* bar = (uint64_t*)ws;
    S* rows = (S*)(ws + 16);
    S* laneD = rows + 2 * 32 * SST;
    S* laneL = laneD + 32 * T;
    const NodeRec nt = A.nodes[t];
    int tcx, tcy, tcz;
    centre_fine32(nt, tcx, tcy, tcz);
    const S unit = (S)A.box->unit;
    const S eps2 = (S)A.eps2;
    const S* Msrc = (const S*)A.Mm2l;
    const S* __restrict__ dtab = (const S*)A.dtab;
    const uint32_t off = A.m2l_off[t], cnt = A.m2l_cnt[t];
    const uint32_t nbatch = (cnt + 31) / 32;
    S Lreg[LS ? 1 : T];
    if constexpr (LS) {
        for (int a = 0; a < T; ++a) laneL[a * 32 + lane] = S(0);
    } else {
#pragma unroll
        for (int a = 0; a < T; ++a) Lreg[a] = S(0);
    }
    if (lane == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    __syncwarp();
    // this lane's list entry of batch b (0 past the end)
    auto entry = [&](uint32_t b) -> uint32_t {
        const uint32_t j = 32 * b + lane;
        return b < nbatch && j < cnt ? NB_IDX(A.m2l_list[off + j], A.nnodes, NB_SITE_M2L) : 0u;
    };
    // issue the bulk copies of batch b (source s of this lane, loaded one batch earlier) into stage
    // b & 1; returns the lane's source node record, loaded now and used one batch later
    auto issue = [&](uint32_t b, uint32_t s) -> NodeRec {
        const uint32_t nb = min(32u, cnt - 32 * b);
        const uint32_t k = b & 1;
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_expect_tx(&bar[k], nb * ROWB);
        __syncwarp();
        if ((uint32_t)lane < nb) bulk_g2s(rows + (k * 32 + lane) * SST, Msrc + (int64_t)s * TM, ROWB, &bar[k]);
        return A.nodes[s];
    };
    bool failed = false;
    uint32_t b_fail = 0;
    NodeRec sn_next;
    uint32_t s_ahead = entry(1);       // list entries run two batches ahead of the computation
    if (nbatch) sn_next = issue(0, entry(0));
    for (uint32_t b = 0; b < nbatch; ++b) {
        const NodeRec sn = sn_next;
        const uint32_t k = b & 1;
        const uint32_t nb = min(32u, cnt - 32 * b);
        if (b + 1 < nbatch) {
            sn_next = issue(b + 1, s_ahead);
            s_ahead = entry(b + 2);
        }
        if (!mbar_wait_warp(&bar[k], (b >> 1) & 1, A.wait_cycles)) { failed = true; b_fail = b; break; }
        if ((uint32_t)lane < nb) {
            int sx, sy, sz;
            centre_fine32(sn, sx, sy, sz);
            const S dx = (S)(tcx - sx) * unit, dy = (S)(tcy - sy) * unit, dz = (S)(tcz - sz) * unit;
            const S* row = rows + (k * 32 + lane) * SST;
            if constexpr (LS) {
                const int drow = dtab ? dtab_row(nt, sn, A.dt_R, A.dt_levels) : -1;
                if (drow >= 0) {
                    const S* dr = dtab + (int64_t)drow * TM;
                    for (int a = 0; a < T; ++a) laneD[a * 32 + lane] = dr[a];
                } else {
                    Ops<S, P>::template derivs<32>(dx, dy, dz, eps2, laneD + lane);
                }
                Ops<S, P>::template m2l_v<32>(row, laneD + lane, laneL + lane);
            } else {
                S D[T];
                Ops<S, P>::template derivs<1>(dx, dy, dz, eps2, D);
                Ops<S, P>::template m2l_v<1>(row, D, Lreg);
            }
        }
        __syncwarp();
    }
    if (failed) {
        // let every copy already issued land before the shared memory is released (with the
        // default bound, whatever the configured one: these copies are in flight)
        if (lane == 0) atomicOr((unsigned int*)&A.info[INFO_ERR], NB_ERRBIT_ASYNC);
        mbar_wait_warp(&bar[b_fail & 1], (b_fail >> 1) & 1, NB_COPY_CYCLES);
        if (b_fail + 1 < nbatch)
            mbar_wait_warp(&bar[(b_fail + 1) & 1], ((b_fail + 1) >> 1) & 1, NB_COPY_CYCLES);
        return;
    }
    // lane-order butterfly sums; lane a % 32 keeps coefficient a and converts only its own
    constexpr int NPL = (T + 31) / 32;
    S own[NPL];
#pragma unroll
    for (int j = 0; j < NPL; ++j) own[j] = S(0);
#pragma unroll
    for (int a = 0; a < T; ++a) {
        S v;
        if constexpr (LS) v = laneL[a * 32 + lane];
        else v = Lreg[a];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += shfl_xor_t(v, o);
        if ((a & 31) == lane) own[a >> 5] = v;
    }
    H* Lg = (H*)A.L;
#pragma unroll
    for (int j = 0; j < NPL; ++j)
        if (lane + 32 * j < T) Lg[t * T + lane + 32 * j] = (H)own[j];
}

// ---------------------------------------------------------------------------
// far field, part 3: L2L, one level per launch (top down), warp per cell:
// L(t) = M2L sum of t + parent's L shifted to t's centre (exact FP64 offset
// in the mixed and FP64 forms).
// ---------------------------------------------------------------------------
template <int MODE, int P>
__global__ void __launch_bounds__(128) k_l2l(int lo, int hi, const NodeRec* __restrict__ nodes,
                                             const BoxDev* __restrict__ boxp, typename Prec<MODE>::H* __restrict__ L) {
    typedef typename Prec<MODE>::H H;
    constexpr int T = nb_terms<P>::value;
    __shared__ H sLp[4][T];
    __shared__ H sY[4][T];
    __shared__ H spw[4][3][P + 1];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int t = lo + blockIdx.x * 4 + wib;
    if (t >= hi) return;
    const NodeRec nt = nodes[t];
    const int par = nt.parent;
    const NodeRec pn = nodes[par];
    double dx, dy, dz;
    disp(nt, pn, boxp->unit, dx, dy, dz);
    for (int a = lane; a < T; a += 32) sLp[wib][a] = L[(int64_t)par * T + a];
    if (lane < 3) {
        H d = (H)(lane == 0 ? dx : lane == 1 ? dy : dz), p = H(1);
        for (int e = 0; e <= P; ++e) { spw[wib][lane][e] = p; p *= d; }
    }
    __syncwarp();
    for (int a = lane; a < T; a += 32)
        sY[wib][a] = spw[wib][0][nb_mi[a][0]] * spw[wib][1][nb_mi[a][1]] * spw[wib][2][nb_mi[a][2]] *
                     (H)nb_invfact[a];
    __syncwarp();
    const unsigned short* st = Tabs<P>::l2l_start();
    const unsigned short* pr = Tabs<P>::l2l_pairs();
    for (int a = lane; a < T; a += 32) {
        H v = L[(int64_t)t * T + a];
        for (int u = st[a]; u < st[a + 1]; ++u) v = nb_fma(sLp[wib][pr[2 * u]], sY[wib][pr[2 * u + 1]], v);
        L[(int64_t)t * T + a] = v;
    }
}

// ---------------------------------------------------------------------------
// near field + L2P + integrator epilogue
//
// Work item = (leaf, chunk of at most P2P_CHUNK partner leaves); a leaf with a
// long partner list (a large sparse leaf next to a dense region) is spread
// over several warps whose partial sums are added in chunk order by
// k_p2p_final.  Within a warp, lanes hold target particles (groups of CT
// lanes); NG = 32/CT groups take partner leaves round-robin.  Partner node
// records are fetched 32 at a time (one per lane) and broadcast by shuffle;
// each source tile is prefetched into registers while the previous one is
// evaluated out of shared memory.
// ---------------------------------------------------------------------------
struct P2PArgs {
    const uint32_t* leaves;
    int64_t nleaves;
    int64_t nnodes, n;      // node and particle counts (index checks of the debug build)
    const NodeRec* nodes;
    const BoxDev* box;
    const void* src;        // S4*
    const void* L;          // H*
    const uint32_t *p2p_off, *p2p_cnt, *p2p_list;
    const uint32_t* work_off;   // nleaves + 1: first work item of each leaf
    int64_t nwork;
    const uint32_t* part_off;   // nleaves + 1: partial-sum slot of each multi-chunk leaf
    void* part;                 // R[4] per (chunk, target particle)
    void *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az;   // R*
    const void *m, *q;      // R*
    void* pot;              // R* or null
    double eps2, G, dt;
    int integ;
    const uint8_t* leaf_active;   // block steps: per leaf (near-field order), 0 = no particle closes a step
                                  // at this substep, its near field and L2P are skipped; null: every leaf
};

template <typename S>
__device__ __forceinline__ void kahan_add(S& sum, S& comp, S v) {
    S yv = v - comp;
    S tv = sum + yv;
    comp = (tv - sum) - yv;
    sum = tv;
}

constexpr int P2P_WARPS = 4;
constexpr int P2P_TILE = 32;      // source particles per tile and group
constexpr int P2P_CHUNK = NB_P2P_CHUNK;   // partner leaves per work item

template <int MODE, int P>
__device__ __forceinline__ void p2p_epilogue(const P2PArgs& A, uint32_t i, const typename Prec<MODE>::S* sL,
                                             typename Prec<MODE>::S4 yi, typename Prec<MODE>::R Ex,
                                             typename Prec<MODE>::R Ey, typename Prec<MODE>::R Ez,
                                             typename Prec<MODE>::R Ps, bool pot) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    S fx, fy, fz, fp;
    Ops<S, P>::l2p(sL, yi.x, yi.y, yi.z, fx, fy, fz, fp);
    Ex += (R)fx; Ey += (R)fy; Ez += (R)fz;
    Ps += (R)fp;
    const R* mq = (const R*)A.m;
    const R* qq = (const R*)A.q;
    const R f = (R)A.G * qq[i] / mq[i];
    const R axv = f * Ex, ayv = f * Ey, azv = f * Ez;
    R* X = (R*)A.x; R* Y = (R*)A.y; R* Z = (R*)A.z;
    R* VX = (R*)A.vx; R* VY = (R*)A.vy; R* VZ = (R*)A.vz;
    R* AX = (R*)A.ax; R* AY = (R*)A.ay; R* AZ = (R*)A.az;
    AX[i] = axv; AY[i] = ayv; AZ[i] = azv;
    if (A.integ == NB_INTEG_KDK_CLOSE) {
        const R h = (R)(0.5 * A.dt);
        VX[i] += h * axv; VY[i] += h * ayv; VZ[i] += h * azv;
    } else if (A.integ == NB_INTEG_EULER) {
        const R dt = (R)A.dt;
        const R vx0 = VX[i], vy0 = VY[i], vz0 = VZ[i];
        VX[i] = vx0 + axv * dt; VY[i] = vy0 + ayv * dt; VZ[i] = vz0 + azv * dt;
        X[i] += vx0 * dt; Y[i] += vy0 * dt; Z[i] += vz0 * dt;
    }
    if (pot) ((R*)A.pot)[i] = -(R)A.G * Ps;
}

// lanes per target group and targets per lane of near-field class CLS (see nb_p2p_class)
template <int CLS> struct P2PShape;
template <> struct P2PShape<0> { static constexpr int CT = 4, TPL = 2; };
template <> struct P2PShape<1> { static constexpr int CT = 8, TPL = 2; };
template <> struct P2PShape<2> { static constexpr int CT = 8, TPL = 3; };
template <> struct P2PShape<3> { static constexpr int CT = 16, TPL = 2; };
template <> struct P2PShape<4> { static constexpr int CT = 16, TPL = 3; };
template <> struct P2PShape<5> { static constexpr int CT = 32, TPL = 2; };
constexpr int P2P_WTILE = 128;    // shared source entries per warp (groups x entries per group)
// shared rows per warp: each group's tile is followed by one pad entry, so the groups of a half-warp
// (which read different entries in the same step) fall in distinct shared-memory banks
constexpr int P2P_WROWS = P2P_WTILE + 8;

// which leaf / chunk a near-field work item is: last li in [lo, hi) with work_off[li] <= w
__device__ __forceinline__ int64_t p2p_leaf_of(const uint32_t* work_off, int64_t lo, int64_t hi, uint32_t w) {
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (work_off[mid] <= w) lo = mid; else hi = mid;
    }
    return lo;
}

// One warp's share of a near-field work item: every target of the leaf (TPL per lane, CT lanes per
// group) against the partner leaves [s_lo, s_hi) of its list.  NG = 32/CT groups take partner
// leaves round-robin; each group's source tile (TILE entries) is prefetched into registers while
// the previous one is evaluated from shared memory.  GUARD: unsoftened kernel, r = 0 gives 0.
template <int MODE, int P, bool POT, bool GUARD, int CT, int TPL>
__device__ __forceinline__ void p2p_item(const P2PArgs& A, typename Prec<MODE>::S4* tile,
                                         const typename Prec<MODE>::S* sL, uint32_t k, const NodeRec& nt,
                                         int64_t li, uint32_t chunk, uint32_t nchunk, uint32_t s_lo,
                                         uint32_t s_hi) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::S4 S4;
    constexpr bool KH = Prec<MODE>::kahan;
    constexpr int NG = 32 / CT;
    constexpr int TILE = P2P_WTILE / NG < 32 ? P2P_WTILE / NG : 32;
    constexpr int EPL = TILE / CT;          // tile entries each lane loads
    static_assert(NG * (TILE + 1) <= P2P_WROWS, "group tiles exceed the warp's shared rows");
    const int lane = lane_id();
    const int grp = lane / CT, gl = lane % CT;
    S4* gtile = tile + grp * (TILE + 1);
    const double unit = A.box->unit;
    const S4* src = (const S4*)A.src;
    const uint32_t cnt_t = nt.count;
    const uint32_t loff = A.p2p_off[k];
    const S eps2 = (S)A.eps2;
    S4 zero4;
    zero4.x = 0; zero4.y = 0; zero4.z = 0; zero4.w = 0;
    for (uint32_t tc = 0; tc < cnt_t; tc += TPL * CT) {
        uint32_t ti[TPL], ii[TPL];
        bool tv[TPL];
        S4 y[TPL];
        S acc[TPL][4], cmp[TPL][4];
#pragma unroll
        for (int j = 0; j < TPL; ++j) {
            ti[j] = tc + gl + j * CT;
            tv[j] = ti[j] < cnt_t;
            ii[j] = nt.begin + (tv[j] ? ti[j] : 0);
            y[j] = src[ii[j]];
#pragma unroll
            for (int q = 0; q < 4; ++q) { acc[j][q] = 0; cmp[j][q] = 0; }
        }
        for (uint32_t base = s_lo; base < s_hi; base += 32) {
            const uint32_t nb = min(32u, s_hi - base);
            uint32_t my_s = 0, my_beg = 0, my_cnt = 0;
            S my_dx = 0, my_dy = 0, my_dz = 0;
            if ((uint32_t)lane < nb) {
                my_s = NB_IDX(A.p2p_list[loff + base + lane], A.nnodes, NB_SITE_P2P);
                const NodeRec sn = A.nodes[my_s];
                my_beg = NB_IDX(sn.begin, A.n, NB_SITE_P2P);
                my_cnt = NB_IDX(sn.count, A.n + 1 - my_beg, NB_SITE_P2P);
                disp_s<S>(sn, nt, unit, my_dx, my_dy, my_dz);
            }
            // partners of this batch in descending particle count: the NG groups of a round then
            // take leaves of similar size, so fewer lanes wait on the longest one
            {
                const uint32_t key = (min(my_cnt, 1u << 26) << 5) | (31u - (uint32_t)lane);
                const int from = 31 - (int)(warp_sort_desc(key) & 31u);
                my_s = __shfl_sync(0xffffffffu, my_s, from);
                my_beg = __shfl_sync(0xffffffffu, my_beg, from);
                my_cnt = __shfl_sync(0xffffffffu, my_cnt, from);
                my_dx = __shfl_sync(0xffffffffu, my_dx, from);
                my_dy = __shfl_sync(0xffffffffu, my_dy, from);
                my_dz = __shfl_sync(0xffffffffu, my_dz, from);
            }
            const uint32_t rounds = (nb + NG - 1) / NG;
            uint32_t rr = 0, sb = 0;
            S4 pre[EPL];
            {
                const uint32_t cbeg = __shfl_sync(0xffffffffu, my_beg, grp);
                const uint32_t ccnt0 = __shfl_sync(0xffffffffu, my_cnt, grp);
                const uint32_t ccnt = (uint32_t)grp < nb ? ccnt0 : 0u;
#pragma unroll
                for (int e = 0; e < EPL; ++e) {
                    const uint32_t j = gl + e * CT;
                    pre[e] = j < ccnt ? src[cbeg + j] : zero4;
                }
            }
            while (rr < rounds) {
                const uint32_t q = rr * NG + grp;
                const uint32_t qs = q & 31;
                const uint32_t s_id = __shfl_sync(0xffffffffu, my_s, qs);
                const S dx = __shfl_sync(0xffffffffu, my_dx, qs), dy = __shfl_sync(0xffffffffu, my_dy, qs),
                        dz = __shfl_sync(0xffffffffu, my_dz, qs);
                const uint32_t scnt0 = __shfl_sync(0xffffffffu, my_cnt, qs);
                const uint32_t scnt = q < nb ? scnt0 : 0u;
                // the round's largest partner: partners are sorted by particle count, so it is the first
                const uint32_t mx = __shfl_sync(0xffffffffu, my_cnt, (rr * NG) & 31);
#pragma unroll
                for (int e = 0; e < EPL; ++e) gtile[gl + e * CT] = pre[e];
                __syncwarp();
                uint32_t nrr = rr, nsb = sb + TILE;
                if (nsb >= mx) { nrr = rr + 1; nsb = 0; }
                {
                    const uint32_t nq = nrr * NG + grp;
                    const uint32_t nbeg = __shfl_sync(0xffffffffu, my_beg, nq & 31);
                    const uint32_t ncnt0 = __shfl_sync(0xffffffffu, my_cnt, nq & 31);
                    const uint32_t ncnt = (nrr < rounds && nq < nb) ? ncnt0 : 0u;
#pragma unroll
                    for (int e = 0; e < EPL; ++e) {
                        const uint32_t j = nsb + gl + e * CT;
                        pre[e] = j < ncnt ? src[nbeg + j] : zero4;
                    }
                }
                // targets shifted into the source leaf's frame
                S xs[TPL][3];
#pragma unroll
                for (int j = 0; j < TPL; ++j) { xs[j][0] = y[j].x - dx; xs[j][1] = y[j].y - dy; xs[j][2] = y[j].z - dz; }
                const int nj = scnt > sb ? min((int)(scnt - sb), TILE) : 0;
                const bool self = POT && s_id == k;
                S p[TPL][4];
#pragma unroll
                for (int j = 0; j < TPL; ++j) { p[j][0] = 0; p[j][1] = 0; p[j][2] = 0; p[j][3] = 0; }
#pragma unroll (TPL == 2 ? 4 : 2)
                for (int e = 0; e < nj; ++e) {
                    const S4 sj = gtile[e];
#pragma unroll
                    for (int j = 0; j < TPL; ++j) {
                        const S rx = sj.x - xs[j][0], ry = sj.y - xs[j][1], rz = sj.z - xs[j][2];
                        S s2 = nb_fma(rx, rx, nb_fma(ry, ry, nb_fma(rz, rz, eps2)));
                        if (GUARD) s2 = s2 > S(0) ? s2 : S(1e30);
                        S inv = GUARD ? nb_rsqrt(s2) : nb_rsqrt_n(s2);
                        if (self && sb + e == ti[j]) inv = S(0);
                        const S w = sj.w * inv * inv * inv;
                        p[j][0] = nb_fma(rx, w, p[j][0]);
                        p[j][1] = nb_fma(ry, w, p[j][1]);
                        p[j][2] = nb_fma(rz, w, p[j][2]);
                        if (POT) p[j][3] = nb_fma(sj.w, inv, p[j][3]);
                    }
                }
#pragma unroll
                for (int j = 0; j < TPL; ++j)
#pragma unroll
                    for (int q = 0; q < (POT ? 4 : 3); ++q) {
                        if (KH) kahan_add(acc[j][q], cmp[j][q], p[j][q]);
                        else acc[j][q] += p[j][q];
                    }
                __syncwarp();
                rr = nrr;
                sb = nsb;
            }
        }
        // combine the source groups in a fixed order
        R tot[TPL][4];
#pragma unroll
        for (int j = 0; j < TPL; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) tot[j][q] = (POT || q < 3) ? group_sum<MODE>(acc[j][q], cmp[j][q], CT) : R(0);
        if (grp == 0) {
#pragma unroll
            for (int j = 0; j < TPL; ++j) {
                if (!tv[j]) continue;
                if (nchunk == 1) {
                    p2p_epilogue<MODE, P>(A, ii[j], sL, y[j], tot[j][0], tot[j][1], tot[j][2], tot[j][3], POT);
                } else {
                    R* pt = (R*)A.part + 4 * ((int64_t)A.part_off[li] + (int64_t)chunk * cnt_t + ti[j]);
                    pt[0] = tot[j][0]; pt[1] = tot[j][1]; pt[2] = tot[j][2]; pt[3] = tot[j][3];
                }
            }
        }
        __syncwarp();
    }
}

// near-field work items of one leaf-size class: items [w_lo, w_hi) of leaves [li_lo, li_hi)
template <int MODE, int P, bool POT, int CLS>
__global__ void __launch_bounds__(32 * P2P_WARPS, P2PShape<CLS>::TPL == 3 ? 4 : 5) k_p2p(P2PArgs A, int64_t li_lo,
                                                                                      int64_t li_hi, uint32_t w_lo,
                                                                                      uint32_t w_hi) {
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    typedef typename Prec<MODE>::S4 S4;
    constexpr int T = nb_terms<P>::value;
    constexpr int CT = P2PShape<CLS>::CT, TPL = P2PShape<CLS>::TPL;
    __shared__ S4 tile[P2P_WARPS][P2P_WROWS];
    __shared__ S sL[P2P_WARPS][T];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const uint32_t w = w_lo + blockIdx.x * P2P_WARPS + wib;
    if (w >= w_hi) return;
    const int64_t li = p2p_leaf_of(A.work_off, li_lo, li_hi, w);
    if (A.leaf_active && !A.leaf_active[li]) return;
    const uint32_t chunk = w - A.work_off[li];
    const uint32_t nchunk = A.work_off[li + 1] - A.work_off[li];
    const uint32_t k = A.leaves[li];
    const NodeRec nt = A.nodes[k];
    if (nchunk == 1) {
        const H* Lg = (const H*)A.L;
        for (int a = lane; a < T; a += 32) sL[wib][a] = (S)Lg[(int64_t)k * T + a];
    }
    const uint32_t lcnt = A.p2p_cnt[k];
    const uint32_t s_lo = chunk * P2P_CHUNK, s_hi = min(lcnt, s_lo + P2P_CHUNK);
    __syncwarp();
    if (A.eps2 > 0.0)
        p2p_item<MODE, P, POT, false, CT, TPL>(A, tile[wib], sL[wib], k, nt, li, chunk, nchunk, s_lo, s_hi);
    else
        p2p_item<MODE, P, POT, true, CT, TPL>(A, tile[wib], sL[wib], k, nt, li, chunk, nchunk, s_lo, s_hi);
}

// sums the chunk partials of multi-chunk leaves in chunk order, then L2P + epilogue
template <int MODE, int P, bool POT>
__global__ void __launch_bounds__(32 * P2P_WARPS) k_p2p_final(P2PArgs A) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    typedef typename Prec<MODE>::S4 S4;
    constexpr int T = nb_terms<P>::value;
    __shared__ S sL[P2P_WARPS][T];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int64_t li = (int64_t)blockIdx.x * P2P_WARPS + wib;
    if (li >= A.nleaves) return;
    const uint32_t nchunk = A.work_off[li + 1] - A.work_off[li];
    if (nchunk <= 1) return;
    if (A.leaf_active && !A.leaf_active[li]) return;
    const uint32_t k = A.leaves[li];
    const NodeRec nt = A.nodes[k];
    const H* Lg = (const H*)A.L;
    for (int a = lane; a < T; a += 32) sL[wib][a] = (S)Lg[(int64_t)k * T + a];
    __syncwarp();
    const S4* src = (const S4*)A.src;
    for (uint32_t ti = lane; ti < nt.count; ti += 32) {
        R e[4] = {0, 0, 0, 0};
        for (uint32_t c = 0; c < nchunk; ++c) {
            const R* pt = (const R*)A.part + 4 * ((int64_t)A.part_off[li] + (int64_t)c * nt.count + ti);
            e[0] += pt[0]; e[1] += pt[1]; e[2] += pt[2]; e[3] += pt[3];
        }
        const uint32_t i = nt.begin + ti;
        p2p_epilogue<MODE, P>(A, i, sL[wib], src[i], e[0], e[1], e[2], e[3], POT);
    }
}

// ---------------------------------------------------------------------------
// host driver for one (mode, order)
// ---------------------------------------------------------------------------
// one launch per non-empty leaf-size class, over that class's work items
template <int MODE, int P, bool POT>
int p2p_launch_classes(nbody_ctx* c, const P2PArgs& B) {
    const int32_t* hi = c->h_info;
    auto one = [&](auto cls_tag) -> int {
        constexpr int CLS = decltype(cls_tag)::value;
        const uint32_t w0 = (uint32_t)hi[INFO_CLS_WORK + CLS], w1 = (uint32_t)hi[INFO_CLS_WORK + CLS + 1];
        if (w1 <= w0) return NBODY_OK;
        const int64_t l0 = (uint32_t)hi[INFO_CLS_LEAF + CLS], l1 = (uint32_t)hi[INFO_CLS_LEAF + CLS + 1];
        k_p2p<MODE, P, POT, CLS><<<(w1 - w0 + P2P_WARPS - 1) / P2P_WARPS, 32 * P2P_WARPS, 0, c->side[CLS]>>>(B, l0, l1,
                                                                                                      w0, w1);
        NB_LAUNCHED(c, "p2p");
        c->launches += 1;
        return NBODY_OK;
    };
    // the classes write disjoint particles: run them side by side so no launch tail idles the GPU
    NB_TRY(nb_fork(c));
    NB_TRY(one(std::integral_constant<int, 5>()));
    NB_TRY(one(std::integral_constant<int, 4>()));
    NB_TRY(one(std::integral_constant<int, 3>()));
    NB_TRY(one(std::integral_constant<int, 2>()));
    NB_TRY(one(std::integral_constant<int, 1>()));
    NB_TRY(one(std::integral_constant<int, 0>()));
    return nb_join(c);
}
// (re)builds the FP64 form's derivative table when the root box side, the softening, the opening
// angle's offset range or the order changed, or the tree is deeper than the table
template <int MODE, int P>
int dtab_ensure(nbody_ctx* c) {
    typedef typename Prec<MODE>::S S;
    if (!Prec<MODE>::lane_smem) return NBODY_OK;   // the FP32 bulk forms compute D per pair
    const int R = (int)std::floor(2.0 * std::sqrt(3.0) / c->prm.theta) + 1;
    const int levels = c->depth + 1;
    if (R > 24) return NBODY_OK;        // small opening angles: too many offsets, D is computed per pair
    if (c->dt_prec == MODE && c->dt_order == P && c->dt_R == R && c->dt_side == c->box_side &&
        c->dt_eps == c->prm.eps && c->dt_levels >= levels)
        return NBODY_OK;
    const int lv = std::max(levels, c->dt_prec == MODE && c->dt_order == P && c->dt_R == R ? c->dt_levels : 0);
    const int64_t rows = (int64_t)lv * dtab_rows_per_level(R);
    NB_TRY(nb_grow(c, c->dtab, sizeof(S) * nb_tm<P>::value * (size_t)rows));
    k_dtab<S, P><<<(unsigned)((rows + 127) / 128), 128, 0, c->st>>>(lv, R, DP<BoxDev>(c->box),
                                                                    c->prm.eps * c->prm.eps, DP<S>(c->dtab));
    NB_LAUNCHED(c, "m2l derivative table");
    c->launches += 1;
    c->dt_prec = MODE;
    c->dt_order = P;
    c->dt_R = R;
    c->dt_side = c->box_side;
    c->dt_eps = c->prm.eps;
    c->dt_levels = lv;
    return NBODY_OK;
}

template <int MODE, int P>
void dtab_args(const nbody_ctx* c, M2LArgs& B) {
    const bool ok = Prec<MODE>::lane_smem && c->dt_prec == MODE && c->dt_order == P && c->dt_side == c->box_side &&
                    c->dt_eps == c->prm.eps;
    B.dtab = ok ? c->dtab.p : nullptr;
    B.dt_R = c->dt_R;
    B.dt_levels = ok ? c->dt_levels : 0;
}

template <int MODE, int P>
int fmm_forces(nbody_ctx* c, int integ, bool want_pot) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    typedef typename Prec<MODE>::S4 S4;
    constexpr int T = nb_terms<P>::value;
    const int64_t nn = c->nnodes, n = c->n;
    const int cur = c->cur;
    constexpr int TM = nb_tm<P>::value;
    NB_TRY(nb_grow(c, c->M, sizeof(H) * TM * nn));
    NB_TRY(nb_grow(c, c->L, sizeof(H) * T * nn));
    NB_TRY(nb_grow(c, c->src, sizeof(S4) * n));
    const BoxDev* box = DP<BoxDev>(c->box);

    if (c->timing) cudaEventRecord(c->ev[3], c->st);
    k_p2m<MODE, P><<<(unsigned)((c->nleaves + 3) / 4), 128, 0, c->st>>>(
        c->nleaves, DP<uint32_t>(c->leaves), DP<NodeRec>(c->nodes), box, DP<R>(c->x[cur]), DP<R>(c->y[cur]),
        DP<R>(c->z[cur]), DP<R>(c->q[cur]), DP<S4>(c->src), DP<H>(c->M));
    NB_LAUNCHED(c, "p2m");
    c->launches += 1;
    for (int l = c->depth - 1; l >= 0; --l) {
        const int lo = c->level_start[l], hi = c->level_start[l + 1];
        if (hi <= lo) continue;
        k_m2m<MODE, P><<<(unsigned)((hi - lo + 3) / 4), 128, 0, c->st>>>(lo, hi, DP<NodeRec>(c->nodes), box,
                                                                         DP<H>(c->M));
        NB_LAUNCHED(c, "m2m");
        c->launches += 1;
    }
    if (c->timing) cudaEventRecord(c->ev[4], c->st);

    if (!c->lists_frozen) NB_TRY(nb_build_lists(c));
    if (c->timing) cudaEventRecord(c->ev[5], c->st);
    {
        M2LArgs B;
        B.nodes = DP<NodeRec>(c->nodes);
        B.box = box;
        B.Mm2l = c->M.p;
        B.L = c->L.p;
        B.m2l_off = DP<uint32_t>(c->m2l_off); B.m2l_cnt = DP<uint32_t>(c->m2l_cnt);
        B.m2l_list = DP<uint32_t>(c->m2l_list);
        B.eps2 = c->prm.eps * c->prm.eps;
        B.nnodes = nn;
        B.info = DP<int32_t>(c->info);
        B.wait_cycles = c->copy_cycles;
        NB_TRY((dtab_ensure<MODE, P>(c)));
        dtab_args<MODE, P>(c, B);
        constexpr int W = M2LSmem<MODE, P>::warps;
        const size_t smem = (size_t)W * M2LSmem<MODE, P>::per_warp;
        NB_CU(c, cudaFuncSetAttribute(k_m2l<MODE, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_m2l<MODE, P><<<(unsigned)((nn + W - 1) / W), 32 * W, smem, c->st>>>(B);
        NB_LAUNCHED(c, "m2l");
        c->launches += 1;
        for (int r = 1; r <= c->depth; ++r) {
            const int lo = c->level_start[r], hi = c->level_start[r + 1];
            if (hi <= lo) continue;
            k_l2l<MODE, P><<<(unsigned)((hi - lo + 3) / 4), 128, 0, c->st>>>(lo, hi, DP<NodeRec>(c->nodes), box,
                                                                             DP<H>(c->L));
            NB_LAUNCHED(c, "l2l");
            c->launches += 1;
        }
    }
    if (c->timing) cudaEventRecord(c->ev[6], c->st);

    if (integ == NB_INTEG_FAR_ONLY) {
        if (c->timing) cudaEventRecord(c->ev[7], c->st);
        return NBODY_OK;
    }
    const int64_t nl = c->nleaves;
    const int64_t nwork = (uint32_t)c->h_info[INFO_P2P_WORK];
    const int64_t npart = (uint32_t)c->h_info[INFO_P2P_PART];
    NB_TRY(nb_grow(c, c->p2p_part, sizeof(R) * 4 * (size_t)(npart + 1)));
    P2PArgs B;
    B.leaves = DP<uint32_t>(c->leaves);
    B.nleaves = c->nleaves;
    B.nnodes = nn;
    B.n = n;
    B.nodes = DP<NodeRec>(c->nodes);
    B.box = box;
    B.src = c->src.p;
    B.L = c->L.p;
    B.p2p_off = DP<uint32_t>(c->p2p_off); B.p2p_cnt = DP<uint32_t>(c->p2p_cnt); B.p2p_list = DP<uint32_t>(c->p2p_list);
    B.work_off = DP<uint32_t>(c->p2p_work_off);
    B.nwork = nwork;
    B.part_off = DP<uint32_t>(c->p2p_part_off);
    B.part = c->p2p_part.p;
    B.x = c->x[cur].p; B.y = c->y[cur].p; B.z = c->z[cur].p;
    B.vx = c->vx[cur].p; B.vy = c->vy[cur].p; B.vz = c->vz[cur].p;
    B.ax = c->ax[cur].p; B.ay = c->ay[cur].p; B.az = c->az[cur].p;
    B.m = c->m[cur].p; B.q = c->q[cur].p;
    B.pot = want_pot ? c->pot.p : nullptr;
    B.eps2 = c->prm.eps * c->prm.eps;
    B.G = c->prm.G;
    B.dt = c->prm.dt;
    B.integ = integ;
    B.leaf_active = nullptr;
    if (c->blk_s > 0) {
        NB_TRY(nb_block_active_leaves(c));
        B.leaf_active = DP<uint8_t>(c->blk_active);
    }
    const unsigned gf = (unsigned)((nl + P2P_WARPS - 1) / P2P_WARPS);
    {
        const int rc = want_pot ? p2p_launch_classes<MODE, P, true>(c, B) : p2p_launch_classes<MODE, P, false>(c, B);
        if (rc != NBODY_OK) return rc;
    }
    if (npart) {
        if (want_pot) k_p2p_final<MODE, P, true><<<gf, 32 * P2P_WARPS, 0, c->st>>>(B);
        else k_p2p_final<MODE, P, false><<<gf, 32 * P2P_WARPS, 0, c->st>>>(B);
        NB_LAUNCHED(c, "p2p final");
        c->launches += 1;
    }
    if (c->timing) cudaEventRecord(c->ev[7], c->st);
    return NBODY_OK;
}

template <int MODE>
int fmm_dispatch(nbody_ctx* c, int integ, bool want_pot) {
    switch (c->prm.order) {
        case 1: return fmm_forces<MODE, 1>(c, integ, want_pot);
        case 2: return fmm_forces<MODE, 2>(c, integ, want_pot);
        case 3: return fmm_forces<MODE, 3>(c, integ, want_pot);
        case 4: return fmm_forces<MODE, 4>(c, integ, want_pot);
        case 5: return fmm_forces<MODE, 5>(c, integ, want_pot);
        case 6: return fmm_forces<MODE, 6>(c, integ, want_pot);
        case 7: return fmm_forces<MODE, 7>(c, integ, want_pot);
        case 8: return fmm_forces<MODE, 8>(c, integ, want_pot);
        default: return nb_fail(c, NBODY_ERR_INVALID, "order must be 1..8");
    }
}

}  // namespace nbfmm
