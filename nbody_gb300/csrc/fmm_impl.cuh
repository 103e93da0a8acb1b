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
//   k_classify  one tree level per launch: a warp per target cell refines its
//               parent's pending partners (src/interaction.cl:10-100 MAC and
//               split rules) into contiguous per-target far-field, near-field
//               and pending lists; leaf targets descend remaining partners
//               with a per-warp stack;
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
    typedef double H;
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

constexpr int STK = 512;         // descent stack entries per warp
constexpr int CAND = 256;        // expanded candidates per chunk (32 partners x 8 children)
constexpr uint32_t NONE = 0xffffffffu;

__device__ __forceinline__ int mac_accept(long long tcx, long long tcy, long long tcz, long long tw,
                                          const NodeRec& s, double theta2x4) {
    long long sx, sy, sz;
    nb_centre_fine(s, sx, sy, sz);
    long long dx = sx - tcx, dy = sy - tcy, dz = sz - tcz;
    long long d2 = dx * dx + dy * dy + dz * dz;
    long long e = tw + nb_width_fine(s);
    return 3.0 * (double)e * (double)e < theta2x4 * (double)d2;
}

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
                                             typename Prec<MODE>::H* __restrict__ M, float* __restrict__ M32) {
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
            if (M32) M32[(int64_t)k * TM + a] = (float)v;
        }
    }
}

// ---------------------------------------------------------------------------
// M2M: one level, warp per internal node
// ---------------------------------------------------------------------------
template <int MODE, int P>
__global__ void __launch_bounds__(128) k_m2m(int lo, int hi, const NodeRec* __restrict__ nodes,
                                             const BoxDev* __restrict__ boxp, typename Prec<MODE>::H* __restrict__ M,
                                             float* __restrict__ M32) {
    typedef typename Prec<MODE>::H H;
    constexpr int T = nb_terms<P>::value;
    constexpr int TM = nb_tm<P>::value;
    __shared__ H sM[4][T];
    __shared__ H sY[4][T];
    __shared__ H spw[4][3][P + 1];
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
    for (int c = 0; c < nd.nchild; ++c) {
        const int ch = nd.child_begin + c;
        const NodeRec cn = nodes[ch];
        double dx, dy, dz;
        disp(cn, nd, unit, dx, dy, dz);
        for (int a = lane; a < T; a += 32) sM[wib][a] = M[(int64_t)ch * TM + a];
        if (lane < 3) {
            H d = (H)(lane == 0 ? dx : lane == 1 ? dy : dz), p = H(1);
            for (int e = 0; e <= P; ++e) { spw[wib][lane][e] = p; p *= d; }
        }
        __syncwarp();
        for (int a = lane; a < T; a += 32)
            sY[wib][a] = spw[wib][0][nb_mi[a][0]] * spw[wib][1][nb_mi[a][1]] * spw[wib][2][nb_mi[a][2]] *
                         (H)nb_invfact[a];
        __syncwarp();
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            int a = lane + 32 * j;
            if (a < T) {
                H s = acc[j];
                for (int u = st[a]; u < st[a + 1]; ++u) s = nb_fma(sM[wib][pr[2 * u]], sY[wib][pr[2 * u + 1]], s);
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
            if (M32) M32[(int64_t)k * TM + a] = (float)acc[j];
        }
    }
}

// ---------------------------------------------------------------------------
// far field, part 1: interaction lists, one tree level per launch
//
// A warp per target cell t of the level refines the pending partners of its
// parent (src/interaction.cl:10-100 split rules, reorganised per target):
// each candidate s is a child of a pending partner, or the partner itself if
// it is a leaf.  s is accepted for the far field when the MAC holds
// (src/interaction.cl:64-79), kept as a near-field partner when both are
// leaves, kept pending when t has children, and otherwise (t a leaf, s not)
// descended with a per-warp stack.  Two passes: the first counts, one
// atomicAdd per list reserves a contiguous block per target, the second
// writes in the same order.
// ---------------------------------------------------------------------------
template <int MODE, int P>
__global__ void k_root(const NodeRec* __restrict__ nodes, uint32_t* pend_off, uint32_t* pend_cnt,
                       uint32_t* pend_list, uint32_t* p2p_off, uint32_t* p2p_cnt, uint32_t* p2p_list,
                       uint32_t* m2l_off, uint32_t* m2l_cnt, int32_t* info) {
    if (threadIdx.x == 0) {
        const bool leaf = nodes[0].nchild == 0;
        uint32_t* tail = (uint32_t*)&info[leaf ? INFO_P2P_TAIL : INFO_PEND_TAIL];
        uint32_t o = *tail;
        *tail = o + 1;
        if (leaf) { p2p_list[o] = 0; p2p_off[0] = o; p2p_cnt[0] = 1; pend_cnt[0] = 0; }
        else { pend_list[o] = 0; pend_off[0] = o; pend_cnt[0] = 1; p2p_cnt[0] = 0; }
        m2l_off[0] = 0;
        m2l_cnt[0] = 0;
    }
}

struct ClassArgs {
    const NodeRec* nodes;
    uint32_t *pend_off, *pend_cnt, *pend_list, *p2p_off, *p2p_cnt, *p2p_list, *m2l_off, *m2l_cnt, *m2l_list;
    uint32_t pend_cap, p2p_cap, m2l_cap;
    unsigned long long* stats;   // [0] M2L pairs, [1] P2P particle pairs, [2] P2P leaf pairs
    int32_t* info;
    float theta2;                // theta^2 formed in FP32, as the reference does
    int lo, hi;                  // target node range (one level)
};

// centre (2i+1) << (21 - level) in fine units (side / 2^22); fits in 32 bits
__device__ __forceinline__ void centre_fine32(const NodeRec& nd, int& cx, int& cy, int& cz) {
    const int sh = NB_LEVELS - nd.level;
    cx = (int)((2u * nd.ix + 1u) << sh);
    cy = (int)((2u * nd.iy + 1u) << sh);
    cz = (int)((2u * nd.iz + 1u) << sh);
}

// MAC of src/interaction.cl:64-79 in its own FP32 operation order: displacement of centres,
// distance^2 = ((x*x + y*y) + z*z) + w*w with w = 0, extent^2 = (0.75 * (wA+wB)) * (wA+wB),
// approximate iff extent^2 / distance^2 < theta^2 (correctly rounded division).  Lengths are in
// fine units, an exact power-of-two rescaling of the reference's box units, so every rounding is
// the reference's.  The division is only evaluated when a cheap estimate is within 0.1 % of the
// threshold, where it could matter; elsewhere the estimate decides the same way.
__device__ __forceinline__ bool mac_f32(int tcx, int tcy, int tcz, float tw, const NodeRec& s, float theta2) {
    int sx, sy, sz;
    centre_fine32(s, sx, sy, sz);
    const float dx = (float)(sx - tcx), dy = (float)(sy - tcy), dz = (float)(sz - tcz);
    const float d2 = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)), 0.0f);
    const float es = __fadd_rn(tw, (float)(1u << (NB_LEVELS + 1 - s.level)));
    const float e2 = __fmul_rn(__fmul_rn(0.75f, es), es);
    const float est = __fdividef(e2, d2);   // within a few ulp of the quotient
    if (est < 0.999f * theta2) return true;
    if (est > 1.001f * theta2) return false;
    return __fdiv_rn(e2, d2) < theta2;
}

// geometry (level, cell coordinates) of the child in octant oct of a node
struct CellGeom {
    uint32_t ix, iy, iz;
    int level;
};
__device__ __forceinline__ CellGeom child_geom(const CellGeom& p, int oct) {
    return CellGeom{2u * p.ix + (oct & 1), 2u * p.iy + ((oct >> 1) & 1), 2u * p.iz + (oct >> 2), p.level + 1};
}
__device__ __forceinline__ void geom_centre(const CellGeom& g, int& cx, int& cy, int& cz) {
    const int sh = NB_LEVELS - g.level;
    cx = (int)((2u * g.ix + 1u) << sh);
    cy = (int)((2u * g.iy + 1u) << sh);
    cz = (int)((2u * g.iz + 1u) << sh);
}

constexpr int CLS_WARPS = 8;

static __global__ void __launch_bounds__(32 * CLS_WARPS) k_classify(ClassArgs A) {
    __shared__ uint32_t s_cand[CLS_WARPS][CAND];
    __shared__ uint32_t s_stk[CLS_WARPS][STK];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int t = A.lo + blockIdx.x * CLS_WARPS + wib;
    if (t >= A.hi) return;
    uint32_t* cand = s_cand[wib];
    uint32_t* stk = s_stk[wib];
    const NodeRec nt = A.nodes[t];
    const bool tleaf = nt.nchild == 0;
    int tcx, tcy, tcz;
    centre_fine32(nt, tcx, tcy, tcz);
    const float tw = (float)(1u << (NB_LEVELS + 1 - nt.level));
    const int par = nt.parent;
    const uint32_t pb = A.pend_off[par], pc = A.pend_cnt[par];
    uint32_t* out_list = tleaf ? A.p2p_list : A.pend_list;
    uint32_t out_base = 0, n_out = 0, m_base = 0, n_apx = 0;
    bool can_write = false, m_write = false;
    unsigned long long src_particles = 0;

    for (int pass = 0; pass < 2; ++pass) {
        uint32_t wpos = 0, mpos = 0;
        int top = 0;
        auto classify = [&](uint32_t s) {
            const bool valid = s != NONE;
            NodeRec sn;
            sn.nchild = 0;
            sn.count = 0;
            if (valid) sn = A.nodes[s];
            const bool approx = valid && (int)s != t && mac_f32(tcx, tcy, tcz, tw, sn, A.theta2);
            const bool sleaf = valid && sn.nchild == 0;
            const bool out = valid && !approx && (!tleaf || sleaf);
            const bool desc = valid && !approx && tleaf && !sleaf;
            const uint32_t mo = __ballot_sync(0xffffffffu, out);
            if (out && pass == 1 && can_write) {
                const uint32_t pos = wpos + __popc(mo & lanemask_lt());
                if (pos < n_out) out_list[out_base + pos] = s;
                if (tleaf) src_particles += sn.count;
            }
            wpos += __popc(mo);
            const uint32_t ma = __ballot_sync(0xffffffffu, approx);
            if (approx && pass == 1 && m_write) {
                const uint32_t pos = mpos + __popc(ma & lanemask_lt());
                if (pos < n_apx) A.m2l_list[m_base + pos] = s;
            }
            mpos += __popc(ma);
            const uint32_t md = __ballot_sync(0xffffffffu, desc);
            if (desc) {
                const int pos = top + __popc(md & lanemask_lt());
                if (pos < STK) stk[pos] = s;
                else atomicOr((unsigned int*)&A.info[INFO_ERR], NB_ERRBIT_STACK);
            }
            top = min(top + __popc(md), STK);
        };
        auto drain_stack = [&]() {
            while (top > 0) {
                const int kk = min(top, 4);
                const int qn = lane >> 3, ci = lane & 7;
                uint32_t s2 = NONE;
                if (qn < kk) {
                    const NodeRec pn = A.nodes[stk[top - 1 - qn]];
                    if (ci < pn.nchild) s2 = (uint32_t)(pn.child_begin + ci);
                }
                __syncwarp();
                top -= kk;
                classify(s2);
                __syncwarp();
            }
        };
        for (uint32_t chunk = 0; chunk < pc; chunk += 32) {
            const uint32_t j = chunk + lane;
            uint32_t s = NONE, ns = 0;
            NodeRec sn;
            sn.nchild = 0;
            sn.child_begin = 0;
            if (j < pc) {
                s = A.pend_list[pb + j];
                sn = A.nodes[s];
                ns = sn.nchild ? sn.nchild : 1u;
            }
            const uint32_t inc = warp_incl_scan(ns);
            const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
            const uint32_t ex = inc - ns;
            if (ns == 1 && sn.nchild == 0) cand[ex] = s;
            else
                for (uint32_t u = 0; u < ns; ++u) cand[ex + u] = (uint32_t)(sn.child_begin + u);
            __syncwarp();
            for (uint32_t g = 0; g < total; g += 32) {
                const uint32_t s2 = g + lane < total ? cand[g + lane] : NONE;
                classify(s2);
            }
            __syncwarp();
            drain_stack();
        }
        if (pass == 0) {
            n_out = wpos;
            n_apx = mpos;
            uint32_t base = 0, mb = 0;
            int ok = 0, mok = 0;
            if (lane == 0) {
                uint32_t* tail = (uint32_t*)&A.info[tleaf ? INFO_P2P_TAIL : INFO_PEND_TAIL];
                const uint32_t cap = tleaf ? A.p2p_cap : A.pend_cap;
                base = atomicAdd(tail, n_out);
                ok = (uint64_t)base + n_out <= cap;
                if (!ok) atomicOr((unsigned int*)&A.info[INFO_ERR], tleaf ? NB_ERRBIT_P2P_CAP : NB_ERRBIT_PEND_CAP);
                mb = atomicAdd((uint32_t*)&A.info[INFO_M2L_TAIL], n_apx);
                mok = (uint64_t)mb + n_apx <= A.m2l_cap;
                if (!mok) atomicOr((unsigned int*)&A.info[INFO_ERR], NB_ERRBIT_M2L_CAP);
                if (tleaf) {
                    A.p2p_off[t] = base; A.p2p_cnt[t] = ok ? n_out : 0;
                    A.pend_cnt[t] = 0;
                } else {
                    A.pend_off[t] = base; A.pend_cnt[t] = ok ? n_out : 0;
                    A.p2p_cnt[t] = 0;
                }
                A.m2l_off[t] = mb;
                A.m2l_cnt[t] = mok ? n_apx : 0;
            }
            out_base = __shfl_sync(0xffffffffu, base, 0);
            can_write = __shfl_sync(0xffffffffu, ok, 0);
            m_base = __shfl_sync(0xffffffffu, mb, 0);
            m_write = __shfl_sync(0xffffffffu, mok, 0);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) src_particles += __shfl_xor_sync(0xffffffffu, src_particles, o);
    if (lane == 0) {
        atomicAdd(&A.stats[0], (unsigned long long)n_apx);
        if (tleaf) {
            atomicAdd(&A.stats[1], src_particles * nt.count);
            atomicAdd(&A.stats[2], (unsigned long long)n_out);
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
};

template <int MODE, int P>
struct M2LSmem {
    typedef typename Prec<MODE>::S S;
    static constexpr int T = nb_terms<P>::value;
    static constexpr int TM = nb_tm<P>::value;
    // 16-byte chunks per shared row must be odd: the 8 lanes of a quarter warp then read 8 distinct bank groups
    static constexpr int SST = sizeof(S) == 4 ? ((TM / 4) % 2 ? TM : TM + 4) : TM + 2;
    static constexpr int warps = Prec<MODE>::lane_smem ? 1 : 4;
    static constexpr size_t rows = (size_t)2 * 32 * SST * sizeof(S);
    static constexpr size_t lane_arrays = Prec<MODE>::lane_smem ? (size_t)2 * 32 * T * sizeof(S) : 0;
    static constexpr size_t per_warp = (16 + rows + lane_arrays + 255) / 256 * 256;
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
// warp-uniform bounded wait (about a second at GB300 clocks); false on timeout
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    bool ok = false;
    for (;;) {
        ok = ok || mbar_try_wait(bar, parity);
        if (__all_sync(0xffffffffu, ok)) return true;
        const long long dt = __shfl_sync(0xffffffffu, clock64() - t0, 0);
        if (dt > 2000000000ll) return false;
    }
}

template <int MODE, int P>
__global__ void __launch_bounds__(32 * M2LSmem<MODE, P>::warps) k_m2l(M2LArgs A) {
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
    // issue the bulk copies of batch b into stage b & 1; returns this lane's source
    auto issue = [&](uint32_t b) -> uint32_t {
        const uint32_t nb = min(32u, cnt - 32 * b);
        const uint32_t k = b & 1;
        const uint32_t s = (uint32_t)lane < nb ? A.m2l_list[off + 32 * b + lane] : 0u;
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) mbar_expect_tx(&bar[k], nb * ROWB);
        __syncwarp();
        if ((uint32_t)lane < nb) bulk_g2s(rows + (k * 32 + lane) * SST, Msrc + (int64_t)s * TM, ROWB, &bar[k]);
        return s;
    };
    bool failed = false;
    uint32_t b_fail = 0;
    uint32_t s_next = nbatch ? issue(0) : 0u;
    for (uint32_t b = 0; b < nbatch; ++b) {
        const uint32_t s_cur = s_next;
        const uint32_t k = b & 1;
        const uint32_t nb = min(32u, cnt - 32 * b);
        if (b + 1 < nbatch) s_next = issue(b + 1);
        if (!mbar_wait_warp(&bar[k], (b >> 1) & 1)) { failed = true; b_fail = b; break; }
        if ((uint32_t)lane < nb) {
            const NodeRec sn = A.nodes[s_cur];
            int sx, sy, sz;
            centre_fine32(sn, sx, sy, sz);
            const S dx = (S)(tcx - sx) * unit, dy = (S)(tcy - sy) * unit, dz = (S)(tcz - sz) * unit;
            const S* row = rows + (k * 32 + lane) * SST;
            if constexpr (LS) {
                Ops<S, P>::template derivs<32>(dx, dy, dz, eps2, laneD + lane);
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
        // let every copy already issued land before the shared memory is released
        if (lane == 0) atomicOr((unsigned int*)&A.info[INFO_ERR], NB_ERRBIT_ASYNC);
        mbar_wait_warp(&bar[b_fail & 1], (b_fail >> 1) & 1);
        if (b_fail + 1 < nbatch) mbar_wait_warp(&bar[(b_fail + 1) & 1], ((b_fail + 1) >> 1) & 1);
        return;
    }
    H* Lg = (H*)A.L;
#pragma unroll
    for (int a = 0; a < T; ++a) {
        S v;
        if constexpr (LS) v = laneL[a * 32 + lane];
        else v = Lreg[a];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += shfl_xor_t(v, o);
        if ((a & 31) == lane) Lg[t * T + a] = (H)v;
    }
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
constexpr int P2P_CHUNK = 256;    // partner leaves per work item

static __global__ void k_p2p_plan(int64_t nleaves, const uint32_t* __restrict__ leaves, const NodeRec* __restrict__ nodes,
                           const uint32_t* __restrict__ p2p_cnt, uint32_t* __restrict__ nch,
                           uint32_t* __restrict__ psize) {
    const int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (li > nleaves) return;
    if (li == nleaves) { nch[li] = 0; psize[li] = 0; return; }
    const uint32_t k = leaves[li];
    const uint32_t c = (p2p_cnt[k] + P2P_CHUNK - 1) / P2P_CHUNK;
    const uint32_t n = c > 1 ? c : 1u;
    nch[li] = n;
    psize[li] = n > 1 ? n * nodes[k].count : 0u;
}

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

// One warp's share of a near-field work item: every target of the leaf
// (two per lane, CT lanes per group) against the partner leaves
// [s_lo, s_hi) of its list.  GUARD: unsoftened kernel, so r = 0 must give 0.
template <int MODE, int P, bool POT, bool GUARD>
__device__ __forceinline__ void p2p_item(const P2PArgs& A, typename Prec<MODE>::S4 (*tile)[P2P_TILE],
                                         const typename Prec<MODE>::S* sL, uint32_t k, const NodeRec& nt,
                                         int64_t li, uint32_t chunk, uint32_t nchunk, uint32_t s_lo,
                                         uint32_t s_hi) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::S4 S4;
    constexpr bool KH = Prec<MODE>::kahan;
    const int lane = lane_id();
    const double unit = A.box->unit;
    const S4* src = (const S4*)A.src;
    const uint32_t cnt_t = nt.count;
    const int CT = cnt_t <= 16 ? 8 : cnt_t <= 32 ? 16 : 32;
    const int NG = 32 / CT, grp = lane / CT, gl = lane % CT, TPL = P2P_TILE / CT;
    const uint32_t loff = A.p2p_off[k];
    const S eps2 = (S)A.eps2;
    S4 zero4;
    zero4.x = 0; zero4.y = 0; zero4.z = 0; zero4.w = 0;
    for (uint32_t tc = 0; tc < cnt_t; tc += 2 * CT) {
        const uint32_t ta = tc + gl, tb = tc + CT + gl;
        const bool va = ta < cnt_t, vb = tb < cnt_t;
        const uint32_t ia = nt.begin + (va ? ta : 0), ib = nt.begin + (vb ? tb : 0);
        const S4 ya = src[ia], yb = src[ib];
        S ax = 0, ay = 0, az = 0, ap = 0, bx = 0, by = 0, bz = 0, bp = 0;
        S cax = 0, cay = 0, caz = 0, cap = 0, cbx = 0, cby = 0, cbz = 0, cbp = 0;
        for (uint32_t base = s_lo; base < s_hi; base += 32) {
            const uint32_t nb = min(32u, s_hi - base);
            uint32_t my_s = 0, my_beg = 0, my_cnt = 0;
            S my_dx = 0, my_dy = 0, my_dz = 0;
            if ((uint32_t)lane < nb) {
                my_s = A.p2p_list[loff + base + lane];
                const NodeRec sn = A.nodes[my_s];
                my_beg = sn.begin;
                my_cnt = sn.count;
                double ddx, ddy, ddz;
                disp(sn, nt, unit, ddx, ddy, ddz);
                my_dx = (S)ddx; my_dy = (S)ddy; my_dz = (S)ddz;
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
            const uint32_t cur_beg = __shfl_sync(0xffffffffu, my_beg, grp);
            const uint32_t cur_cnt0 = __shfl_sync(0xffffffffu, my_cnt, grp);
            const uint32_t cur_cnt = (uint32_t)grp < nb ? cur_cnt0 : 0u;
            S4 pre[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const uint32_t j = sb + gl + e * CT;
                pre[e] = (e < TPL && j < cur_cnt) ? src[cur_beg + j] : zero4;
            }
            while (rr < rounds) {
                const uint32_t q = rr * NG + grp;
                const uint32_t qs = q & 31;
                const uint32_t s_id = __shfl_sync(0xffffffffu, my_s, qs);
                const S dx = __shfl_sync(0xffffffffu, my_dx, qs), dy = __shfl_sync(0xffffffffu, my_dy, qs),
                        dz = __shfl_sync(0xffffffffu, my_dz, qs);
                const uint32_t scnt0 = __shfl_sync(0xffffffffu, my_cnt, qs);
                const uint32_t scnt = q < nb ? scnt0 : 0u;
                uint32_t mx = scnt;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (e < TPL) tile[grp][gl + e * CT] = pre[e];
                __syncwarp();
                uint32_t nrr = rr, nsb = sb + P2P_TILE;
                if (nsb >= mx) { nrr = rr + 1; nsb = 0; }
                {
                    const uint32_t nq = nrr * NG + grp;
                    const uint32_t nbeg = __shfl_sync(0xffffffffu, my_beg, nq & 31);
                    const uint32_t ncnt0 = __shfl_sync(0xffffffffu, my_cnt, nq & 31);
                    const uint32_t ncnt = (nrr < rounds && nq < nb) ? ncnt0 : 0u;
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const uint32_t j = nsb + gl + e * CT;
                        pre[e] = (e < TPL && j < ncnt) ? src[nbeg + j] : zero4;
                    }
                }
                // both targets, shifted into the source leaf's frame
                const S xa = ya.x - dx, ya_ = ya.y - dy, za = ya.z - dz;
                const S xb = yb.x - dx, yb_ = yb.y - dy, zb = yb.z - dz;
                const int nj = scnt > sb ? min((int)(scnt - sb), P2P_TILE) : 0;
                S pax = 0, pay = 0, paz = 0, pap = 0, pbx = 0, pby = 0, pbz = 0, pbp = 0;
#pragma unroll 2
                for (int e = 0; e < nj; ++e) {
                    const S4 sj = tile[grp][e];
                    const S rxa = sj.x - xa, rya = sj.y - ya_, rza = sj.z - za;
                    const S rxb = sj.x - xb, ryb = sj.y - yb_, rzb = sj.z - zb;
                    S s2a = nb_fma(rxa, rxa, nb_fma(rya, rya, nb_fma(rza, rza, eps2)));
                    S s2b = nb_fma(rxb, rxb, nb_fma(ryb, ryb, nb_fma(rzb, rzb, eps2)));
                    if (GUARD) { s2a = s2a > S(0) ? s2a : S(1e30); s2b = s2b > S(0) ? s2b : S(1e30); }
                    S inva = nb_rsqrt(s2a), invb = nb_rsqrt(s2b);
                    if (POT && s_id == k && sb + e == ta) inva = S(0);
                    if (POT && s_id == k && sb + e == tb) invb = S(0);
                    const S wa = sj.w * inva * inva * inva, wb = sj.w * invb * invb * invb;
                    pax = nb_fma(rxa, wa, pax); pay = nb_fma(rya, wa, pay); paz = nb_fma(rza, wa, paz);
                    pbx = nb_fma(rxb, wb, pbx); pby = nb_fma(ryb, wb, pby); pbz = nb_fma(rzb, wb, pbz);
                    if (POT) { pap = nb_fma(sj.w, inva, pap); pbp = nb_fma(sj.w, invb, pbp); }
                }
                if (KH) {
                    kahan_add(ax, cax, pax); kahan_add(ay, cay, pay); kahan_add(az, caz, paz);
                    kahan_add(bx, cbx, pbx); kahan_add(by, cby, pby); kahan_add(bz, cbz, pbz);
                    if (POT) { kahan_add(ap, cap, pap); kahan_add(bp, cbp, pbp); }
                } else {
                    ax += pax; ay += pay; az += paz; bx += pbx; by += pby; bz += pbz;
                    if (POT) { ap += pap; bp += pbp; }
                }
                __syncwarp();
                rr = nrr;
                sb = nsb;
            }
        }
        // combine the source groups in a fixed order, in the state precision
        R Ax = (R)ax - (R)cax, Ay = (R)ay - (R)cay, Az = (R)az - (R)caz, Ap = (R)ap - (R)cap;
        R Bx = (R)bx - (R)cbx, By = (R)by - (R)cby, Bz = (R)bz - (R)cbz, Bp = (R)bp - (R)cbp;
        for (int o = CT; o < 32; o <<= 1) {
            Ax += shfl_xor_t(Ax, o); Ay += shfl_xor_t(Ay, o); Az += shfl_xor_t(Az, o);
            Bx += shfl_xor_t(Bx, o); By += shfl_xor_t(By, o); Bz += shfl_xor_t(Bz, o);
            if (POT) { Ap += shfl_xor_t(Ap, o); Bp += shfl_xor_t(Bp, o); }
        }
        if (grp == 0) {
            if (nchunk == 1) {
                if (va) p2p_epilogue<MODE, P>(A, ia, sL, ya, Ax, Ay, Az, Ap, POT);
                if (vb) p2p_epilogue<MODE, P>(A, ib, sL, yb, Bx, By, Bz, Bp, POT);
            } else {
                R* pt = (R*)A.part + 4 * ((int64_t)A.part_off[li] + (int64_t)chunk * cnt_t);
                if (va) { pt[4 * ta] = Ax; pt[4 * ta + 1] = Ay; pt[4 * ta + 2] = Az; pt[4 * ta + 3] = Ap; }
                if (vb) { pt[4 * tb] = Bx; pt[4 * tb + 1] = By; pt[4 * tb + 2] = Bz; pt[4 * tb + 3] = Bp; }
            }
        }
        __syncwarp();
    }
}

template <int MODE, int P, bool POT>
__global__ void __launch_bounds__(32 * P2P_WARPS, 5) k_p2p(P2PArgs A) {
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    typedef typename Prec<MODE>::S4 S4;
    constexpr int T = nb_terms<P>::value;
    __shared__ S4 tile[P2P_WARPS][4][P2P_TILE];
    __shared__ S sL[P2P_WARPS][T];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * P2P_WARPS + wib;
    if (w >= A.nwork) return;
    // which leaf / chunk: last li with work_off[li] <= w
    int64_t lo = 0, hi = A.nleaves;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (A.work_off[mid] <= (uint32_t)w) lo = mid; else hi = mid;
    }
    const int64_t li = lo;
    const uint32_t chunk = (uint32_t)w - A.work_off[li];
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
    if (A.eps2 > 0.0) p2p_item<MODE, P, POT, false>(A, tile[wib], sL[wib], k, nt, li, chunk, nchunk, s_lo, s_hi);
    else p2p_item<MODE, P, POT, true>(A, tile[wib], sL[wib], k, nt, li, chunk, nchunk, s_lo, s_hi);
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
    if (MODE == NBODY_PREC_MIXED) NB_TRY(nb_grow(c, c->M32, sizeof(float) * TM * nn));
    NB_TRY(nb_grow(c, c->L, sizeof(H) * T * nn));
    NB_TRY(nb_grow(c, c->src, sizeof(S4) * n));
    NB_TRY(nb_grow(c, c->pend_off, sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->pend_cnt, sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->p2p_off, sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->p2p_cnt, sizeof(uint32_t) * nn));
    float* M32 = MODE == NBODY_PREC_MIXED ? DP<float>(c->M32) : nullptr;
    const BoxDev* box = DP<BoxDev>(c->box);

    if (c->timing) cudaEventRecord(c->ev[3], c->st);
    k_p2m<MODE, P><<<(unsigned)((c->nleaves + 3) / 4), 128, 0, c->st>>>(
        c->nleaves, DP<uint32_t>(c->leaves), DP<NodeRec>(c->nodes), box, DP<R>(c->x[cur]), DP<R>(c->y[cur]),
        DP<R>(c->z[cur]), DP<R>(c->q[cur]), DP<S4>(c->src), DP<H>(c->M), M32);
    NB_LAUNCHED(c, "p2m");
    c->launches += 1;
    for (int l = c->depth - 1; l >= 0; --l) {
        const int lo = c->level_start[l], hi = c->level_start[l + 1];
        if (hi <= lo) continue;
        k_m2m<MODE, P><<<(unsigned)((hi - lo + 3) / 4), 128, 0, c->st>>>(lo, hi, DP<NodeRec>(c->nodes), box,
                                                                         DP<H>(c->M), M32);
        NB_LAUNCHED(c, "m2m");
        c->launches += 1;
    }
    if (c->timing) cudaEventRecord(c->ev[4], c->st);

    NB_TRY(nb_grow(c, c->m2l_off, sizeof(uint32_t) * nn));
    NB_TRY(nb_grow(c, c->m2l_cnt, sizeof(uint32_t) * nn));
    for (int attempt = 0; attempt < 8; ++attempt) {
        size_t want_pend = (size_t)64 * nn + 1024, want_p2p = (size_t)96 * c->nleaves + 1024;
        size_t want_m2l = (size_t)512 * nn + 1024;
        if (c->pend_cap < want_pend) c->pend_cap = want_pend;
        if (c->p2p_cap < want_p2p) c->p2p_cap = want_p2p;
        if (c->m2l_cap < want_m2l) c->m2l_cap = want_m2l;
        c->pend_cap = std::min<size_t>(c->pend_cap, 0xffffffffu);
        c->p2p_cap = std::min<size_t>(c->p2p_cap, 0xffffffffu);
        c->m2l_cap = std::min<size_t>(c->m2l_cap, 0xffffffffu);
        NB_TRY(nb_grow(c, c->pend_list, sizeof(uint32_t) * c->pend_cap));
        NB_TRY(nb_grow(c, c->p2p_list, sizeof(uint32_t) * c->p2p_cap));
        NB_TRY(nb_grow(c, c->m2l_list, sizeof(uint32_t) * c->m2l_cap));
        int32_t* info = DP<int32_t>(c->info);
        NB_TRY(nb_grow(c, c->stats, 8 * sizeof(unsigned long long)));
        NB_CU(c, cudaMemsetAsync(c->stats.p, 0, 8 * sizeof(unsigned long long), c->st));
        NB_CU(c, cudaMemsetAsync(info + INFO_PEND_TAIL, 0, 3 * sizeof(int32_t), c->st));
        NB_CU(c, cudaMemsetAsync(info + INFO_ERR, 0, sizeof(int32_t), c->st));
        k_root<MODE, P><<<1, 32, 0, c->st>>>(DP<NodeRec>(c->nodes), DP<uint32_t>(c->pend_off),
                                             DP<uint32_t>(c->pend_cnt), DP<uint32_t>(c->pend_list),
                                             DP<uint32_t>(c->p2p_off), DP<uint32_t>(c->p2p_cnt),
                                             DP<uint32_t>(c->p2p_list), DP<uint32_t>(c->m2l_off),
                                             DP<uint32_t>(c->m2l_cnt), info);
        NB_LAUNCHED(c, "root");
        c->launches += 1;
        ClassArgs A;
        A.nodes = DP<NodeRec>(c->nodes);
        A.pend_off = DP<uint32_t>(c->pend_off); A.pend_cnt = DP<uint32_t>(c->pend_cnt);
        A.pend_list = DP<uint32_t>(c->pend_list);
        A.p2p_off = DP<uint32_t>(c->p2p_off); A.p2p_cnt = DP<uint32_t>(c->p2p_cnt);
        A.p2p_list = DP<uint32_t>(c->p2p_list);
        A.m2l_off = DP<uint32_t>(c->m2l_off); A.m2l_cnt = DP<uint32_t>(c->m2l_cnt);
        A.m2l_list = DP<uint32_t>(c->m2l_list);
        A.pend_cap = (uint32_t)c->pend_cap; A.p2p_cap = (uint32_t)c->p2p_cap; A.m2l_cap = (uint32_t)c->m2l_cap;
        A.stats = DP<unsigned long long>(c->stats);
        A.info = info;
        const float th = (float)c->prm.theta;
        A.theta2 = th * th;
        for (int r = 1; r <= c->depth; ++r) {
            A.lo = c->level_start[r];
            A.hi = c->level_start[r + 1];
            if (A.hi <= A.lo) continue;
            k_classify<<<(unsigned)((A.hi - A.lo + CLS_WARPS - 1) / CLS_WARPS), 32 * CLS_WARPS, 0, c->st>>>(A);
            NB_LAUNCHED(c, "classify");
            c->launches += 1;
        }
        // near-field work plan: chunks per leaf and partial-sum slots, scanned
        {
            const int64_t nl = c->nleaves;
            NB_TRY(nb_grow(c, c->p2p_nch, sizeof(uint32_t) * (nl + 1)));
            NB_TRY(nb_grow(c, c->p2p_work_off, sizeof(uint32_t) * (nl + 1)));
            NB_TRY(nb_grow(c, c->p2p_psize, sizeof(uint32_t) * (nl + 1)));
            NB_TRY(nb_grow(c, c->p2p_part_off, sizeof(uint32_t) * (nl + 1)));
            k_p2p_plan<<<(unsigned)((nl + 1 + 255) / 256), 256, 0, c->st>>>(
                nl, DP<uint32_t>(c->leaves), DP<NodeRec>(c->nodes), DP<uint32_t>(c->p2p_cnt), DP<uint32_t>(c->p2p_nch),
                DP<uint32_t>(c->p2p_psize));
            NB_LAUNCHED(c, "p2p_plan");
            c->launches += 1;
            NB_TRY(nb_scan_u32(c, DP<uint32_t>(c->p2p_nch), DP<uint32_t>(c->p2p_work_off), nl + 1,
                               (uint32_t*)(info + INFO_P2P_WORK)));
            NB_TRY(nb_scan_u32(c, DP<uint32_t>(c->p2p_psize), DP<uint32_t>(c->p2p_part_off), nl + 1,
                               (uint32_t*)(info + INFO_P2P_PART)));
        }
        NB_CU(c, cudaMemcpyAsync(c->h_info, info, sizeof(int32_t) * INFO_WORDS, cudaMemcpyDeviceToHost, c->st));
        NB_CU(c, cudaMemcpyAsync(c->h_stats, c->stats.p, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 c->st));
        NB_CU(c, cudaStreamSynchronize(c->st));
        const uint32_t e = (uint32_t)c->h_info[INFO_ERR];
        if (e & NB_ERRBIT_STACK) return nb_fail(c, NBODY_ERR_CAPACITY, "traversal descent stack overflow");
        if (!(e & (NB_ERRBIT_PEND_CAP | NB_ERRBIT_P2P_CAP | NB_ERRBIT_M2L_CAP))) break;
        if (e & NB_ERRBIT_M2L_CAP)
            c->m2l_cap = std::max<size_t>(2 * c->m2l_cap, (size_t)(uint32_t)c->h_info[INFO_M2L_TAIL] + 1024);
        if (e & NB_ERRBIT_PEND_CAP)
            c->pend_cap = std::max<size_t>(2 * c->pend_cap, (size_t)(uint32_t)c->h_info[INFO_PEND_TAIL] + 1024);
        if (e & NB_ERRBIT_P2P_CAP)
            c->p2p_cap = std::max<size_t>(2 * c->p2p_cap, (size_t)(uint32_t)c->h_info[INFO_P2P_TAIL] + 1024);
        if (attempt == 7) return nb_fail(c, NBODY_ERR_CAPACITY, "interaction lists kept overflowing");
    }
    if (c->timing) cudaEventRecord(c->ev[5], c->st);
    {
        M2LArgs B;
        B.nodes = DP<NodeRec>(c->nodes);
        B.box = box;
        B.Mm2l = MODE == NBODY_PREC_MIXED ? (const void*)M32 : (const void*)c->M.p;
        B.L = c->L.p;
        B.m2l_off = DP<uint32_t>(c->m2l_off); B.m2l_cnt = DP<uint32_t>(c->m2l_cnt);
        B.m2l_list = DP<uint32_t>(c->m2l_list);
        B.eps2 = c->prm.eps * c->prm.eps;
        B.nnodes = nn;
        B.info = DP<int32_t>(c->info);
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
    const unsigned g = (unsigned)((nwork + P2P_WARPS - 1) / P2P_WARPS);
    const unsigned gf = (unsigned)((nl + P2P_WARPS - 1) / P2P_WARPS);
    if (want_pot) {
        k_p2p<MODE, P, true><<<g, 32 * P2P_WARPS, 0, c->st>>>(B);
        if (npart) k_p2p_final<MODE, P, true><<<gf, 32 * P2P_WARPS, 0, c->st>>>(B);
    } else {
        k_p2p<MODE, P, false><<<g, 32 * P2P_WARPS, 0, c->st>>>(B);
        if (npart) k_p2p_final<MODE, P, false><<<gf, 32 * P2P_WARPS, 0, c->st>>>(B);
    }
    NB_LAUNCHED(c, "p2p");
    c->launches += npart ? 2 : 1;
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
