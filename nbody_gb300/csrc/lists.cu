// Interaction lists of the step: far-field (M2L) and near-field (P2P) lists
// of every cell, built breadth first.  Replaces the interaction finding of
// src/interaction.cl:10-100 (same acceptance test and split rules,
// reorganised per target; the resulting pair sets are the reference's).
//
// Level r = 1 .. depth processes the active targets of the level: every node
// at level r, with the pending partners of its parent as input, and every
// leaf above level r that still has pending partners of its own.  A
// candidate is a child of an input partner, or the partner itself if it is a
// leaf.  The candidate s of target t goes to
//   the far-field list      if the MAC holds (and s != t),
//   the near-field list     if t and s are leaves,
//   t's pending list        otherwise (t internal: refined by t's children at
//                           level r+1; t a leaf: refined by t itself at r+1).
// Work is split into items (target, chunk of 32 input partners) so a target
// with a long input list (a large sparse leaf next to a dense region) is
// spread over many warps.  Each level classifies every candidate once into a
// per-item staging row, scans the per-item counts, and scatters the rows, so
// every target's output of the level is one contiguous block in a fixed order;
// a final pass concatenates each target's blocks in level order into the
// per-target lists the far- and near-field kernels read.  Nothing depends on
// scheduling: the lists are bitwise reproducible.
#include <algorithm>

#include "nbody_internal.cuh"

namespace {

constexpr uint32_t NONE = 0xffffffffu;
constexpr int LW = 8;                 // warps per block of the item kernels
constexpr int CANDS = 256;            // candidates of one item (32 partners x 8 children)

struct LevelArgs {
    const NodeRec* nodes;
    int r, hi, nn;
    float theta2;
    const uint32_t *pin_off, *pin_cnt, *pin_list;     // pending input (level r - 1)
    uint32_t *pout_off, *pout_cnt, *pout_list;        // pending output (level r)
    uint32_t pend_cap;
    uint32_t *nch, *first;                            // per target: chunks (items), first item
    uint4* item;                                      // per item: target, input offset, input count, chunks
                                                      // of the target (first item only, else 0)
    uint32_t item_cap;
    uint32_t* cnt[3];                                 // per item: far, near, pending outputs
    uint32_t* off[3];                                 // their exclusive scans
    uint32_t *m2l_stage, *p2p_stage;
    uint32_t m2l_cap, p2p_cap;
    uint32_t *m2l_soff, *m2l_scnt, *p2p_soff, *p2p_scnt;   // rows of level r
    uint32_t* rows;                                   // per item: its classified candidates (CANDS each)
    int32_t* info;
    unsigned long long* stats;
};

__device__ __forceinline__ bool active_target(const NodeRec& nd, int r) {
    return nd.level == r || (nd.nchild == 0 && nd.level < r);
}

// pending input of an active target: its parent's (a node of this level) or its own (a carried leaf)
__device__ __forceinline__ void target_input(const LevelArgs& A, uint32_t t, const NodeRec& nd, uint32_t& off,
                                             uint32_t& cnt) {
    const uint32_t src = nd.level == A.r ? (uint32_t)nd.parent : t;
    off = A.pin_off[src];
    cnt = A.pin_cnt[src];
}

constexpr uint32_t LIST_CAP_BITS = NB_ERRBIT_PEND_CAP | NB_ERRBIT_P2P_CAP | NB_ERRBIT_M2L_CAP | NB_ERRBIT_ITEM_CAP;

// after a capacity overflow the offsets of the failed level can point past the buffers: later
// levels and the concatenation then do nothing (the host retries with larger capacities)
__device__ __forceinline__ bool lists_failed(const int32_t* info) {
    return ((uint32_t)*(volatile const int32_t*)&info[INFO_ERR] & LIST_CAP_BITS) != 0;
}

__global__ void k_lv_plan(LevelArgs A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool failed = lists_failed(A.info);
    if (t == 0) {
        // running bases of the staged lists: add the previous level's totals
        A.info[INFO_BASE_M2L] += A.info[INFO_LVL_M2L];
        A.info[INFO_BASE_P2P] += A.info[INFO_LVL_P2P];
    }
    if (t > A.hi) return;
    if (t == A.hi) { A.nch[t] = 0; return; }
    const NodeRec nd = A.nodes[t];
    uint32_t n = 0;
    if (!failed && active_target(nd, A.r)) {
        uint32_t off, cnt;
        target_input(A, t, nd, off, cnt);
        n = (cnt + 31) / 32;
    }
    A.nch[t] = n;
    A.pout_cnt[t] = 0;
    A.m2l_scnt[t] = 0;
    A.p2p_scnt[t] = 0;
}

// the item records of every active target: one item per chunk of 32 input partners, so the item
// kernels start from one 16-byte load instead of a chain of dependent ones
__global__ void k_lv_fill(LevelArgs A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.hi) return;
    const uint32_t n = A.nch[t], f = A.first[t];
    if (n == 0) return;
    if ((uint64_t)f + n > A.item_cap) {
        atomicOr((unsigned int*)&A.info[INFO_ERR], NB_ERRBIT_ITEM_CAP);
        return;
    }
    uint32_t off, cnt;
    target_input(A, (uint32_t)t, A.nodes[t], off, cnt);
    for (uint32_t c = 0; c < n; ++c)
        A.item[f + c] = make_uint4((uint32_t)t, off + 32 * c, min(32u, cnt - 32 * c), c == 0 ? n : 0u);
}

// Classifies the candidates of item i once: each goes to row i of the staging table (candidate
// order, class in the top two bits: 1 far field, 2 near field, 3 pending) and the item's three
// counts are kept for the scans; k_lv_scatter then places the row's entries.
constexpr int CLS_UNROLL = 4;         // candidate groups of 32 whose node records are loaded together

__device__ void lv_classify(const LevelArgs& A, uint32_t i, uint32_t* cand) {
    const int lane = lane_id();
    const uint4 it = A.item[i];
    const uint32_t t = it.x;
    uint32_t s = NONE, ns = 0, cb = 0;
    if ((uint32_t)lane < it.z) s = NB_IDX(A.pin_list[it.y + lane], A.nn, NB_SITE_LISTS);
    const NodeRec nt = A.nodes[t];
    if (s != NONE) {
        const NodeRec sn = A.nodes[s];
        ns = sn.nchild ? sn.nchild : 1u;
        cb = sn.nchild ? (uint32_t)sn.child_begin : s;
    }
    const bool tleaf = nt.nchild == 0;
    int tcx, tcy, tcz;
    centre_fine32(nt, tcx, tcy, tcz);
    const float tw = (float)(1u << (NB_LEVELS + 1 - nt.level));
    const uint32_t inc = warp_incl_scan(ns);
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    for (uint32_t u = 0; u < ns; ++u) cand[inc - ns + u] = cb + u;
    __syncwarp();
    uint32_t* row = A.rows + (size_t)i * CANDS;
    uint32_t nm = 0, np = 0, nq = 0;
    unsigned long long near_particles = 0;
    for (uint32_t g0 = 0; g0 < total; g0 += 32 * CLS_UNROLL) {
        uint32_t sc[CLS_UNROLL];
        NodeRec sn[CLS_UNROLL];
#pragma unroll
        for (int u = 0; u < CLS_UNROLL; ++u) {
            const uint32_t g = g0 + 32 * u + lane;
            sc[u] = g < total ? cand[g] : NONE;
            sn[u].nchild = 0;
            sn[u].count = 0;
            if (sc[u] != NONE) sn[u] = A.nodes[NB_IDX(sc[u], A.nn, NB_SITE_LISTS)];
        }
#pragma unroll
        for (int u = 0; u < CLS_UNROLL; ++u) {
            const bool valid = sc[u] != NONE;
            const bool approx = valid && sc[u] != t && mac_f32(tcx, tcy, tcz, tw, sn[u], A.theta2);
            const bool sleaf = valid && sn[u].nchild == 0;
            const bool near = valid && !approx && tleaf && sleaf;
            const bool pend = valid && !approx && !near;
            if (valid) row[g0 + 32 * u + lane] = sc[u] | ((approx ? 1u : near ? 2u : 3u) << 30);
            if (near) near_particles += sn[u].count;
            nm += __popc(__ballot_sync(0xffffffffu, approx));
            np += __popc(__ballot_sync(0xffffffffu, near));
            nq += __popc(__ballot_sync(0xffffffffu, pend));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) near_particles += __shfl_xor_sync(0xffffffffu, near_particles, o);
    if (lane == 0) {
        A.cnt[0][i] = nm; A.cnt[1][i] = np; A.cnt[2][i] = nq;
        if (near_particles) atomicAdd(&A.stats[1], near_particles * nt.count);
    }
}

__global__ void __launch_bounds__(32 * LW) k_lv_classify(LevelArgs A) {
    __shared__ uint32_t s_cand[LW][CANDS];
    const uint32_t items = (uint32_t)A.info[INFO_ITEMS];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // the scans cover items + 1 entries: the last one (zero) gives every target's end
        const uint32_t m = items < A.item_cap ? items : A.item_cap;
        A.cnt[0][m] = 0; A.cnt[1][m] = 0; A.cnt[2][m] = 0;
        A.info[INFO_ITEMS1] = (int32_t)(m + 1);
    }
    if (items > A.item_cap || lists_failed(A.info)) return;
    const uint32_t stride = gridDim.x * LW;
    for (uint32_t i = blockIdx.x * LW + (threadIdx.x >> 5); i < items; i += stride) {
        lv_classify(A, i, s_cand[threadIdx.x >> 5]);
        __syncwarp();
    }
}

// Places the staged entries of every item at its scanned offsets (candidate order within each
// class); the first item of a target records the target's blocks of this level.
__global__ void __launch_bounds__(32 * LW) k_lv_scatter(LevelArgs A) {
    const uint32_t items = (uint32_t)A.info[INFO_ITEMS];
    if (items > A.item_cap || lists_failed(A.info)) return;
    const int lane = lane_id();
    const uint32_t bm = (uint32_t)A.info[INFO_BASE_M2L], bp = (uint32_t)A.info[INFO_BASE_P2P];
    const uint32_t stride = gridDim.x * LW;
    for (uint32_t i = blockIdx.x * LW + (threadIdx.x >> 5); i < items; i += stride) {
        const uint32_t o_m = bm + A.off[0][i], o_p = bp + A.off[1][i], o_q = A.off[2][i];
        const uint32_t c_m = A.cnt[0][i], c_p = A.cnt[1][i], c_q = A.cnt[2][i];
        const bool ok_m = (uint64_t)o_m + c_m <= A.m2l_cap, ok_p = (uint64_t)o_p + c_p <= A.p2p_cap,
                   ok_q = (uint64_t)o_q + c_q <= A.pend_cap;
        if (lane == 0 && !(ok_m && ok_p && ok_q))
            atomicOr((unsigned int*)&A.info[INFO_ERR],
                     (ok_m ? 0u : NB_ERRBIT_M2L_CAP) | (ok_p ? 0u : NB_ERRBIT_P2P_CAP) | (ok_q ? 0u : NB_ERRBIT_PEND_CAP));
        const uint32_t total = c_m + c_p + c_q;
        const uint32_t* row = A.rows + (size_t)i * CANDS;
        const uint32_t lt = lanemask_lt();
        const uint4 it = A.item[i];
        // the whole row at once (CANDS / 32 loads in flight per lane), then placed group by group
        uint32_t ent[CANDS / 32];
#pragma unroll
        for (int u = 0; u < CANDS / 32; ++u) ent[u] = 32 * u + lane < total ? row[32 * u + lane] : 0u;
        uint32_t nm = 0, np = 0, nq = 0;
#pragma unroll
        for (int u = 0; u < CANDS / 32; ++u) {
            if (32u * u >= total) break;
            const uint32_t e = ent[u];
            const uint32_t cl = e >> 30, sc = e & 0x3fffffffu;
            const uint32_t mm = __ballot_sync(0xffffffffu, cl == 1), mp = __ballot_sync(0xffffffffu, cl == 2),
                           mq = __ballot_sync(0xffffffffu, cl == 3);
            if (cl == 1 && ok_m) A.m2l_stage[o_m + nm + __popc(mm & lt)] = sc;
            if (cl == 2 && ok_p) A.p2p_stage[o_p + np + __popc(mp & lt)] = sc;
            if (cl == 3 && ok_q) A.pout_list[o_q + nq + __popc(mq & lt)] = sc;
            nm += __popc(mm);
            np += __popc(mp);
            nq += __popc(mq);
        }
        if (lane == 0) {
            const uint32_t t = it.x;
            if (it.w) {
                // the target's blocks of this level: its first item's offset, through the end of its last
                const uint32_t e = i + it.w;
                A.m2l_soff[t] = o_m;
                A.m2l_scnt[t] = A.off[0][e] - A.off[0][i];
                A.p2p_soff[t] = o_p;
                A.p2p_scnt[t] = A.off[1][e] - A.off[1][i];
                A.pout_off[t] = o_q;
                A.pout_cnt[t] = A.off[2][e] - A.off[2][i];
            }
        }
    }
}

struct CompactArgs {
    const NodeRec* nodes;
    int nn, depth;
    const uint32_t *m2l_soff, *m2l_scnt, *p2p_soff, *p2p_scnt;   // (depth + 1) rows of nn
    uint32_t *m2l_cnt, *p2p_cnt, *m2l_off, *p2p_off;
    uint32_t *m2l_cp, *p2p_cp, *m2l_cpo, *p2p_cpo;                // entries to move (multi-block targets), scanned
    uint32_t *m2l_list, *p2p_list;
    uint32_t m2l_cap, p2p_cap;
    int32_t* info;
    unsigned long long* stats;
};

// Per target: list length over its rows (its own level through the deepest; only leaves have more
// than one).  A target whose entries sit in one block keeps them in place; one with several blocks
// gets them moved, in level order, behind the staged entries.
__global__ void __launch_bounds__(256) k_lv_totals(CompactArgs A) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t m = 0, p = 0;
    if (t < A.nn) {
        const NodeRec nd = A.nodes[t];
        const int last = nd.nchild ? nd.level : A.depth;
        uint32_t mb = 0, pb = 0, mo = 0, po = 0;
        for (int l = nd.level; l <= last; ++l) {
            const size_t row = (size_t)l * A.nn + t;
            const uint32_t cm = A.m2l_scnt[row], cp = A.p2p_scnt[row];
            if (cm) { ++mb; mo = A.m2l_soff[row]; }
            if (cp) { ++pb; po = A.p2p_soff[row]; }
            m += cm;
            p += cp;
        }
        A.m2l_cnt[t] = m;
        A.p2p_cnt[t] = p;
        A.m2l_off[t] = mb == 1 ? mo : 0u;
        A.p2p_off[t] = pb == 1 ? po : 0u;
        A.m2l_cp[t] = mb > 1 ? m : 0u;
        A.p2p_cp[t] = pb > 1 ? p : 0u;
    }
    if (t == A.nn) { A.m2l_cp[t] = 0; A.p2p_cp[t] = 0; }
    unsigned long long m64 = m, p64 = p;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m64 += __shfl_xor_sync(0xffffffffu, m64, o);
        p64 += __shfl_xor_sync(0xffffffffu, p64, o);
    }
    if ((threadIdx.x & 31) == 0 && (m64 || p64)) {
        atomicAdd(&A.stats[0], m64);
        atomicAdd(&A.stats[2], p64);
    }
}

// Moves the entries of multi-block targets behind the staged ones, one destination entry per
// lane: a warp takes 32 consecutive destinations, finds the target of its first one by binary search
// over the moved-entry offsets (lanes past that target's end search for their own), then each lane
// walks its target's rows in level order to its source entry.  Parallel over entries, so a long
// list (a large leaf with partners on many levels) does not serialise on one warp.
__device__ __forceinline__ int moved_target(const uint32_t* cpo, int nn, uint32_t d) {
    int lo = 0, hi = nn;                        // largest t with cpo[t] <= d
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (cpo[mid] <= d) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void move_entries(const CompactArgs& A, uint32_t d0, uint32_t tot, const uint32_t* cpo,
                                             const uint32_t* soff, const uint32_t* scnt, uint32_t* list, uint32_t base,
                                             uint32_t* off, uint32_t cap) {
    const int lane = lane_id();
    int t0 = 0;
    if (lane == 0) t0 = moved_target(cpo, A.nn, d0);
    t0 = __shfl_sync(0xffffffffu, t0, 0);
    const uint32_t d = d0 + lane;
    if (d >= tot) return;
    const int t = d < cpo[t0 + 1] ? t0 : moved_target(cpo, A.nn, d);
    uint32_t k = d - cpo[t];
    if (k == 0) off[t] = base + cpo[t];
    const NodeRec nd = A.nodes[t];
    for (int l = nd.level; l <= A.depth; ++l) {
        const size_t row = (size_t)l * A.nn + t;
        const uint32_t cn = scnt[row];
        if (k < cn) {
            list[base + d] = list[NB_IDX(soff[row] + k, cap, NB_SITE_MOVE)];
            return;
        }
        k -= cn;
    }
}

__global__ void __launch_bounds__(256) k_lv_move(CompactArgs A) {
    if (lists_failed(A.info)) return;
    const uint32_t em = (uint32_t)(A.info[INFO_BASE_M2L] + A.info[INFO_LVL_M2L]);
    const uint32_t ep = (uint32_t)(A.info[INFO_BASE_P2P] + A.info[INFO_LVL_P2P]);
    const uint32_t tot_m = A.m2l_cpo[A.nn], tot_p = A.p2p_cpo[A.nn];
    if ((uint64_t)em + tot_m > A.m2l_cap || (uint64_t)ep + tot_p > A.p2p_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            atomicOr((unsigned int*)&A.info[INFO_ERR], NB_ERRBIT_M2L_CAP | NB_ERRBIT_P2P_CAP);
        return;
    }
    // warp-sized chunks of destinations: far-field chunks first, then near-field ones
    const uint32_t cm = (tot_m + 31) / 32, cp = (tot_p + 31) / 32;
    const uint32_t stride = gridDim.x * (blockDim.x >> 5);
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < cm + cp; w += stride) {
        if (w < cm)
            move_entries(A, 32 * w, tot_m, A.m2l_cpo, A.m2l_soff, A.m2l_scnt, A.m2l_list, em, A.m2l_off, A.m2l_cap);
        else
            move_entries(A, 32 * (w - cm), tot_p, A.p2p_cpo, A.p2p_soff, A.p2p_scnt, A.p2p_list, ep, A.p2p_off,
                         A.p2p_cap);
    }
}

__global__ void k_lv_root(const NodeRec* nodes, uint32_t* pend_off, uint32_t* pend_cnt, uint32_t* pend_list,
                          uint32_t* m2l_soff, uint32_t* m2l_scnt, uint32_t* p2p_soff, uint32_t* p2p_scnt,
                          uint32_t* p2p_stage, int32_t* info) {
    if (threadIdx.x != 0) return;
    const bool leaf = nodes[0].nchild == 0;
    pend_off[0] = 0;
    pend_cnt[0] = leaf ? 0u : 1u;
    pend_list[0] = 0;
    m2l_soff[0] = 0;
    m2l_scnt[0] = 0;
    p2p_soff[0] = 0;
    p2p_scnt[0] = leaf ? 1u : 0u;
    if (leaf) p2p_stage[0] = 0;
    info[INFO_BASE_M2L] = 0;
    info[INFO_BASE_P2P] = 0;
    info[INFO_LVL_M2L] = 0;
    info[INFO_LVL_P2P] = leaf ? 1 : 0;
}

// near-field work plan, per leaf (tree order): chunks of NB_P2P_CHUNK partner leaves, partial-sum
// slots of split leaves, and the leaf's size class as the sort key
__global__ void k_p2p_plan(int64_t nleaves, const uint32_t* __restrict__ leaves, const NodeRec* __restrict__ nodes,
                           const uint32_t* __restrict__ p2p_cnt, uint32_t* __restrict__ nch,
                           uint32_t* __restrict__ psize, uint64_t* __restrict__ key, uint32_t* __restrict__ val) {
    const int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= nleaves) return;
    const uint32_t k = leaves[li];
    const uint32_t cnt = nodes[k].count;
    const uint32_t c = (p2p_cnt[k] + NB_P2P_CHUNK - 1) / NB_P2P_CHUNK;
    const uint32_t n = c > 1 ? c : 1u;
    nch[li] = n;
    psize[li] = n > 1 ? n * cnt : 0u;
    key[li] = (uint64_t)nb_p2p_class(cnt);
    val[li] = (uint32_t)li;
}

// leaves regrouped by class (stable): new order, its chunk and slot counts, class boundaries
__global__ void k_p2p_order(int64_t nleaves, const uint32_t* __restrict__ leaves_in, uint32_t* __restrict__ leaves_out,
                            const uint32_t* __restrict__ nch_in, const uint32_t* __restrict__ psize_in,
                            uint32_t* __restrict__ nch_out, uint32_t* __restrict__ psize_out,
                            const uint64_t* __restrict__ key, const uint32_t* __restrict__ val, int32_t* info) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j > nleaves) return;
    if (j == nleaves) { nch_out[j] = 0; psize_out[j] = 0; return; }
    const uint32_t o = val[j];
    leaves_out[j] = leaves_in[o];
    nch_out[j] = nch_in[o];
    psize_out[j] = psize_in[o];
    const int cl = (int)key[j], cp = j > 0 ? (int)key[j - 1] : -1;
    for (int x = cp + 1; x <= cl; ++x) info[INFO_CLS_LEAF + x] = (int32_t)j;
    if (j == nleaves - 1)
        for (int x = cl + 1; x <= NB_P2P_CLASSES; ++x) info[INFO_CLS_LEAF + x] = (int32_t)nleaves;
}

__global__ void k_p2p_class_work(const uint32_t* __restrict__ work_off, int32_t* info) {
    const int x = threadIdx.x;
    if (x <= NB_P2P_CLASSES) info[INFO_CLS_WORK + x] = (int32_t)work_off[info[INFO_CLS_LEAF + x]];
}

}  // namespace

int nb_build_lists(nbody_ctx* c) {
    const int64_t nn = c->nnodes, nl = c->nleaves;
    const int depth = c->depth;
    const size_t rows = (size_t)(depth + 1) * nn;
    NB_TRY(nb_grow(c, c->pend_off, sizeof(uint32_t) * 2 * nn));
    NB_TRY(nb_grow(c, c->pend_cnt, sizeof(uint32_t) * 2 * nn));
    NB_TRY(nb_grow(c, c->m2l_off, sizeof(uint32_t) * (nn + 1)));
    NB_TRY(nb_grow(c, c->m2l_cnt, sizeof(uint32_t) * (nn + 1)));
    NB_TRY(nb_grow(c, c->p2p_off, sizeof(uint32_t) * (nn + 1)));
    NB_TRY(nb_grow(c, c->p2p_cnt, sizeof(uint32_t) * (nn + 1)));
    NB_TRY(nb_grow(c, c->lst_seg, sizeof(uint32_t) * 4 * rows));
    NB_TRY(nb_grow(c, c->lst_nch, sizeof(uint32_t) * (nn + 1)));
    NB_TRY(nb_grow(c, c->lst_first, sizeof(uint32_t) * (nn + 1)));
    NB_TRY(nb_grow(c, c->stats, 8 * sizeof(unsigned long long)));
    uint32_t* seg = DP<uint32_t>(c->lst_seg);
    int32_t* info = DP<int32_t>(c->info);
    const int sms = 152;
    for (int attempt = 0; attempt < 8; ++attempt) {
        c->pend_cap = std::min<size_t>(std::max<size_t>(c->pend_cap, (size_t)64 * nn + 1024), 0xffffffffu);
        c->p2p_cap = std::min<size_t>(std::max<size_t>(c->p2p_cap, (size_t)96 * nl + 1024), 0xffffffffu);
        c->m2l_cap = std::min<size_t>(std::max<size_t>(c->m2l_cap, (size_t)512 * nn + 1024), 0xffffffffu);
        c->item_cap = std::min<size_t>(std::max<size_t>(c->item_cap, (size_t)4 * nn + 4096), 0xffffffffu);
        NB_TRY(nb_grow(c, c->pend_list, sizeof(uint32_t) * 2 * c->pend_cap));
        NB_TRY(nb_grow(c, c->p2p_list, sizeof(uint32_t) * c->p2p_cap));
        NB_TRY(nb_grow(c, c->m2l_list, sizeof(uint32_t) * c->m2l_cap));
        NB_TRY(nb_grow(c, c->lst_target, sizeof(uint4) * c->item_cap));
        NB_TRY(nb_grow(c, c->lst_rows, sizeof(uint32_t) * CANDS * c->item_cap));
        NB_TRY(nb_grow(c, c->lst_cnt, sizeof(uint32_t) * 3 * (c->item_cap + 1)));
        NB_TRY(nb_grow(c, c->lst_off, sizeof(uint32_t) * 3 * (c->item_cap + 1)));
        NB_CU(c, cudaMemsetAsync(c->stats.p, 0, 8 * sizeof(unsigned long long), c->st));
        NB_CU(c, cudaMemsetAsync(info + INFO_ERR, 0, sizeof(int32_t), c->st));
        uint32_t* pend_off = DP<uint32_t>(c->pend_off);
        uint32_t* pend_cnt = DP<uint32_t>(c->pend_cnt);
        uint32_t* pend_list = DP<uint32_t>(c->pend_list);
        uint32_t* cnt = DP<uint32_t>(c->lst_cnt);
        uint32_t* off = DP<uint32_t>(c->lst_off);
        const size_t ic = c->item_cap + 1;
        k_lv_root<<<1, 32, 0, c->st>>>(DP<NodeRec>(c->nodes), pend_off, pend_cnt, pend_list, seg + 0 * rows,
                                       seg + 1 * rows, seg + 2 * rows, seg + 3 * rows, DP<uint32_t>(c->p2p_list),
                                       info);
        NB_LAUNCHED(c, "lists root");
        c->launches += 1;
        LevelArgs A;
        A.nodes = DP<NodeRec>(c->nodes);
        A.nn = (int)nn;
        const float th = (float)c->prm.theta;
        A.theta2 = th * th;
        A.pend_cap = (uint32_t)c->pend_cap;
        A.nch = DP<uint32_t>(c->lst_nch);
        A.first = DP<uint32_t>(c->lst_first);
        A.item = DP<uint4>(c->lst_target);
        A.item_cap = (uint32_t)c->item_cap;
        A.rows = DP<uint32_t>(c->lst_rows);
        for (int k = 0; k < 3; ++k) { A.cnt[k] = cnt + k * ic; A.off[k] = off + k * ic; }
        A.m2l_stage = DP<uint32_t>(c->m2l_list);
        A.p2p_stage = DP<uint32_t>(c->p2p_list);
        A.m2l_cap = (uint32_t)c->m2l_cap;
        A.p2p_cap = (uint32_t)c->p2p_cap;
        A.info = info;
        A.stats = DP<unsigned long long>(c->stats);
        for (int r = 1; r <= depth; ++r) {
            const int pi = (r - 1) & 1, po = r & 1;
            A.r = r;
            A.hi = c->level_start[r + 1];
            A.pin_off = pend_off + pi * nn; A.pin_cnt = pend_cnt + pi * nn; A.pin_list = pend_list + pi * c->pend_cap;
            A.pout_off = pend_off + po * nn; A.pout_cnt = pend_cnt + po * nn; A.pout_list = pend_list + po * c->pend_cap;
            A.m2l_soff = seg + 0 * rows + (size_t)r * nn;
            A.m2l_scnt = seg + 1 * rows + (size_t)r * nn;
            A.p2p_soff = seg + 2 * rows + (size_t)r * nn;
            A.p2p_scnt = seg + 3 * rows + (size_t)r * nn;
            const unsigned gt = (unsigned)((A.hi + 1 + 255) / 256);
            k_lv_plan<<<gt, 256, 0, c->st>>>(A);
            NB_LAUNCHED(c, "lists plan");
            NB_TRY(nb_scan_u32(c, A.nch, A.first, A.hi + 1, (uint32_t*)(info + INFO_ITEMS)));
            k_lv_fill<<<gt, 256, 0, c->st>>>(A);
            k_lv_classify<<<sms * 8, 32 * LW, 0, c->st>>>(A);
            NB_LAUNCHED(c, "lists classify");
            // per-item offsets; one extra entry past the last item gives each target's end
            {
                const uint32_t* in3[3] = {A.cnt[0], A.cnt[1], A.cnt[2]};
                uint32_t* out3[3] = {A.off[0], A.off[1], A.off[2]};
                uint32_t* tot3[3] = {(uint32_t*)(info + INFO_LVL_M2L), (uint32_t*)(info + INFO_LVL_P2P),
                                     (uint32_t*)(info + INFO_LVL_PEND)};
                NB_TRY(nb_scan3_u32(c, in3, out3, (int64_t)c->item_cap + 1, tot3, (const uint32_t*)(info + INFO_ITEMS1)));
            }
            k_lv_scatter<<<sms * 8, 32 * LW, 0, c->st>>>(A);
            NB_LAUNCHED(c, "lists scatter");
            c->launches += 4;
        }
        // per-target lists: blocks left in place, multi-block targets concatenated in level order
        NB_TRY(nb_grow(c, c->lst_cp, sizeof(uint32_t) * 4 * (nn + 1)));
        uint32_t* cp = DP<uint32_t>(c->lst_cp);
        CompactArgs B;
        B.nodes = DP<NodeRec>(c->nodes);
        B.nn = (int)nn;
        B.depth = depth;
        B.m2l_soff = seg; B.m2l_scnt = seg + rows; B.p2p_soff = seg + 2 * rows; B.p2p_scnt = seg + 3 * rows;
        B.m2l_cnt = DP<uint32_t>(c->m2l_cnt); B.p2p_cnt = DP<uint32_t>(c->p2p_cnt);
        B.m2l_off = DP<uint32_t>(c->m2l_off); B.p2p_off = DP<uint32_t>(c->p2p_off);
        B.m2l_cp = cp; B.p2p_cp = cp + (nn + 1); B.m2l_cpo = cp + 2 * (nn + 1); B.p2p_cpo = cp + 3 * (nn + 1);
        B.m2l_list = DP<uint32_t>(c->m2l_list); B.p2p_list = DP<uint32_t>(c->p2p_list);
        B.m2l_cap = (uint32_t)c->m2l_cap; B.p2p_cap = (uint32_t)c->p2p_cap;
        B.info = info;
        B.stats = DP<unsigned long long>(c->stats);
        k_lv_totals<<<(unsigned)((nn + 1 + 255) / 256), 256, 0, c->st>>>(B);
        NB_LAUNCHED(c, "lists totals");
        {
            const uint32_t* in3[3] = {B.m2l_cp, B.p2p_cp, nullptr};
            uint32_t* out3[3] = {B.m2l_cpo, B.p2p_cpo, nullptr};
            uint32_t* tot3[3] = {(uint32_t*)(info + INFO_MOVED_M2L), (uint32_t*)(info + INFO_MOVED_P2P), nullptr};
            NB_TRY(nb_scan3_u32(c, in3, out3, nn + 1, tot3));
        }
        k_lv_move<<<sms * 8, 256, 0, c->st>>>(B);
        NB_LAUNCHED(c, "lists move");
        c->launches += 2;
        // near-field work plan: leaves grouped by size class, chunk and slot offsets
        NB_TRY(nb_grow(c, c->p2p_nch, sizeof(uint32_t) * (nl + 1)));
        NB_TRY(nb_grow(c, c->p2p_work_off, sizeof(uint32_t) * (nl + 1)));
        NB_TRY(nb_grow(c, c->p2p_psize, sizeof(uint32_t) * (nl + 1)));
        NB_TRY(nb_grow(c, c->p2p_part_off, sizeof(uint32_t) * (nl + 1)));
        NB_TRY(nb_grow(c, c->leaves_tmp, sizeof(uint32_t) * nl));
        for (int k = 0; k < 2; ++k) {
            NB_TRY(nb_grow(c, c->cls_key[k], sizeof(uint64_t) * nl));
            NB_TRY(nb_grow(c, c->cls_val[k], sizeof(uint32_t) * nl));
        }
        // chunk / slot counts in tree order go to the offset arrays first (scratch until the scans)
        uint32_t* nch0 = DP<uint32_t>(c->p2p_work_off);
        uint32_t* psz0 = DP<uint32_t>(c->p2p_part_off);
        k_p2p_plan<<<(unsigned)((nl + 255) / 256), 256, 0, c->st>>>(nl, DP<uint32_t>(c->leaves), DP<NodeRec>(c->nodes),
                                                                    B.p2p_cnt, nch0, psz0, DP<uint64_t>(c->cls_key[0]),
                                                                    DP<uint32_t>(c->cls_val[0]));
        NB_LAUNCHED(c, "p2p plan");
        int first = 1;
        NB_TRY(nb_radix_sort(c, nl, DP<uint64_t>(c->cls_key[0]), DP<uint32_t>(c->cls_val[0]),
                             DP<uint64_t>(c->cls_key[1]), DP<uint32_t>(c->cls_val[1]), 0, 3, &first));
        const int ks = first ? 0 : 1;
        k_p2p_order<<<(unsigned)((nl + 1 + 255) / 256), 256, 0, c->st>>>(
            nl, DP<uint32_t>(c->leaves), DP<uint32_t>(c->leaves_tmp), nch0, psz0, DP<uint32_t>(c->p2p_nch),
            DP<uint32_t>(c->p2p_psize), DP<uint64_t>(c->cls_key[ks]), DP<uint32_t>(c->cls_val[ks]), info);
        NB_LAUNCHED(c, "p2p order");
        std::swap(c->leaves, c->leaves_tmp);
        {
            const uint32_t* in3[3] = {DP<uint32_t>(c->p2p_nch), DP<uint32_t>(c->p2p_psize), nullptr};
            uint32_t* out3[3] = {DP<uint32_t>(c->p2p_work_off), DP<uint32_t>(c->p2p_part_off), nullptr};
            uint32_t* tot3[3] = {(uint32_t*)(info + INFO_P2P_WORK), (uint32_t*)(info + INFO_P2P_PART), nullptr};
            NB_TRY(nb_scan3_u32(c, in3, out3, nl + 1, tot3));
        }
        k_p2p_class_work<<<1, 32, 0, c->st>>>(DP<uint32_t>(c->p2p_work_off), info);
        NB_LAUNCHED(c, "p2p class work");
        c->launches += 3;
        NB_CU(c, cudaMemcpyAsync(c->h_info, info, sizeof(int32_t) * INFO_WORDS, cudaMemcpyDeviceToHost, c->st));
        NB_CU(c, cudaMemcpyAsync(c->h_stats, c->stats.p, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 c->st));
        NB_CU(c, cudaStreamSynchronize(c->st));
        // extent of each list buffer (staged entries plus the moved ones)
        c->h_info[INFO_M2L_TAIL] = c->h_info[INFO_BASE_M2L] + c->h_info[INFO_LVL_M2L] + c->h_info[INFO_MOVED_M2L];
        c->h_info[INFO_P2P_TAIL] = c->h_info[INFO_BASE_P2P] + c->h_info[INFO_LVL_P2P] + c->h_info[INFO_MOVED_P2P];
        if (c->h_info[INFO_SCAN_ERR]) return nb_fail(c, NBODY_ERR_CUDA, "a device scan did not complete in time");
        const uint32_t e = (uint32_t)c->h_info[INFO_ERR];
        const uint32_t caps = NB_ERRBIT_PEND_CAP | NB_ERRBIT_P2P_CAP | NB_ERRBIT_M2L_CAP | NB_ERRBIT_ITEM_CAP;
        if (!(e & caps)) return NBODY_OK;
        if (attempt == 7) break;
        if (e & NB_ERRBIT_M2L_CAP) c->m2l_cap *= 2;
        if (e & NB_ERRBIT_PEND_CAP) c->pend_cap *= 2;
        if (e & NB_ERRBIT_P2P_CAP) c->p2p_cap *= 2;
        if (e & NB_ERRBIT_ITEM_CAP) c->item_cap *= 2;
    }
    return nb_fail(c, NBODY_ERR_CAPACITY, "interaction lists kept overflowing");
}

NB_DBG_ACCESSOR(lists)
