// Internal definitions shared by the CUDA translation units of libnbody_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/nbody_gb300.h"

#define NB_LEVELS 21               // bits per axis of the Morton grid; deepest level
#define NB_PMAX 8                  // highest expansion order compiled
#define NB_TMAX 165                // terms at NB_PMAX

// error bits raised on the device (ctx->d_info[INFO_ERR])
#define NB_ERRBIT_PEND_CAP 1u      // refinement list capacity exceeded
#define NB_ERRBIT_P2P_CAP 2u       // near-field list capacity exceeded
#define NB_ERRBIT_RANGE 8u         // no representable root box covers the particles
#define NB_ERRBIT_NONFINITE 16u    // a position was not finite
#define NB_ERRBIT_M2L_CAP 32u      // far-field list capacity exceeded
#define NB_ERRBIT_ASYNC 64u        // an asynchronous copy did not complete within its time limit
#define NB_ERRBIT_ITEM_CAP 128u    // list-building work items exceeded their capacity
#define NB_ERRBIT_ESCAPE 256u      // a particle lay outside the fixed root box

#define NB_SCAN_POLLS (1ll << 20)  // default look-back polls of one scan status word (about a second)
#define NB_COPY_CYCLES 2000000000ll   // default bound of the far-field kernel's copy waits (SM cycles)

#define NB_P2P_CHUNK 256           // partner leaves per near-field work item
#define NB_P2P_CLASSES 6           // near-field leaf-size classes (one kernel each)

// near-field class of a leaf of `count` particles: lanes per target group (CT) and targets per
// lane (TPL) are chosen so that CT x TPL target slots fit the leaf closely
//   class  count   CT  TPL  slots
//     0    1-8      4   2     8
//     1    9-16     8   2    16
//     2    17-24    8   3    24
//     3    25-32   16   2    32
//     4    33-48   16   3    48
//     5    49-     32   2    64 (larger leaves take several passes)
__host__ __device__ __forceinline__ int nb_p2p_class(uint32_t count) {
    return count <= 8 ? 0 : count <= 16 ? 1 : count <= 24 ? 2 : count <= 32 ? 3 : count <= 48 ? 4 : 5;
}

// layout of the small device info block (int32 words)
enum {
    INFO_ERR = 0,
    INFO_DEPTH = 1,
    INFO_NNODES = 2,
    INFO_NLEAVES = 3,
    INFO_PEND_TAIL = 4,
    INFO_P2P_TAIL = 5,
    INFO_M2L_TAIL = 6,
    INFO_HIST = 8,                 // 8 .. 8+NB_LEVELS: nodes per level
    INFO_P2P_WORK = 30,            // near-field work items
    INFO_P2P_PART = 31,            // near-field partial-sum slots
    INFO_ITEMS = 32,               // list-building items of the current level
    INFO_LVL_M2L = 33,             // far-field entries written by the current level
    INFO_LVL_P2P = 34,             // near-field entries written by the current level
    INFO_LVL_PEND = 35,            // pending entries written by the current level
    INFO_BASE_M2L = 36,            // staged far-field entries of the levels before
    INFO_BASE_P2P = 37,            // staged near-field entries of the levels before
    INFO_MOVED_M2L = 38,           // far-field entries moved behind the staged ones
    INFO_MOVED_P2P = 39,           // near-field entries moved behind the staged ones
    INFO_ITEMS1 = 40,              // list-building items of the current level plus one (scan length)
    INFO_CLS_LEAF = 48,            // 48 .. 54: first leaf (in near-field order) of each class, then the count
    INFO_CLS_WORK = 56,            // 56 .. 62: first near-field work item of each class, then the total
    INFO_SCAN_ERR = 63,            // sticky: a device scan's look-back gave up waiting (never cleared by a step)
    INFO_WORDS = 64
};

// one octree node, breadth-first order, 32 bytes
struct __align__(16) NodeRec {
    uint32_t ix, iy, iz;           // cell coordinates at its level
    uint32_t begin, count;         // particle range in Morton order
    int32_t parent;                // -1 for the root
    int32_t child_begin;           // first child (children are contiguous)
    uint8_t level, nchild;         // nchild == 0 <=> leaf
    uint8_t child_mask;            // bit k set <=> the child in octant k exists (children stored in octant order)
    uint8_t pad;
};
static_assert(sizeof(NodeRec) == 32, "NodeRec must stay 32 bytes");

// root box on the device: origin xyz, side, 2^21/side, fine unit side/2^22
struct BoxDev {
    double ox, oy, oz, side, scale, unit;
};

// grow-only device allocation
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// one recorded force evaluation: everything the force VJP reads (tree, lists, local expansions,
// particle offsets, sorted charges/masses/accelerations/ids), packed in one device block
struct EvalRecord {
    DevBuf buf;
    int64_t nn = 0, nl = 0;
    int depth = 0;
    double box_side = 0.0;         // root box side of that evaluation
    int level_start[NB_LEVELS + 3] = {0};
    int32_t info[INFO_WORDS] = {0};
};

struct nb_traj;   // trajectory writer (trajectory.cu)

struct nbody_ctx {
    nbody_params prm;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaStream_t side[NB_P2P_CLASSES] = {};   // near-field class kernels run side by side
    cudaEvent_t fork_ev = nullptr, join_ev[NB_P2P_CLASSES] = {};
    int64_t n = 0;
    double time = 0.0;
    bool have_acc = false;
    size_t rsz = 8;                // bytes of a state scalar (4 in the fp32 form)

    // particle state in Morton order (double buffered across the re-sort)
    int cur = 0;
    DevBuf x[2], y[2], z[2], vx[2], vy[2], vz[2], ax[2], ay[2], az[2], m[2], q[2], id[2];
    DevBuf pot;                    // potential per particle (diagnostics)

    // sort scratch
    DevBuf keys[2], vals[2], hist, hist_scan;
    DevBuf scan_part;              // single-pass scan state: ticket counter and tile status words
    uint64_t scan_epoch = 0;       // tag of the last scan's status words
    int64_t scan_polls = NB_SCAN_POLLS;            // look-back polls of one status word before giving up
    long long copy_cycles = NB_COPY_CYCLES;        // far-field wait for its bulk copies (SM clock cycles)
    DevBuf wait_probe;             // status words of nbody_selftest_scan_wait

    // tree scratch and result
    DevBuf cpl, wnd, leaflvl, nc, pfx, seedk[2], seedv[2], nodes, leafflag, leafpfx, leaves;
    int64_t nnodes = 0, nleaves = 0;
    int depth = 0;
    int level_start[NB_LEVELS + 3] = {0};

    // expansions and lists
    DevBuf M, L, src;
    DevBuf pend_off, pend_cnt, pend_list;          // pending lists, two level parities
    DevBuf p2p_off, p2p_cnt, p2p_list, m2l_off, m2l_cnt, m2l_list;   // per-target lists
    DevBuf lst_seg, lst_nch, lst_first, lst_target, lst_cnt, lst_off, lst_cp, lst_rows;   // list-building work
    DevBuf cls_key[2], cls_val[2], leaves_tmp;      // near-field class ordering of the leaves
    size_t pend_cap = 0, p2p_cap = 0, m2l_cap = 0, item_cap = 0;
    DevBuf stage;                  // host <-> device staging (interleaved doubles)
    DevBuf diag;
    DevBuf stats;                  // 8 x uint64 work counters of the last evaluation
    DevBuf p2p_nch, p2p_work_off, p2p_psize, p2p_part_off, p2p_part;   // near-field work plan
    unsigned long long h_stats[8] = {0};
    int64_t launches = 0;          // kernels launched by the last force evaluation
    size_t dev_bytes = 0, dev_peak = 0;   // device memory held by the context, and its high-water mark
    long long alloc_fail_after = -1;      // NBODY_FAIL_ALLOC_AFTER: allocations that succeed before one fails
    long long alloc_calls = 0;

    // small device blocks + pinned mirrors
    DevBuf info, box, bbox;
    int32_t* h_info = nullptr;
    BoxDev* h_box = nullptr;       // root box of the current tree, read at the tree's synchronisation
    double box_side = 0.0;         // its side (the FP64 form's M2L derivative table depends on it)

    // M2L derivative table of the FP64 form: D(r) of every same-level cell offset within +-dt_R and
    // every offset of cells one level apart (odd half-cell offsets within +-(2 dt_R + 1)), levels
    // 0 .. dt_levels - 1
    DevBuf dtab;
    int dt_R = 0, dt_levels = 0, dt_order = 0, dt_prec = -1;
    double dt_side = 0.0, dt_eps = -1.0;

    // adjoint (input-order accumulators, adjoint expansions, trajectory snapshots)
    DevBuf adj_lx, adj_lv, adj_gq, adj_gm, adj_nu, adj_lamL, adj_lamM, adj_near;
    DevBuf snaps;                  // sorted-state snapshots: checkpoints, segment scratch, final state
    size_t snap_bytes = 0;         // bytes of one snapshot
    int ck_steps = 0;              // steps of the recorded run (0: nothing recorded)
    int ck_every = 0;              // checkpoint spacing of the recorded run
    double ck_t0 = 0.0;            // simulated time at its start
    bool tree_at_final = false;    // the last evaluation was the recorded run's final one
    bool rec_mode = false;         // the recorded run kept every evaluation (no re-evaluation backward)
    bool ck_last_recorded = false; // records hold the last checkpoint interval of the recorded run
    bool eval_current = false;     // tree, lists and expansions match the current state
    bool lists_frozen = false;     // the force evaluation reuses the loaded lists (frozen-structure replay)
    std::vector<EvalRecord> recs;  // its evaluations, time points 0 .. steps

    // per-phase timing
    bool timing = false;
    cudaEvent_t ev[16] = {};       // 0..7 force evaluation, 8..13 force VJP
    float phase_ms[16] = {0};

    nb_traj* traj = nullptr;       // open trajectory file, if any

    // particles leaving a fixed root box (nbody_set_escape_policy)
    int escape_policy = NBODY_ESCAPE_GROW;
    int64_t escapes = 0;           // evaluations since nbody_set_state that took a grown root box

    // step-size control (nbody_set_timestep_control)
    int dt_mode = NBODY_DT_FIXED;
    double dt_eta = 0, dt_len = 0, dt_min = 0, dt_max = 0;
    double dt_base = 0;            // params.dt before adaptive steps were switched on
    double dt_last = 0;            // dt of the last step
    bool amax_valid = false;       // amax2 holds max |a|^2 of the current accelerations
    int blk_K = 0;                 // block steps: substeps of dt_max / 2^blk_K (NBODY_DT_BLOCK)
    double blk_dt = 0;             // the substep (drift) length
    DevBuf blk_level;              // per input id: level k of the particle's current step, dt = dt_max / 2^k
    DevBuf blk_count;              // per level: closing kicks of the last base step
    DevBuf blk_active;             // per leaf (near-field order): a particle closes its step at substep blk_s
    int blk_s = 0;                 // substep of the evaluation in progress (0: not a block substep)
    int64_t blk_evals = 0;         // force evaluations of the last block step (substeps where a step ended)
    int64_t blk_leaves = 0, blk_active_leaves = 0;   // near-field leaves evaluated vs skipped (stats)
    unsigned int h_blk_count[32] = {0};
    double amax2 = 0;
    DevBuf amax;                   // device word of the reduction (bits of a non-negative double)
    double* h_amax = nullptr;      // pinned copy

    std::string err;
};

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
int nb_fail(nbody_ctx* c, int code, const std::string& msg);
int nb_cuda(nbody_ctx* c, cudaError_t e, const char* what);
int nb_grow(nbody_ctx* c, DevBuf& b, size_t bytes);

#define NB_TRY(expr)                 \
    do {                             \
        int _rc = (expr);            \
        if (_rc != NBODY_OK) return _rc; \
    } while (0)
#define NB_CU(c, expr) NB_TRY(nb_cuda((c), (expr), #expr))
#define NB_LAUNCHED(c, name) NB_TRY(nb_cuda((c), cudaGetLastError(), name))

template <typename T>
static inline T* DP(const DevBuf& b) { return reinterpret_cast<T*>(b.p); }

// scan + sort (sort.cu)
int nb_scan_u32(nbody_ctx* c, const uint32_t* in, uint32_t* out, int64_t n, uint32_t* total_dev);
// up to three exclusive scans in one set of launches (null inputs skipped); with n_dev, only the
// first *n_dev of the n entries are scanned
int nb_scan3_u32(nbody_ctx* c, const uint32_t* const in[3], uint32_t* const out[3], int64_t n,
                 uint32_t* const total_dev[3], const uint32_t* n_dev = nullptr);
// the scan look-back's wait on a word nothing publishes; NBODY_ERR_CUDA once it ran out (sort.cu)
int nb_scan_wait_selftest(nbody_ctx* c);
// the far-field kernel's copy wait on a barrier no copy completes; NBODY_ERR_CUDA once it ran out
// (fmm_fp32.cu)
int nb_copy_wait_selftest(nbody_ctx* c);
// NBODY_ERR_CUDA if h_info[INFO_ERR] (just read back) says a far-field copy wait ran out (api.cu)
int nb_check_async(nbody_ctx* c);
int nb_radix_sort(nbody_ctx* c, int64_t n, uint64_t* k0, uint32_t* v0, uint64_t* k1, uint32_t* v1, int begin_bit,
                  int end_bit, int* result_in_first);

// state upload (input order, identity ids) into buffer k, and download of the current buffer into
// the staging area (api.cu)
int nb_upload_state(nbody_ctx* c, int k, int64_t n, const double* pos, const double* vel, const double* mass,
                    const double* charge, const double* acc);
int nb_download_state(nbody_ctx* c, int order);

// tree (tree.cu)
int nb_kick_drift(nbody_ctx* c);
int nb_drift(nbody_ctx* c, double dt);
int nb_begin_step(nbody_ctx* c, int kdk);
int nb_sort_and_gather(nbody_ctx* c);
int nb_build_tree(nbody_ctx* c);

// interaction lists and near-field work plan of the current tree (lists.cu); syncs once
int nb_build_lists(nbody_ctx* c);

// side streams: nb_fork makes them wait for the main stream's work so far, nb_join makes the main
// stream wait for what was queued on them since (api.cu)
int nb_fork(nbody_ctx* c);
int nb_join(nbody_ctx* c);

// trajectory rows after a step, and closing the writer (trajectory.cu)
int nb_traj_capture(nbody_ctx* c);
int nb_traj_close(nbody_ctx* c);

// one force evaluation at the current positions (api.cu); kdk = 1 applies the opening kick and drift first
int nb_evaluate(nbody_ctx* c, int kdk, int integ, bool want_pot);
// the far and near field only, on the tree and lists already loaded (lists_frozen) (api.cu)
int nb_evaluate_frozen(nbody_ctx* c, int integ);
// one base step of dt_max with block (individual power-of-two) time steps (blocksteps.cu)
int nb_block_step(nbody_ctx* c);
// marks the near-field leaves holding a particle whose step ends at substep blk_s (blocksteps.cu)
int nb_block_active_leaves(nbody_ctx* c);

// fmm (fmm_*.cu)
int nb_fmm_forces_fp32(nbody_ctx* c, int integ, bool want_pot);
int nb_fmm_forces_mixed(nbody_ctx* c, int integ, bool want_pot);
int nb_fmm_forces_fp64(nbody_ctx* c, int integ, bool want_pot);
// adjoint of the last force evaluation (fmm_*.cu): mu = coef * adj_lv, accumulated into adj_lx/adj_gq/adj_gm
int nb_fmm_vjp_fp32(nbody_ctx* c, double coef);
int nb_fmm_vjp_mixed(nbody_ctx* c, double coef);
int nb_fmm_vjp_fp64(nbody_ctx* c, double coef);

// integration modes of the force epilogue
// NB_INTEG_FAR_ONLY: tree, lists and far field only (accelerations already known, e.g. from a snapshot)
enum { NB_INTEG_NONE = 0, NB_INTEG_KDK_CLOSE = 1, NB_INTEG_EULER = 2, NB_INTEG_FAR_ONLY = 3 };

// ---------------------------------------------------------------------------
// index checks of the NBODY_DEBUG_BOUNDS build
//
// NB_IDX(i, n, site) is i when i < n.  In the debug build an index out of range sets bit `site` of
// this translation unit's debug word and yields 0, an index that is always in bounds, so the kernel
// goes on without a fault; the host reads and clears the words after each evaluation
// (nb_dbg_check) and reports NBODY_ERR_CUDA naming the sites.  The release build compiles to i.
// ---------------------------------------------------------------------------
enum {
    NB_SITE_GATHER = 0,            // sorted-order permutation entry (k_gather)
    NB_SITE_TREE = 1,              // first particle of a node (k_tree_nodes)
    NB_SITE_SORT = 2,              // radix scatter destination
    NB_SITE_LISTS = 3,             // pending partner / candidate node ids (k_lv_classify)
    NB_SITE_MOVE = 4,              // staged list entry moved behind the staged ones (k_lv_move)
    NB_SITE_M2L = 5,               // far-field list entry (k_m2l)
    NB_SITE_P2P = 6,               // near-field list entry and its particle range (k_p2p)
    NB_SITE_ADJ = 7                // near-field list entry and its particle range (k_adj_p2p)
};
#ifdef NBODY_DEBUG_BOUNDS
static __device__ unsigned int nb_dbg_word;     // one per translation unit
__device__ __forceinline__ uint32_t nb_idx_check(uint64_t i, uint64_t n, int site) {
    if (i < n) return (uint32_t)i;
    atomicOr(&nb_dbg_word, 1u << site);
    return 0u;
}
#define NB_IDX(i, n, site) nb_idx_check((uint64_t)(i), (uint64_t)(n), (site))
// host accessor of this translation unit's word: returns it and clears it
#define NB_DBG_ACCESSOR(name)                                                              \
    unsigned int nb_dbg_take_##name() {                                                    \
        unsigned int v = 0, z = 0;                                                         \
        if (cudaMemcpyFromSymbol(&v, nb_dbg_word, sizeof(v)) != cudaSuccess) v = 0x80000000u; \
        cudaMemcpyToSymbol(nb_dbg_word, &z, sizeof(z));                                   \
        return v;                                                                          \
    }
#else
#define NB_IDX(i, n, site) (i)
#define NB_DBG_ACCESSOR(name)
#endif
// reads and clears every translation unit's debug word; NBODY_ERR_CUDA if a check fired (api.cu)
int nb_dbg_check(nbody_ctx* c);

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float nb_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double nb_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float nb_rsqrt(float s) { return rsqrtf(s); }
// four consecutive values from a 16-byte aligned address
__device__ __forceinline__ void nb_ld4(const float* p, float* o) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void nb_ld4(const double* p, double* o) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
__device__ __forceinline__ double nb_rsqrt(double s) { return rsqrt(s); }
// rsqrt for arguments known to be normal (bounded below by a softening or a cell separation): the
// PTX approximation with flush-to-zero, one special-function instruction, no subnormal handling
__device__ __forceinline__ float nb_rsqrt_n(float s) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s));
    return r;
}
__device__ __forceinline__ double nb_rsqrt_n(double s) { return rsqrt(s); }

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() { return (1u << lane_id()) - 1u; }

// inclusive warp scan of v
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane_id() >= (uint32_t)o) v += t;
    }
    return v;
}

// bitonic sort of one unique key per lane, descending across the warp
__device__ __forceinline__ uint32_t warp_sort_desc(uint32_t v) {
    const uint32_t lane = lane_id();
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const uint32_t o = __shfl_xor_sync(0xffffffffu, v, j);
            const bool keep_max = ((lane & j) == 0) == ((lane & k) == 0);
            v = keep_max ? max(v, o) : min(v, o);
        }
    }
    return v;
}

// 21-bit spread / compact for Morton interleaving (x = bit 0 of each triple)
__host__ __device__ __forceinline__ uint64_t nb_spread3(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__host__ __device__ __forceinline__ uint32_t nb_compact3(uint64_t v) {
    v &= 0x1249249249249249ull;
    v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
    v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
    v = (v ^ (v >> 8)) & 0x1f0000ff0000ffull;
    v = (v ^ (v >> 16)) & 0x1f00000000ffffull;
    v = (v ^ (v >> 32)) & 0x1fffffull;
    return (uint32_t)v;
}

// centre of a node in fine units (side / 2^22): (2 i + 1) << (21 - level)
__device__ __forceinline__ void nb_centre_fine(const NodeRec& nd, long long& cx, long long& cy, long long& cz) {
    int sh = NB_LEVELS - nd.level;
    cx = (2ll * nd.ix + 1) << sh;
    cy = (2ll * nd.iy + 1) << sh;
    cz = (2ll * nd.iz + 1) << sh;
}
__device__ __forceinline__ long long nb_width_fine(const NodeRec& nd) { return 1ll << (NB_LEVELS + 1 - nd.level); }

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
