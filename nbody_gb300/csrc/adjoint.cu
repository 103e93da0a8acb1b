// C ABI of the adjoint: one force vector-Jacobian product, a leapfrog run that
// records sorted-state snapshots, and the reverse sweep over that run.
// Declarations are in include/nbody_gb300.h.
//
// Reverse sweep of N kick-drift-kick steps (time points 0..N):
//   lambda_v is continuous through the kicks, lambda_x through the drifts;
//   at time point pt the force a(x_pt) entered the kicks with weight
//   c = dt/2 (pt = 0 or N) or dt (both half kicks of an interior point), so
//   its VJP is taken with mu = c lambda_v and added to lambda_x, q and m;
//   before time point pt < N the drift x_{pt+1} = x_pt + dt v gives
//   lambda_v += dt lambda_x.
// The VJP at a time point needs its tree, lists and local expansions.  With
// checkpoints, each segment is recomputed forward from its checkpoint (whose
// snapshot already holds the accelerations: its far field only is evaluated)
// and every evaluation of the segment is recorded whole, so the segment's
// reverse pass re-evaluates nothing; memory: one snapshot per checkpoint plus
// the records of one segment.  The last segment, the first one the reverse
// sweep needs, is recorded during the forward run itself and not recomputed.
// Snapshots hold the sorted state (positions, velocities, accelerations,
// masses, charges, ids), so a recomputed segment is bitwise the recorded one.
#include <algorithm>

#include "nbody_internal.cuh"

namespace {

constexpr int TB = 256;
inline unsigned nblk(int64_t n) { return (unsigned)((n + TB - 1) / TB); }

template <typename R>
__global__ void k_to_r(int64_t n, const double* __restrict__ a, R* __restrict__ o) {
    const int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i < n) o[i] = (R)a[i];
}

template <typename R>
__global__ void k_to_d(int64_t n, const R* __restrict__ a, double* __restrict__ o) {
    const int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i < n) o[i] = (double)a[i];
}

// reverse drift: lambda_v += dt lambda_x
template <typename R>
__global__ void k_rev_drift(int64_t n, R* __restrict__ lv, const R* __restrict__ lx, double dt) {
    const int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i < n) lv[i] += (R)dt * lx[i];
}

// row_of[id[i]] = i: where each particle sits in the order of `id`
__global__ void k_row_of(int64_t n, const uint32_t* __restrict__ id, uint32_t* __restrict__ row_of) {
    const int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i < n) row_of[id[i]] = (uint32_t)i;
}

// positions, velocities, masses and charges of buffer `a` (rows located by row_of) re-ordered into
// the order id_new of buffer `b`
template <typename R>
struct Arr8 {
    R* p[8];
};
template <typename R>
__global__ void k_reorder(int64_t n, const uint32_t* __restrict__ id_new, const uint32_t* __restrict__ row_of,
                          Arr8<R> a, Arr8<R> b) {
    const int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    const uint32_t j = row_of[id_new[i]];
#pragma unroll
    for (int k = 0; k < 8; ++k) b.p[k][i] = a.p[k][j];
}

// snapshot layout: 11 state arrays of n scalars (x y z vx vy vz ax ay az m q) then n ids
size_t snapshot_bytes(const nbody_ctx* c) {
    const size_t b = (11 * c->rsz + sizeof(uint32_t)) * (size_t)c->n;
    return (b + 255) / 256 * 256;
}

DevBuf* state_arrays(nbody_ctx* c, int k, DevBuf** out) {
    DevBuf* a[11] = {&c->x[k], &c->y[k], &c->z[k], &c->vx[k], &c->vy[k], &c->vz[k],
                     &c->ax[k], &c->ay[k], &c->az[k], &c->m[k], &c->q[k]};
    for (int i = 0; i < 11; ++i) out[i] = a[i];
    return &c->id[k];
}

int snap_save(nbody_ctx* c, int slot) {
    unsigned char* base = (unsigned char*)c->snaps.p + (size_t)slot * c->snap_bytes;
    const size_t rb = c->rsz * (size_t)c->n;
    DevBuf* arr[11];
    DevBuf* id = state_arrays(c, c->cur, arr);
    for (int i = 0; i < 11; ++i)
        NB_CU(c, cudaMemcpyAsync(base + i * rb, arr[i]->p, rb, cudaMemcpyDeviceToDevice, c->st));
    NB_CU(c, cudaMemcpyAsync(base + 11 * rb, id->p, sizeof(uint32_t) * c->n, cudaMemcpyDeviceToDevice, c->st));
    return NBODY_OK;
}

int snap_load(nbody_ctx* c, int slot) {
    const unsigned char* base = (const unsigned char*)c->snaps.p + (size_t)slot * c->snap_bytes;
    const size_t rb = c->rsz * (size_t)c->n;
    DevBuf* arr[11];
    DevBuf* id = state_arrays(c, c->cur, arr);
    for (int i = 0; i < 11; ++i)
        NB_CU(c, cudaMemcpyAsync(arr[i]->p, base + i * rb, rb, cudaMemcpyDeviceToDevice, c->st));
    NB_CU(c, cudaMemcpyAsync(id->p, base + 11 * rb, sizeof(uint32_t) * c->n, cudaMemcpyDeviceToDevice, c->st));
    c->have_acc = true;
    c->eval_current = false;
    c->amax_valid = false;     // the adaptive step's max |a| belonged to the state before the load
    return NBODY_OK;
}

int vjp(nbody_ctx* c, double coef) {
    switch (c->prm.precision) {
        case NBODY_PREC_FP32: return nb_fmm_vjp_fp32(c, coef);
        case NBODY_PREC_MIXED: return nb_fmm_vjp_mixed(c, coef);
        default: return nb_fmm_vjp_fp64(c, coef);
    }
}

int alloc_adjoint(nbody_ctx* c) {
    const size_t rb = c->rsz * (size_t)c->n;
    NB_TRY(nb_grow(c, c->adj_lx, 3 * rb));
    NB_TRY(nb_grow(c, c->adj_lv, 3 * rb));
    NB_TRY(nb_grow(c, c->adj_gq, rb));
    NB_TRY(nb_grow(c, c->adj_gm, rb));
    return NBODY_OK;
}

// host or device double array -> R buffer (through the staging area)
int upload_r(nbody_ctx* c, const double* src, int64_t cnt, DevBuf& dst, double* stage) {
    if (src) {
        NB_CU(c, cudaMemcpyAsync(stage, src, sizeof(double) * cnt, cudaMemcpyDefault, c->st));
        if (c->rsz == 4) k_to_r<float><<<nblk(cnt), TB, 0, c->st>>>(cnt, stage, DP<float>(dst));
        else k_to_r<double><<<nblk(cnt), TB, 0, c->st>>>(cnt, stage, DP<double>(dst));
        NB_LAUNCHED(c, "adjoint upload");
    } else {
        NB_CU(c, cudaMemsetAsync(dst.p, 0, c->rsz * cnt, c->st));
    }
    return NBODY_OK;
}

int download_r(nbody_ctx* c, const DevBuf& src, int64_t cnt, double* dst, double* stage) {
    if (!dst) return NBODY_OK;
    if (c->rsz == 4) k_to_d<float><<<nblk(cnt), TB, 0, c->st>>>(cnt, DP<float>(src), stage);
    else k_to_d<double><<<nblk(cnt), TB, 0, c->st>>>(cnt, DP<double>(src), stage);
    NB_LAUNCHED(c, "adjoint download");
    NB_CU(c, cudaMemcpyAsync(dst, stage, sizeof(double) * cnt, cudaMemcpyDefault, c->st));
    return NBODY_OK;
}

int rev_drift(nbody_ctx* c) {
    const int64_t n3 = 3 * c->n;
    if (c->rsz == 4) k_rev_drift<float><<<nblk(n3), TB, 0, c->st>>>(n3, DP<float>(c->adj_lv), DP<float>(c->adj_lx),
                                                                      c->prm.dt);
    else k_rev_drift<double><<<nblk(n3), TB, 0, c->st>>>(n3, DP<double>(c->adj_lv), DP<double>(c->adj_lx),
                                                           c->prm.dt);
    NB_LAUNCHED(c, "reverse drift");
    return NBODY_OK;
}

// evaluation records: the buffers the force VJP reads, with their sizes for a given tree
struct RecField {
    DevBuf* buf;
    size_t bytes;
};

int rec_fields(nbody_ctx* c, int64_t nn, int64_t nl, uint32_t m2l_ext, uint32_t p2p_ext, RecField* f) {
    const int64_t n = c->n;
    const int k = c->cur;
    const int p = c->prm.order;
    const size_t terms = (size_t)(p + 1) * (p + 2) * (p + 3) / 6;
    const size_t s4 = c->prm.precision == NBODY_PREC_FP64 ? 32 : 16;
    const size_t hs = c->prm.precision == NBODY_PREC_FP64 ? 8 : 4;
    int i = 0;
    f[i++] = {&c->nodes, sizeof(NodeRec) * (size_t)nn};
    f[i++] = {&c->leaves, sizeof(uint32_t) * (size_t)nl};
    f[i++] = {&c->box, sizeof(BoxDev)};
    f[i++] = {&c->src, s4 * (size_t)n};
    f[i++] = {&c->id[k], sizeof(uint32_t) * (size_t)n};
    for (DevBuf* b : {&c->q[k], &c->m[k], &c->ax[k], &c->ay[k], &c->az[k]}) f[i++] = {b, c->rsz * (size_t)n};
    f[i++] = {&c->L, hs * terms * (size_t)nn};
    f[i++] = {&c->m2l_off, sizeof(uint32_t) * (size_t)nn};
    f[i++] = {&c->m2l_cnt, sizeof(uint32_t) * (size_t)nn};
    f[i++] = {&c->m2l_list, sizeof(uint32_t) * (size_t)m2l_ext};
    f[i++] = {&c->p2p_off, sizeof(uint32_t) * (size_t)nn};
    f[i++] = {&c->p2p_cnt, sizeof(uint32_t) * (size_t)nn};
    f[i++] = {&c->p2p_list, sizeof(uint32_t) * (size_t)p2p_ext};
    f[i++] = {&c->p2p_work_off, sizeof(uint32_t) * (size_t)(nl + 1)};
    f[i++] = {&c->p2p_part_off, sizeof(uint32_t) * (size_t)(nl + 1)};
    return i;
}

inline size_t al256(size_t b) { return (b + 255) / 256 * 256; }

// records the current evaluation as record j
int rec_save(nbody_ctx* c, int j) {
    if ((int)c->recs.size() <= j) c->recs.resize(j + 1);
    EvalRecord& R = c->recs[j];
    RecField f[24] = {};
    const int nf = rec_fields(c, c->nnodes, c->nleaves, (uint32_t)c->h_info[INFO_M2L_TAIL],
                              (uint32_t)c->h_info[INFO_P2P_TAIL], f);
    size_t total = 0;
    for (int i = 0; i < nf; ++i) total += al256(f[i].bytes);
    NB_TRY(nb_grow(c, R.buf, total));
    size_t o = 0;
    for (int i = 0; i < nf; ++i) {
        if (f[i].bytes)
            NB_CU(c, cudaMemcpyAsync((char*)R.buf.p + o, f[i].buf->p, f[i].bytes, cudaMemcpyDeviceToDevice, c->st));
        o += al256(f[i].bytes);
    }
    R.nn = c->nnodes;
    R.nl = c->nleaves;
    R.depth = c->depth;
    R.box_side = c->box_side;
    std::copy(c->level_start, c->level_start + NB_LEVELS + 3, R.level_start);
    std::copy(c->h_info, c->h_info + INFO_WORDS, R.info);
    return NBODY_OK;
}

// makes record j the context's current evaluation (the particle state arrays it includes are the
// sorted charges, masses, accelerations and ids; positions and velocities are left alone); the
// tree is then the record's, neither the current state's nor the recorded run's final one until a
// caller says so
int rec_load(nbody_ctx* c, int j) {
    EvalRecord& R = c->recs[j];
    c->eval_current = false;
    c->tree_at_final = false;
    RecField f[24] = {};
    const int nf = rec_fields(c, R.nn, R.nl, (uint32_t)R.info[INFO_M2L_TAIL], (uint32_t)R.info[INFO_P2P_TAIL], f);
    size_t o = 0;
    for (int i = 0; i < nf; ++i) {
        NB_TRY(nb_grow(c, *f[i].buf, f[i].bytes));
        if (f[i].bytes)
            NB_CU(c, cudaMemcpyAsync(f[i].buf->p, (const char*)R.buf.p + o, f[i].bytes, cudaMemcpyDeviceToDevice, c->st));
        o += al256(f[i].bytes);
    }
    c->nnodes = R.nn;
    c->nleaves = R.nl;
    c->depth = R.depth;
    c->box_side = R.box_side;
    std::copy(R.level_start, R.level_start + NB_LEVELS + 3, c->level_start);
    std::copy(R.info, R.info + INFO_WORDS, c->h_info);
    const int64_t npart = (uint32_t)R.info[INFO_P2P_PART];
    NB_TRY(nb_grow(c, c->p2p_part, c->rsz * 4 * (size_t)(npart + 1)));
    return NBODY_OK;
}

// snapshot slots: 0 .. nck-1 checkpoints, then the final state
int nck(const nbody_ctx* c) { return c->rec_mode ? 0 : (c->ck_steps + c->ck_every - 1) / c->ck_every; }
int final_slot(const nbody_ctx* c) { return nck(c); }

}  // namespace

extern "C" {

int nbody_force_vjp(nbody_ctx* c, const double* mu, double* gx, double* gq, double* gm) {
    if (!c || !mu) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    NB_CU(c, cudaSetDevice(c->device));
    const int64_t n = c->n;
    NB_TRY(alloc_adjoint(c));
    NB_TRY(nb_evaluate(c, 0, NB_INTEG_NONE, false));
    c->have_acc = c->prm.integrator == NBODY_INTEG_LEAPFROG;
    double* st = DP<double>(c->stage);
    NB_TRY(upload_r(c, mu, 3 * n, c->adj_lv, st));
    NB_CU(c, cudaMemsetAsync(c->adj_lx.p, 0, 3 * c->rsz * n, c->st));
    NB_CU(c, cudaMemsetAsync(c->adj_gq.p, 0, c->rsz * n, c->st));
    NB_CU(c, cudaMemsetAsync(c->adj_gm.p, 0, c->rsz * n, c->st));
    const int64_t l0 = c->launches;
    NB_TRY(vjp(c, 1.0));
    NB_TRY(download_r(c, c->adj_lx, 3 * n, gx, st));
    NB_TRY(download_r(c, c->adj_gq, n, gq, st + 3 * n));
    NB_TRY(download_r(c, c->adj_gm, n, gm, st + 4 * n));
    NB_CU(c, cudaStreamSynchronize(c->st));
    NB_TRY(nb_dbg_check(c));
    c->launches = c->launches - l0;
    if (c->timing)
        for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&c->phase_ms[7 + i], c->ev[8 + i], c->ev[9 + i]);
    return NBODY_OK;
}

int nbody_forward_checkpointed(nbody_ctx* c, int nsteps, int every, double* t_out) {
    if (!c) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    if (c->prm.integrator != NBODY_INTEG_LEAPFROG)
        return nb_fail(c, NBODY_ERR_INVALID, "the recorded run needs the leapfrog integrator");
    if (c->dt_mode != NBODY_DT_FIXED)
        return nb_fail(c, NBODY_ERR_STATE, "the recorded run differentiates fixed steps: switch adaptive steps off");
    if (nsteps < 1 || every < 0) return nb_fail(c, NBODY_ERR_INVALID, "nsteps must be >= 1 and every >= 0");
    NB_CU(c, cudaSetDevice(c->device));
    const bool rec = every == 0;
    every = rec ? 1 : std::min(every, nsteps);
    c->ck_steps = 0;
    c->rec_mode = rec;
    c->snap_bytes = snapshot_bytes(c);
    const int slots = rec ? 1 : (nsteps + every - 1) / every + 1;
    NB_TRY(nb_grow(c, c->snaps, c->snap_bytes * (size_t)slots));
    // first time point of the last checkpoint interval: its evaluations are recorded as they happen
    const int s_last = rec ? 0 : ((nsteps - 1) / every) * every;
    c->ck_last_recorded = false;
    // time point 0 needs its accelerations, and its whole evaluation where it is recorded (the far
    // field only where the accelerations are known, as the reverse sweep's recomputation does)
    if (!c->have_acc) {
        NB_TRY(nb_evaluate(c, 0, NB_INTEG_NONE, false));
        c->have_acc = true;
    } else if (s_last == 0 && !c->eval_current) {
        NB_TRY(nb_evaluate(c, 0, rec ? NB_INTEG_NONE : NB_INTEG_FAR_ONLY, false));
    }
    c->ck_t0 = c->time;
    c->ck_every = every;
    c->ck_steps = nsteps;
    if (rec) NB_TRY(rec_save(c, 0));
    else NB_TRY(snap_save(c, 0));
    if (!rec && s_last == 0) NB_TRY(rec_save(c, 0));
    for (int s = 0; s < nsteps; ++s) {
        NB_TRY(nb_evaluate(c, 1, NB_INTEG_KDK_CLOSE, false));
        c->time += c->prm.dt;
        const int pt = s + 1;
        if (rec) NB_TRY(rec_save(c, pt));
        else if (pt < nsteps && pt % every == 0) NB_TRY(snap_save(c, pt / every));
        if (!rec && pt >= s_last && pt < nsteps) NB_TRY(rec_save(c, pt - s_last));
    }
    c->ck_last_recorded = !rec;
    NB_TRY(snap_save(c, final_slot(c)));
    NB_CU(c, cudaStreamSynchronize(c->st));
    c->tree_at_final = true;
    if (t_out) *t_out = c->time;
    return NBODY_OK;
}

}  // extern "C"

namespace {

// buffer `from` (ordered by its ids) -> buffer c->cur in the order of c->id[c->cur]
template <typename R>
int reorder_t(nbody_ctx* c, int from) {
    const int k = c->cur;
    const int64_t n = c->n;
    uint32_t* row_of = DP<uint32_t>(c->pfx);          // tree scratch, free between evaluations
    k_row_of<<<nblk(n), TB, 0, c->st>>>(n, DP<uint32_t>(c->id[from]), row_of);
    Arr8<R> a = {{DP<R>(c->x[from]), DP<R>(c->y[from]), DP<R>(c->z[from]), DP<R>(c->vx[from]), DP<R>(c->vy[from]),
                  DP<R>(c->vz[from]), DP<R>(c->m[from]), DP<R>(c->q[from])}};
    Arr8<R> b = {{DP<R>(c->x[k]), DP<R>(c->y[k]), DP<R>(c->z[k]), DP<R>(c->vx[k]), DP<R>(c->vy[k]), DP<R>(c->vz[k]),
                  DP<R>(c->m[k]), DP<R>(c->q[k])}};
    k_reorder<R><<<nblk(n), TB, 0, c->st>>>(n, DP<uint32_t>(c->id[k]), row_of, a, b);
    NB_LAUNCHED(c, "replay reorder");
    return NBODY_OK;
}

// time points 0 .. nsteps of the recorded run, each evaluated on its recorded tree and lists from
// the given initial state
int replay(nbody_ctx* c, const double* pos, const double* vel, const double* mass, const double* charge, int nsteps,
           double* pos_out, double* vel_out) {
    const int64_t n = c->n;
    int from = 1 - c->cur;            // the initial state, input order, identity ids
    NB_TRY(nb_upload_state(c, from, n, pos, vel, mass, charge, nullptr));
    c->lists_frozen = true;
    for (int pt = 0; pt <= nsteps; ++pt) {
        int rc = NBODY_OK;
        if (pt > 0) rc = nb_kick_drift(c);                               // in the previous order
        if (rc == NBODY_OK) {
            c->cur = 1 - from;
            rc = rec_load(c, pt);                                        // tree, lists and plan of pt
        }
        if (rc == NBODY_OK) rc = c->rsz == 4 ? reorder_t<float>(c, from) : reorder_t<double>(c, from);
        if (rc == NBODY_OK) rc = nb_evaluate_frozen(c, pt == 0 ? NB_INTEG_NONE : NB_INTEG_KDK_CLOSE);
        if (rc != NBODY_OK) {
            c->lists_frozen = false;
            return rc;
        }
        from = c->cur;
    }
    c->lists_frozen = false;
    NB_TRY(nb_download_state(c, 1));
    const double* st = DP<double>(c->stage);
    if (pos_out) NB_CU(c, cudaMemcpyAsync(pos_out, st, sizeof(double) * 3 * n, cudaMemcpyDefault, c->st));
    if (vel_out) NB_CU(c, cudaMemcpyAsync(vel_out, st + 3 * n, sizeof(double) * 3 * n, cudaMemcpyDefault, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    return NBODY_OK;
}

}  // namespace

extern "C" {

int nbody_forward_replay(nbody_ctx* c, const double* pos, const double* vel, const double* mass,
                         const double* charge, int nsteps, double* pos_out, double* vel_out) {
    if (!c || !pos || !mass) return NBODY_ERR_INVALID;
    if (c->ck_steps < 1 || !c->rec_mode)
        return nb_fail(c, NBODY_ERR_STATE, "no run recorded with every evaluation (nbody_forward_checkpointed, every = 0)");
    if (nsteps < 0) nsteps = c->ck_steps;
    if (nsteps > c->ck_steps) return nb_fail(c, NBODY_ERR_INVALID, "nsteps exceeds the recorded steps");
    NB_CU(c, cudaSetDevice(c->device));
    const int rc = replay(c, pos, vel, mass, charge, nsteps, pos_out, vel_out);
    // back to the recorded run's final state with its evaluation current, replay or not
    NB_TRY(snap_load(c, final_slot(c)));
    NB_TRY(rec_load(c, c->ck_steps));
    c->eval_current = true;
    c->tree_at_final = true;
    NB_CU(c, cudaStreamSynchronize(c->st));
    return rc;
}

int nbody_backward(nbody_ctx* c, const double* gxT, const double* gvT, double* gx0, double* gv0, double* gq,
                   double* gm) {
    if (!c) return NBODY_ERR_INVALID;
    if (c->ck_steps < 1) return nb_fail(c, NBODY_ERR_STATE, "no recorded run (call nbody_forward_checkpointed)");
    NB_CU(c, cudaSetDevice(c->device));
    const int64_t n = c->n;
    const int N = c->ck_steps, every = c->ck_every;
    const double dt = c->prm.dt;
    NB_TRY(alloc_adjoint(c));
    double* st = DP<double>(c->stage);
    NB_TRY(upload_r(c, gxT, 3 * n, c->adj_lx, st));
    NB_TRY(upload_r(c, gvT, 3 * n, c->adj_lv, st + 3 * n));
    NB_CU(c, cudaMemsetAsync(c->adj_gq.p, 0, c->rsz * n, c->st));
    NB_CU(c, cudaMemsetAsync(c->adj_gm.p, 0, c->rsz * n, c->st));
    if (c->rec_mode) {
        // every time point's evaluation was recorded: no re-evaluation
        for (int pt = N; pt >= 0; --pt) {
            if (pt < N) NB_TRY(rev_drift(c));
            if (pt < N || !c->tree_at_final) NB_TRY(rec_load(c, pt));
            NB_TRY(vjp(c, pt == N || pt == 0 ? 0.5 * dt : dt));
        }
        NB_TRY(download_r(c, c->adj_lx, 3 * n, gx0, st));
        NB_TRY(download_r(c, c->adj_lv, 3 * n, gv0, st + 3 * n));
        NB_TRY(download_r(c, c->adj_gq, n, gq, st + 6 * n));
        NB_TRY(download_r(c, c->adj_gm, n, gm, st + 7 * n));
        // back to the final state with its evaluation current
        NB_TRY(snap_load(c, final_slot(c)));
        NB_TRY(rec_load(c, N));
        c->eval_current = true;
        c->tree_at_final = true;
        c->time = c->ck_t0 + N * dt;
        NB_CU(c, cudaStreamSynchronize(c->st));
        return nb_dbg_check(c);
    }
    // time point N
    if (!c->tree_at_final) {
        NB_TRY(snap_load(c, final_slot(c)));
        NB_TRY(nb_evaluate(c, 0, NB_INTEG_FAR_ONLY, false));
    }
    NB_TRY(vjp(c, 0.5 * dt));
    // segments [s0, e), last first: the checkpoint's tree, lists and far field (its snapshot holds
    // the accelerations), then the recomputed steps s0+1 .. e-1, each evaluation recorded whole, so
    // the segment's reverse pass re-evaluates nothing.  The last segment's records come from the
    // forward run, as long as no earlier segment has been recomputed over them since.
    const int s_last = ((N - 1) / every) * every;
    for (int s0 = s_last; s0 >= 0; s0 -= every) {
        const int e = std::min(s0 + every, N);
        const bool recorded = s0 == s_last && c->ck_last_recorded;
        if (!recorded) {
            c->ck_last_recorded = false;
            NB_TRY(snap_load(c, s0 / every));
            c->time = c->ck_t0 + s0 * dt;
            NB_TRY(nb_evaluate(c, 0, NB_INTEG_FAR_ONLY, false));
            NB_TRY(rec_save(c, 0));
            for (int pt = s0 + 1; pt <= e - 1; ++pt) {
                NB_TRY(nb_evaluate(c, 1, NB_INTEG_KDK_CLOSE, false));
                NB_TRY(rec_save(c, pt - s0));
            }
        }
        for (int pt = e - 1; pt >= s0; --pt) {
            NB_TRY(rev_drift(c));
            // after a recomputation, pt = e - 1 is the current evaluation
            if (recorded || pt < e - 1) NB_TRY(rec_load(c, pt - s0));
            NB_TRY(vjp(c, pt == 0 ? 0.5 * dt : dt));
        }
    }
    // the records hold the last segment again only if it was the only one
    c->ck_last_recorded = s_last == 0;
    NB_TRY(download_r(c, c->adj_lx, 3 * n, gx0, st));
    NB_TRY(download_r(c, c->adj_lv, 3 * n, gv0, st + 3 * n));
    NB_TRY(download_r(c, c->adj_gq, n, gq, st + 6 * n));
    NB_TRY(download_r(c, c->adj_gm, n, gm, st + 7 * n));
    // back to the recorded run's final state
    NB_TRY(snap_load(c, final_slot(c)));
    c->time = c->ck_t0 + N * dt;
    NB_CU(c, cudaStreamSynchronize(c->st));
    return nb_dbg_check(c);
}

}  // extern "C"
