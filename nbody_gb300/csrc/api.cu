// C ABI of libnbody_gb300: context lifetime, state upload/download, the step
// loop and inspection calls.  Declarations and reference citations are in
// include/nbody_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "nbody_internal.cuh"

static thread_local std::string g_create_err;

int nb_fail(nbody_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    else g_create_err = msg;
    return code;
}

int nb_cuda(nbody_ctx* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return NBODY_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();
    return nb_fail(c, e == cudaErrorMemoryAllocation ? NBODY_ERR_NOMEM : NBODY_ERR_CUDA, m);
}

int nb_grow(nbody_ctx* c, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return NBODY_OK;
    // allocation-failure injection for the error paths (NBODY_FAIL_ALLOC_AFTER at nbody_create)
    if (c->alloc_fail_after >= 0 && c->alloc_calls++ >= c->alloc_fail_after)
        return nb_fail(c, NBODY_ERR_NOMEM, "cudaMalloc: allocation failure injected by NBODY_FAIL_ALLOC_AFTER");
    if (b.p) {
        NB_CU(c, cudaStreamSynchronize(c->st));
        NB_CU(c, cudaFree(b.p));
        c->dev_bytes -= b.bytes;
        b.p = nullptr;
        b.bytes = 0;
    }
    size_t want = bytes + bytes / 4;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        e = cudaMalloc(&p, bytes);
        want = bytes;
    }
    NB_TRY(nb_cuda(c, e, "cudaMalloc"));
    b.p = p;
    b.bytes = want;
    c->dev_bytes += want;
    c->dev_peak = std::max(c->dev_peak, c->dev_bytes);
    return NBODY_OK;
}

int nb_fork(nbody_ctx* c) {
    NB_CU(c, cudaEventRecord(c->fork_ev, c->st));
    for (int i = 0; i < NB_P2P_CLASSES; ++i) NB_CU(c, cudaStreamWaitEvent(c->side[i], c->fork_ev, 0));
    return NBODY_OK;
}

int nb_join(nbody_ctx* c) {
    for (int i = 0; i < NB_P2P_CLASSES; ++i) {
        NB_CU(c, cudaEventRecord(c->join_ev[i], c->side[i]));
        NB_CU(c, cudaStreamWaitEvent(c->st, c->join_ev[i], 0));
    }
    return NBODY_OK;
}

static void release(DevBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

namespace {

constexpr int TB = 256;
inline unsigned nblk(int64_t n) { return (unsigned)((n + TB - 1) / TB); }

template <typename R>
__global__ void k_upload(int64_t n, const double* __restrict__ st, R* x, R* y, R* z, R* vx, R* vy, R* vz, R* ax,
                         R* ay, R* az, R* m, R* q, uint32_t* id, int have_charge, int have_acc) {
    int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    const double* pos = st;
    const double* vel = st + 3 * n;
    const double* ms = st + 6 * n;
    const double* cs = st + 7 * n;
    x[i] = (R)pos[3 * i]; y[i] = (R)pos[3 * i + 1]; z[i] = (R)pos[3 * i + 2];
    vx[i] = (R)vel[3 * i]; vy[i] = (R)vel[3 * i + 1]; vz[i] = (R)vel[3 * i + 2];
    if (have_acc) {
        const double* ac = st + 9 * n;
        ax[i] = (R)ac[3 * i]; ay[i] = (R)ac[3 * i + 1]; az[i] = (R)ac[3 * i + 2];
    } else {
        ax[i] = 0; ay[i] = 0; az[i] = 0;
    }
    m[i] = (R)ms[i];
    q[i] = (R)(have_charge ? cs[i] : ms[i]);
    id[i] = (uint32_t)i;
}

// which: bit 0 pos, 1 vel, 2 mass, 3 charge, 4 ids, 5 acc, 6 pot
template <typename R>
__global__ void k_download(int64_t n, int input_order, const R* x, const R* y, const R* z, const R* vx, const R* vy,
                           const R* vz, const R* ax, const R* ay, const R* az, const R* m, const R* q, const R* pot,
                           const uint32_t* id, double* st) {
    int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    int64_t o = input_order ? (int64_t)id[i] : i;
    double* pos = st;
    double* vel = st + 3 * n;
    double* ms = st + 6 * n;
    double* cs = st + 7 * n;
    int64_t* ids = (int64_t*)(st + 8 * n);
    double* acc = st + 9 * n;
    double* pt = st + 12 * n;
    pos[3 * o] = x[i]; pos[3 * o + 1] = y[i]; pos[3 * o + 2] = z[i];
    vel[3 * o] = vx[i]; vel[3 * o + 1] = vy[i]; vel[3 * o + 2] = vz[i];
    ms[o] = m[i];
    cs[o] = q[i];
    ids[o] = (int64_t)id[i];
    acc[3 * o] = ax[i]; acc[3 * o + 1] = ay[i]; acc[3 * o + 2] = az[i];
    pt[o] = pot ? (double)pot[i] : 0.0;
}

// FP64 partial sums per block: KE, W, p(3), J(3), M ; fixed-order block reduction
template <typename R>
__global__ void __launch_bounds__(TB) k_diag(int64_t n, const R* x, const R* y, const R* z, const R* vx, const R* vy,
                                             const R* vz, const R* m, const R* q, const R* pot, double* part) {
    __shared__ double sh[9][TB];
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x; i < n; i += (int64_t)gridDim.x * TB) {
        double mi = m[i], X = x[i], Y = y[i], Z = z[i], VX = vx[i], VY = vy[i], VZ = vz[i];
        v[0] += 0.5 * mi * (VX * VX + VY * VY + VZ * VZ);
        v[1] += 0.5 * (double)q[i] * (double)pot[i];
        v[2] += mi * VX; v[3] += mi * VY; v[4] += mi * VZ;
        v[5] += mi * (Y * VZ - Z * VY); v[6] += mi * (Z * VX - X * VZ); v[7] += mi * (X * VY - Y * VX);
        v[8] += mi;
    }
    for (int k = 0; k < 9; ++k) sh[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int s = TB / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < 9; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 9) part[(int64_t)blockIdx.x * 9 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void k_diag_final(int nb, const double* part, double* out) {
    if (threadIdx.x < 9) {
        double s = 0;
        for (int b = 0; b < nb; ++b) s += part[(int64_t)b * 9 + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

int alloc_state(nbody_ctx* c, int64_t n) {
    const size_t rb = c->rsz * (size_t)n;
    for (int k = 0; k < 2; ++k) {
        for (DevBuf* b : {&c->x[k], &c->y[k], &c->z[k], &c->vx[k], &c->vy[k], &c->vz[k], &c->ax[k], &c->ay[k],
                          &c->az[k], &c->m[k], &c->q[k]})
            NB_TRY(nb_grow(c, *b, rb));
        NB_TRY(nb_grow(c, c->id[k], sizeof(uint32_t) * n));
        NB_TRY(nb_grow(c, c->keys[k], sizeof(uint64_t) * n));
        NB_TRY(nb_grow(c, c->vals[k], sizeof(uint32_t) * n));
    }
    NB_TRY(nb_grow(c, c->pot, rb));
    NB_TRY(nb_grow(c, c->cpl, sizeof(int32_t) * n));
    NB_TRY(nb_grow(c, c->wnd, sizeof(int32_t) * n));
    NB_TRY(nb_grow(c, c->nc, sizeof(uint32_t) * n));
    NB_TRY(nb_grow(c, c->pfx, sizeof(uint32_t) * n));
    NB_TRY(nb_grow(c, c->stage, sizeof(double) * 13 * (size_t)n));
    return NBODY_OK;
}

template <typename R>
int download_t(nbody_ctx* c, int input_order) {
    const int k = c->cur;
    k_download<R><<<nblk(c->n), TB, 0, c->st>>>(c->n, input_order, DP<R>(c->x[k]), DP<R>(c->y[k]), DP<R>(c->z[k]),
                                                 DP<R>(c->vx[k]), DP<R>(c->vy[k]), DP<R>(c->vz[k]), DP<R>(c->ax[k]),
                                                 DP<R>(c->ay[k]), DP<R>(c->az[k]), DP<R>(c->m[k]), DP<R>(c->q[k]),
                                                 DP<R>(c->pot), DP<uint32_t>(c->id[k]), DP<double>(c->stage));
    NB_LAUNCHED(c, "download");
    return NBODY_OK;
}

int fmm(nbody_ctx* c, int integ, bool want_pot) {
    switch (c->prm.precision) {
        case NBODY_PREC_FP32: return nb_fmm_forces_fp32(c, integ, want_pot);
        case NBODY_PREC_MIXED: return nb_fmm_forces_mixed(c, integ, want_pot);
        default: return nb_fmm_forces_fp64(c, integ, want_pot);
    }
}

// max_i |a_i|^2 of the current accelerations for the adaptive step: block maxima, then one atomicMax
// per block on the bit pattern (non-negative doubles order like their bits; NaN never wins a compare)
template <typename R>
__global__ void __launch_bounds__(TB) k_amax2(int64_t n, const R* __restrict__ ax, const R* __restrict__ ay,
                                               const R* __restrict__ az, unsigned long long* out) {
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x; i < n; i += (int64_t)gridDim.x * TB) {
        const double x = (double)ax[i], y = (double)ay[i], z = (double)az[i];
        const double a2 = x * x + y * y + z * z;
        m = a2 > m ? a2 : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double v = __shfl_xor_sync(0xffffffffu, m, o);
        m = v > m ? v : m;
    }
    __shared__ double s_m[TB / 32];
    if ((threadIdx.x & 31) == 0) s_m[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < TB / 32; ++w) m = s_m[w] > m ? s_m[w] : m;
        atomicMax(out, (unsigned long long)__double_as_longlong(m));
    }
}

// queues the reduction and the copy of its result to pinned memory (read after the next sync)
template <typename R>
int amax_t(nbody_ctx* c) {
    const int k = c->cur;
    unsigned g = std::min<unsigned>(nblk(c->n), 152 * 8);
    if (g == 0) g = 1;
    NB_CU(c, cudaMemsetAsync(c->amax.p, 0, sizeof(unsigned long long), c->st));
    k_amax2<R><<<g, TB, 0, c->st>>>(c->n, DP<R>(c->ax[k]), DP<R>(c->ay[k]), DP<R>(c->az[k]),
                                    DP<unsigned long long>(c->amax));
    NB_LAUNCHED(c, "acceleration maximum");
    c->launches += 1;
    NB_CU(c, cudaMemcpyAsync(c->h_amax, c->amax.p, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    return NBODY_OK;
}

}  // namespace

#ifdef NBODY_DEBUG_BOUNDS
unsigned int nb_dbg_take_tree();
unsigned int nb_dbg_take_sort();
unsigned int nb_dbg_take_lists();
unsigned int nb_dbg_take_fmm_fp32();
unsigned int nb_dbg_take_fmm_mixed();
unsigned int nb_dbg_take_fmm_fp64();
#endif

int nb_dbg_check(nbody_ctx* c) {
#ifdef NBODY_DEBUG_BOUNDS
    const unsigned int w = nb_dbg_take_tree() | nb_dbg_take_sort() | nb_dbg_take_lists() | nb_dbg_take_fmm_fp32() |
                           nb_dbg_take_fmm_mixed() | nb_dbg_take_fmm_fp64();
    if (w) {
        char msg[96];
        std::snprintf(msg, sizeof msg, "index check failed (debug build), site bits 0x%x", w);
        return nb_fail(c, NBODY_ERR_CUDA, msg);
    }
#else
    (void)c;
#endif
    return NBODY_OK;
}

int nb_check_async(nbody_ctx* c) {
    if ((uint32_t)c->h_info[INFO_ERR] & NB_ERRBIT_ASYNC)
        return nb_fail(c, NBODY_ERR_CUDA, "a far-field copy did not complete in time");
    return NBODY_OK;
}

// one force evaluation at the current positions, with an optional integrator epilogue
int nb_evaluate(nbody_ctx* c, int kdk, int integ, bool want_pot) {
    c->launches = 0;
    c->tree_at_final = false;
    c->eval_current = false;
    if (c->timing) cudaEventRecord(c->ev[0], c->st);
    NB_TRY(nb_begin_step(c, kdk));
    if (c->timing) cudaEventRecord(c->ev[1], c->st);
    NB_TRY(nb_sort_and_gather(c));
    if (c->timing) cudaEventRecord(c->ev[2], c->st);
    NB_TRY(nb_build_tree(c));
    NB_TRY(fmm(c, integ, want_pot));
    // adaptive steps: the largest acceleration of this evaluation, read at the sync below
    c->amax_valid = false;
    const bool adaptive = c->dt_mode == NBODY_DT_ADAPTIVE;
    if (adaptive) NB_TRY(c->rsz == 4 ? amax_t<float>(c) : amax_t<double>(c));
    // error bits raised after the traversal check (asynchronous copies of the far field)
    NB_CU(c, cudaMemcpyAsync(c->h_info, c->info.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    NB_TRY(nb_check_async(c));
    NB_TRY(nb_dbg_check(c));
    if (c->timing) {
        NB_CU(c, cudaEventSynchronize(c->ev[7]));
        for (int i = 0; i < 7; ++i) cudaEventElapsedTime(&c->phase_ms[i], c->ev[i], c->ev[i + 1]);
    }
    if (adaptive) {
        c->amax2 = *c->h_amax;
        c->amax_valid = true;
    }
    c->eval_current = true;
    return NBODY_OK;
}

// the far and near field (with the integrator epilogue) on the tree and lists already loaded
// (lists_frozen set): no kick, re-sort, tree or list building
int nb_evaluate_frozen(nbody_ctx* c, int integ) {
    c->launches = 0;
    c->eval_current = false;
    NB_CU(c, cudaMemsetAsync(c->info.p, 0, sizeof(int32_t), c->st));   // INFO_ERR
    NB_TRY(fmm(c, integ, false));
    NB_CU(c, cudaMemcpyAsync(c->h_info, c->info.p, sizeof(int32_t), cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    NB_TRY(nb_check_async(c));
    NB_TRY(nb_dbg_check(c));
    return NBODY_OK;
}

// the adaptive dt from the last evaluation's largest acceleration (nbody_set_timestep_control)
static double adaptive_dt(const nbody_ctx* c) {
    const double len = c->dt_len > 0.0 ? c->dt_len : c->prm.eps;
    double dt = c->amax2 > 0.0 ? c->dt_eta * std::sqrt(len / std::sqrt(c->amax2)) : c->dt_max;
    if (!(dt >= c->dt_min)) dt = c->dt_min;       // also a non-finite candidate
    if (dt > c->dt_max) dt = c->dt_max;
    return dt;
}

namespace {

template <typename R>
int diag_t(nbody_ctx* c, double* out) {
    const int k = c->cur;
    int nb = (int)std::min<int64_t>(nblk(c->n), 1024);
    if (nb < 1) nb = 1;
    NB_TRY(nb_grow(c, c->diag, sizeof(double) * (9 * (size_t)nb + 9)));
    double* part = DP<double>(c->diag);
    k_diag<R><<<nb, TB, 0, c->st>>>(c->n, DP<R>(c->x[k]), DP<R>(c->y[k]), DP<R>(c->z[k]), DP<R>(c->vx[k]),
                                    DP<R>(c->vy[k]), DP<R>(c->vz[k]), DP<R>(c->m[k]), DP<R>(c->q[k]), DP<R>(c->pot), part);
    k_diag_final<<<1, 32, 0, c->st>>>(nb, part, part + 9 * (size_t)nb);
    NB_LAUNCHED(c, "diagnostics");
    NB_CU(c, cudaMemcpyAsync(out, part + 9 * (size_t)nb, 9 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    return NBODY_OK;
}

}  // namespace

// arrays in input order (host or device memory) -> state buffer k with identity ids (the state
// buffers and the staging area must already hold n particles)
int nb_upload_state(nbody_ctx* c, int k, int64_t n, const double* pos, const double* vel, const double* mass,
                    const double* charge, const double* acc) {
    double* st = DP<double>(c->stage);
    NB_CU(c, cudaMemcpyAsync(st, pos, sizeof(double) * 3 * n, cudaMemcpyDefault, c->st));
    if (vel) NB_CU(c, cudaMemcpyAsync(st + 3 * n, vel, sizeof(double) * 3 * n, cudaMemcpyDefault, c->st));
    else NB_CU(c, cudaMemsetAsync(st + 3 * n, 0, sizeof(double) * 3 * n, c->st));
    NB_CU(c, cudaMemcpyAsync(st + 6 * n, mass, sizeof(double) * n, cudaMemcpyDefault, c->st));
    if (charge) NB_CU(c, cudaMemcpyAsync(st + 7 * n, charge, sizeof(double) * n, cudaMemcpyDefault, c->st));
    if (acc) NB_CU(c, cudaMemcpyAsync(st + 9 * n, acc, sizeof(double) * 3 * n, cudaMemcpyDefault, c->st));
    if (c->rsz == 4)
        k_upload<float><<<nblk(n), TB, 0, c->st>>>(n, st, DP<float>(c->x[k]), DP<float>(c->y[k]), DP<float>(c->z[k]),
                                                   DP<float>(c->vx[k]), DP<float>(c->vy[k]), DP<float>(c->vz[k]),
                                                   DP<float>(c->ax[k]), DP<float>(c->ay[k]), DP<float>(c->az[k]),
                                                   DP<float>(c->m[k]), DP<float>(c->q[k]), DP<uint32_t>(c->id[k]),
                                                   charge != nullptr, acc != nullptr);
    else
        k_upload<double><<<nblk(n), TB, 0, c->st>>>(n, st, DP<double>(c->x[k]), DP<double>(c->y[k]),
                                                    DP<double>(c->z[k]), DP<double>(c->vx[k]), DP<double>(c->vy[k]),
                                                    DP<double>(c->vz[k]), DP<double>(c->ax[k]), DP<double>(c->ay[k]),
                                                    DP<double>(c->az[k]), DP<double>(c->m[k]), DP<double>(c->q[k]),
                                                    DP<uint32_t>(c->id[k]), charge != nullptr, acc != nullptr);
    NB_LAUNCHED(c, "upload");
    return NBODY_OK;
}

// the current state buffer -> the staging area, input order (order = 1) or sorted (0)
int nb_download_state(nbody_ctx* c, int order) {
    return c->rsz == 4 ? download_t<float>(c, order) : download_t<double>(c, order);
}

extern "C" {

void nbody_default_params(nbody_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->precision = NBODY_PREC_FP32;
    p->order = 1;
    p->leaf_capacity = 8;
    p->max_level = NB_LEVELS;
    p->theta = 0.5;
    p->eps = 0.01;
    p->G = 1.0;
    p->dt = 1e-3;
    p->integrator = NBODY_INTEG_EULER;
    p->fixed_box = 1;
    p->box_min[0] = p->box_min[1] = p->box_min[2] = 0.0;
    p->box_size = 1.0;
    p->device = 0;
}

int nbody_create(const nbody_params* p, nbody_ctx** out) {
    if (!p || !out) return nb_fail(nullptr, NBODY_ERR_INVALID, "null argument");
    *out = nullptr;
    if (p->precision < 0 || p->precision > 2) return nb_fail(nullptr, NBODY_ERR_INVALID, "precision must be 0..2");
    if (p->order < 1 || p->order > NB_PMAX) return nb_fail(nullptr, NBODY_ERR_INVALID, "order must be 1..8");
    if (p->leaf_capacity < 1 || p->leaf_capacity > 64)
        return nb_fail(nullptr, NBODY_ERR_INVALID, "leaf_capacity must be 1..64");
    if (p->max_level < 0 || p->max_level > NB_LEVELS) return nb_fail(nullptr, NBODY_ERR_INVALID, "max_level must be 0..21");
    if (!(p->theta > 0.0) || !(p->eps >= 0.0) || !(p->dt >= 0.0))
        return nb_fail(nullptr, NBODY_ERR_INVALID, "theta must be > 0, eps and dt >= 0");
    if (p->fixed_box && !(p->box_size > 0.0)) return nb_fail(nullptr, NBODY_ERR_INVALID, "box_size must be > 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return nb_fail(nullptr, NBODY_ERR_NO_DEVICE, "no CUDA device");
    }
    if (p->device < 0 || p->device >= ndev) return nb_fail(nullptr, NBODY_ERR_INVALID, "device ordinal out of range");
    nbody_ctx* c = new (std::nothrow) nbody_ctx();
    if (!c) return nb_fail(nullptr, NBODY_ERR_NOMEM, "host allocation failed");
    c->prm = *p;
    c->device = p->device;
    if (const char* f = std::getenv("NBODY_FAIL_ALLOC_AFTER")) {
        char* end = nullptr;
        const long long k = std::strtoll(f, &end, 10);
        if (end != f && k >= 0) c->alloc_fail_after = k;
    }
    c->rsz = p->precision == NBODY_PREC_FP32 ? 4 : 8;
    int rc = NBODY_OK;
    do {
        if ((rc = nb_cuda(c, cudaSetDevice(c->device), "cudaSetDevice"))) break;
        if ((rc = nb_cuda(c, cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking), "cudaStreamCreate"))) break;
        if ((rc = nb_grow(c, c->info, sizeof(int32_t) * INFO_WORDS))) break;
        if ((rc = nb_grow(c, c->box, sizeof(BoxDev)))) break;
        if ((rc = nb_grow(c, c->bbox, 6 * sizeof(unsigned long long)))) break;
        if ((rc = nb_cuda(c, cudaMallocHost(&c->h_info, sizeof(int32_t) * INFO_WORDS), "cudaMallocHost"))) break;
        if ((rc = nb_cuda(c, cudaMallocHost(&c->h_box, sizeof(BoxDev)), "cudaMallocHost"))) break;
        if ((rc = nb_cuda(c, cudaMemsetAsync(c->info.p, 0, sizeof(int32_t) * INFO_WORDS, c->st), "memset"))) break;
        for (int i = 0; i < 14 && !rc; ++i) rc = nb_cuda(c, cudaEventCreate(&c->ev[i]), "cudaEventCreate");
        for (int i = 0; i < NB_P2P_CLASSES && !rc; ++i) {
            rc = nb_cuda(c, cudaStreamCreateWithFlags(&c->side[i], cudaStreamNonBlocking), "cudaStreamCreate");
            if (!rc) rc = nb_cuda(c, cudaEventCreateWithFlags(&c->join_ev[i], cudaEventDisableTiming), "cudaEventCreate");
        }
        if (!rc) rc = nb_cuda(c, cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming), "cudaEventCreate");
    } while (0);
    if (rc) {
        g_create_err = c->err;
        nbody_destroy(c);
        return rc;
    }
    *out = c;
    return NBODY_OK;
}

int nbody_destroy(nbody_ctx* c) {
    if (!c) return NBODY_OK;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    nb_traj_close(c);
    for (int k = 0; k < 2; ++k)
        for (DevBuf* b : {&c->x[k], &c->y[k], &c->z[k], &c->vx[k], &c->vy[k], &c->vz[k], &c->ax[k], &c->ay[k], &c->az[k],
                          &c->m[k], &c->q[k], &c->id[k], &c->keys[k], &c->vals[k], &c->seedk[k], &c->seedv[k]})
            release(*b);
    for (DevBuf* b : {&c->pot, &c->stats, &c->p2p_nch, &c->p2p_work_off, &c->p2p_psize, &c->p2p_part_off,
                      &c->p2p_part, &c->hist, &c->hist_scan, &c->scan_part, &c->cpl, &c->wnd, &c->leaflvl, &c->nc, &c->pfx,
                      &c->nodes, &c->leafflag, &c->leafpfx, &c->leaves, &c->M, &c->L, &c->src, &c->pend_off,
                      &c->pend_cnt, &c->p2p_off, &c->p2p_cnt, &c->pend_list, &c->p2p_list, &c->m2l_off, &c->m2l_cnt,
                      &c->m2l_list, &c->stage, &c->diag, &c->info, &c->box, &c->bbox, &c->adj_lx, &c->adj_lv,
                      &c->adj_gq, &c->adj_gm, &c->adj_nu, &c->adj_lamL, &c->adj_lamM, &c->adj_near,
                      &c->snaps, &c->lst_seg, &c->lst_nch, &c->lst_first, &c->lst_target, &c->lst_cnt,
                      &c->lst_off, &c->lst_cp, &c->lst_rows, &c->cls_key[0], &c->cls_key[1], &c->cls_val[0], &c->cls_val[1],
                      &c->leaves_tmp, &c->wait_probe, &c->dtab})
        release(*b);
    for (EvalRecord& r : c->recs) release(r.buf);
    if (c->h_info) cudaFreeHost(c->h_info);
    if (c->h_box) cudaFreeHost(c->h_box);
    if (c->h_amax) cudaFreeHost(c->h_amax);
    release(c->amax);
    for (int i = 0; i < 16; ++i)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    for (int i = 0; i < NB_P2P_CLASSES; ++i) {
        if (c->side[i]) cudaStreamSynchronize(c->side[i]), cudaStreamDestroy(c->side[i]);
        if (c->join_ev[i]) cudaEventDestroy(c->join_ev[i]);
    }
    if (c->fork_ev) cudaEventDestroy(c->fork_ev);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return NBODY_OK;
}

int nbody_set_state(nbody_ctx* c, int64_t n, const double* pos, const double* vel, const double* mass,
                    const double* charge, const double* acc) {
    if (!c) return NBODY_ERR_INVALID;
    if (n < 1 || n > (int64_t)0x7fffffff) return nb_fail(c, NBODY_ERR_INVALID, "n must be in 1..2^31-1");
    if (!pos || !mass) return nb_fail(c, NBODY_ERR_INVALID, "pos and mass are required");
    NB_CU(c, cudaSetDevice(c->device));
    NB_TRY(nb_traj_close(c));   // a trajectory file holds one particle set
    // no particles until the upload below has succeeded: a failed allocation leaves the context
    // without state, so later calls fail with NBODY_ERR_STATE instead of reading missing buffers
    c->n = 0;
    c->ck_steps = 0;
    c->eval_current = false;
    c->cur = 0;
    NB_TRY(alloc_state(c, n));
    NB_TRY(nb_upload_state(c, 0, n, pos, vel, mass, charge, acc));
    NB_CU(c, cudaStreamSynchronize(c->st));
    c->n = n;
    c->escapes = 0;
    c->time = 0.0;
    c->have_acc = acc != nullptr;
    c->amax_valid = false;
    c->ck_steps = 0;
    c->eval_current = false;
    return NBODY_OK;
}

static int fetch(nbody_ctx* c, int order) {
    NB_CU(c, cudaSetDevice(c->device));
    return c->rsz == 4 ? download_t<float>(c, order) : download_t<double>(c, order);
}

int nbody_get_state(nbody_ctx* c, int order, double* pos, double* vel, double* mass, double* charge, int64_t* ids,
                    double* acc) {
    if (!c) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    NB_TRY(fetch(c, order ? 1 : 0));
    const int64_t n = c->n;
    double* st = DP<double>(c->stage);
    if (pos) NB_CU(c, cudaMemcpyAsync(pos, st, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->st));
    if (vel) NB_CU(c, cudaMemcpyAsync(vel, st + 3 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->st));
    if (mass) NB_CU(c, cudaMemcpyAsync(mass, st + 6 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
    if (charge) NB_CU(c, cudaMemcpyAsync(charge, st + 7 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
    if (ids) NB_CU(c, cudaMemcpyAsync(ids, st + 8 * n, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, c->st));
    if (acc) NB_CU(c, cudaMemcpyAsync(acc, st + 9 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    return NBODY_OK;
}

int nbody_step(nbody_ctx* c, int nsteps, double* t_out) {
    if (!c) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    if (nsteps < 0) return nb_fail(c, NBODY_ERR_INVALID, "nsteps must be >= 0");
    NB_CU(c, cudaSetDevice(c->device));
    if (nsteps > 0) c->ck_steps = 0;
    for (int s = 0; s < nsteps; ++s) {
        if (c->dt_mode == NBODY_DT_BLOCK) {
            NB_TRY(nb_block_step(c));
            c->dt_last = c->dt_max;
            c->time += c->dt_max;
            NB_TRY(nb_traj_capture(c));
            continue;
        }
        if (c->dt_mode == NBODY_DT_ADAPTIVE) {
            // this step's dt needs the largest acceleration at the current positions (leapfrog) or
            // of the last evaluation (Euler); without one, evaluate the forces first
            if (!c->amax_valid) {
                NB_TRY(nb_evaluate(c, 0, NB_INTEG_NONE, false));
                c->have_acc = c->prm.integrator == NBODY_INTEG_LEAPFROG;
            }
            c->prm.dt = adaptive_dt(c);
        }
        c->dt_last = c->prm.dt;
        if (c->prm.integrator == NBODY_INTEG_LEAPFROG) {
            if (!c->have_acc) {
                NB_TRY(nb_evaluate(c, 0, NB_INTEG_NONE, false));
                c->have_acc = true;
            }
            NB_TRY(nb_evaluate(c, 1, NB_INTEG_KDK_CLOSE, false));
        } else {
            NB_TRY(nb_evaluate(c, 0, NB_INTEG_EULER, false));
            c->have_acc = false;
        }
        c->time += c->prm.dt;
        NB_TRY(nb_traj_capture(c));
    }
    NB_CU(c, cudaStreamSynchronize(c->st));
    if (t_out) *t_out = c->time;
    return NBODY_OK;
}

int nbody_compute_forces(nbody_ctx* c, double* acc, double* pot) {
    if (!c) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    NB_CU(c, cudaSetDevice(c->device));
    NB_TRY(nb_evaluate(c, 0, NB_INTEG_NONE, pot != nullptr));
    c->have_acc = c->prm.integrator == NBODY_INTEG_LEAPFROG;
    if (acc || pot) {
        NB_TRY(fetch(c, 1));
        const int64_t n = c->n;
        double* st = DP<double>(c->stage);
        if (acc) NB_CU(c, cudaMemcpyAsync(acc, st + 9 * n, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->st));
        if (pot) NB_CU(c, cudaMemcpyAsync(pot, st + 12 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st));
    }
    NB_CU(c, cudaStreamSynchronize(c->st));
    return NBODY_OK;
}

int nbody_diagnostics(nbody_ctx* c, double* out) {
    if (!c || !out) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    NB_CU(c, cudaSetDevice(c->device));
    NB_TRY(nb_evaluate(c, 0, NB_INTEG_NONE, true));
    c->have_acc = c->prm.integrator == NBODY_INTEG_LEAPFROG;
    return c->rsz == 4 ? diag_t<float>(c, out) : diag_t<double>(c, out);
}

int nbody_get_stats(nbody_ctx* c, int64_t* out, int n) {
    if (!c || !out) return NBODY_ERR_INVALID;
    const int64_t v[11] = {(int64_t)c->h_stats[0], (int64_t)c->h_stats[1], (int64_t)c->h_stats[2], c->nnodes,
                           c->nleaves, c->depth, c->launches, c->escapes, c->blk_leaves, c->blk_active_leaves,
                           c->blk_evals};
    for (int i = 0; i < n && i < 11; ++i) out[i] = v[i];
    return NBODY_OK;
}

int nbody_tree_info(nbody_ctx* c, int64_t* n, int64_t* nnodes, int64_t* nleaves, int* depth) {
    if (!c) return NBODY_ERR_INVALID;
    if (n) *n = c->n;
    if (nnodes) *nnodes = c->nnodes;
    if (nleaves) *nleaves = c->nleaves;
    if (depth) *depth = c->depth;
    return NBODY_OK;
}

int nbody_get_tree(nbody_ctx* c, uint64_t* keys, int64_t* perm, int32_t* nodes) {
    if (!c) return NBODY_ERR_INVALID;
    if (c->nnodes == 0) return nb_fail(c, NBODY_ERR_STATE, "no tree built yet");
    NB_CU(c, cudaSetDevice(c->device));
    const int64_t n = c->n;
    if (keys) NB_CU(c, cudaMemcpyAsync(keys, c->keys[0].p, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, c->st));
    std::vector<uint32_t> ids;
    std::vector<NodeRec> nr;
    if (perm) {
        ids.resize(n);
        NB_CU(c, cudaMemcpyAsync(ids.data(), c->id[c->cur].p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, c->st));
    }
    if (nodes) {
        nr.resize(c->nnodes);
        NB_CU(c, cudaMemcpyAsync(nr.data(), c->nodes.p, sizeof(NodeRec) * c->nnodes, cudaMemcpyDeviceToHost, c->st));
    }
    NB_CU(c, cudaStreamSynchronize(c->st));
    if (perm)
        for (int64_t i = 0; i < n; ++i) perm[i] = ids[i];
    if (nodes)
        for (int64_t k = 0; k < c->nnodes; ++k) {
            int32_t* r = nodes + 9 * k;
            r[0] = nr[k].level; r[1] = (int32_t)nr[k].ix; r[2] = (int32_t)nr[k].iy; r[3] = (int32_t)nr[k].iz;
            r[4] = (int32_t)nr[k].begin; r[5] = (int32_t)nr[k].count; r[6] = nr[k].parent;
            r[7] = nr[k].child_begin; r[8] = nr[k].nchild;
        }
    return NBODY_OK;
}

int nbody_get_interactions(nbody_ctx* c, int which, int64_t* npairs, int32_t* pairs) {
    if (!c || !npairs || (which != 0 && which != 1)) return NBODY_ERR_INVALID;
    if (c->nnodes == 0) return nb_fail(c, NBODY_ERR_STATE, "no tree built yet");
    NB_CU(c, cudaSetDevice(c->device));
    const int64_t nn = c->nnodes;
    std::vector<uint32_t> off(nn), cnt(nn);
    const DevBuf& bo = which == 0 ? c->m2l_off : c->p2p_off;
    const DevBuf& bc = which == 0 ? c->m2l_cnt : c->p2p_cnt;
    const DevBuf& bl = which == 0 ? c->m2l_list : c->p2p_list;
    NB_CU(c, cudaMemcpyAsync(off.data(), bo.p, sizeof(uint32_t) * nn, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaMemcpyAsync(cnt.data(), bc.p, sizeof(uint32_t) * nn, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    int64_t total = 0;
    for (int64_t k = 0; k < nn; ++k) total += cnt[k];
    *npairs = total;
    if (pairs) {
        uint32_t tail = (uint32_t)c->h_info[which == 0 ? INFO_M2L_TAIL : INFO_P2P_TAIL];
        std::vector<uint32_t> list(tail ? tail : 1);
        if (tail)
            NB_CU(c, cudaMemcpyAsync(list.data(), bl.p, sizeof(uint32_t) * tail, cudaMemcpyDeviceToHost, c->st));
        NB_CU(c, cudaStreamSynchronize(c->st));
        int64_t o = 0;
        for (int64_t k = 0; k < nn; ++k)
            for (uint32_t j = 0; j < cnt[k]; ++j) {
                pairs[2 * o] = (int32_t)k;
                pairs[2 * o + 1] = (int32_t)list[off[k] + j];
                ++o;
            }
    }
    return NBODY_OK;
}

int nbody_set_timing(nbody_ctx* c, int on) {
    if (!c) return NBODY_ERR_INVALID;
    c->timing = on != 0;
    return NBODY_OK;
}

int nbody_phase_times(nbody_ctx* c, float* ms, int n) {
    if (!c || !ms) return NBODY_ERR_INVALID;
    for (int i = 0; i < n && i < 12; ++i) ms[i] = c->phase_ms[i];
    return NBODY_OK;
}

void* nbody_stream(nbody_ctx* c) { return c ? (void*)c->st : nullptr; }

int nbody_device_memory(nbody_ctx* c, int64_t* current, int64_t* peak) {
    if (!c) return NBODY_ERR_INVALID;
    if (current) *current = (int64_t)c->dev_bytes;
    if (peak) *peak = (int64_t)c->dev_peak;
    return NBODY_OK;
}

int nbody_set_timestep_control(nbody_ctx* c, int mode, double eta, double length, double dt_min, double dt_max) {
    if (!c) return NBODY_ERR_INVALID;
    if (mode == NBODY_DT_FIXED) {
        if (c->dt_mode != NBODY_DT_FIXED) c->prm.dt = c->dt_base;
        c->dt_mode = NBODY_DT_FIXED;
        c->amax_valid = false;
        return NBODY_OK;
    }
    if (mode != NBODY_DT_ADAPTIVE && mode != NBODY_DT_BLOCK)
        return nb_fail(c, NBODY_ERR_INVALID, "mode must be NBODY_DT_FIXED, NBODY_DT_ADAPTIVE or NBODY_DT_BLOCK");
    int K = 0;
    if (mode == NBODY_DT_BLOCK) {
        if (c->prm.integrator != NBODY_INTEG_LEAPFROG)
            return nb_fail(c, NBODY_ERR_INVALID, "block time steps need the leapfrog integrator");
        const double r = dt_max / dt_min;
        while (K < 20 && (double)(1 << K) < r * (1.0 - 1e-12)) ++K;
        if (!(dt_min > 0.0) || !(std::fabs((double)(1 << K) - r) <= 1e-9 * r))
            return nb_fail(c, NBODY_ERR_INVALID, "block steps need dt_max / dt_min = 2^K, K <= 20");
    }
    if (!(eta > 0.0) || !std::isfinite(eta)) return nb_fail(c, NBODY_ERR_INVALID, "eta must be > 0");
    if (!(dt_min > 0.0) || !(dt_max >= dt_min) || !std::isfinite(dt_max))
        return nb_fail(c, NBODY_ERR_INVALID, "need 0 < dt_min <= dt_max < inf");
    if (!(length > 0.0) && !(c->prm.eps > 0.0))
        return nb_fail(c, NBODY_ERR_INVALID, "length must be > 0 when the softening eps is 0");
    if (!std::isfinite(length)) return nb_fail(c, NBODY_ERR_INVALID, "length must be finite");
    NB_CU(c, cudaSetDevice(c->device));
    NB_TRY(nb_grow(c, c->amax, sizeof(unsigned long long)));
    if (!c->h_amax) NB_CU(c, cudaMallocHost(&c->h_amax, sizeof(double)));
    if (c->dt_mode == NBODY_DT_FIXED) c->dt_base = c->prm.dt;
    c->dt_mode = mode;
    c->blk_K = K;
    if (mode == NBODY_DT_BLOCK) c->prm.dt = dt_max;
    c->dt_eta = eta;
    c->dt_len = length;
    c->dt_min = dt_min;
    c->dt_max = dt_max;
    c->amax_valid = false;
    return NBODY_OK;
}

int nbody_set_escape_policy(nbody_ctx* c, int policy) {
    if (!c) return NBODY_ERR_INVALID;
    if (policy != NBODY_ESCAPE_GROW && policy != NBODY_ESCAPE_ERROR)
        return nb_fail(c, NBODY_ERR_INVALID, "policy must be NBODY_ESCAPE_GROW or NBODY_ESCAPE_ERROR");
    c->escape_policy = policy;
    return NBODY_OK;
}

int nbody_set_wait_limits(nbody_ctx* c, int64_t scan_polls, int64_t copy_cycles) {
    if (!c) return NBODY_ERR_INVALID;
    c->scan_polls = scan_polls > 0 ? scan_polls : NB_SCAN_POLLS;
    c->copy_cycles = copy_cycles > 0 ? (long long)copy_cycles : NB_COPY_CYCLES;
    return NBODY_OK;
}

int nbody_selftest_wait(nbody_ctx* c, int which) {
    if (!c) return NBODY_ERR_INVALID;
    if (which != 0 && which != 1) return nb_fail(c, NBODY_ERR_INVALID, "which must be 0 (scan) or 1 (copy)");
    NB_CU(c, cudaSetDevice(c->device));
    return which == 0 ? nb_scan_wait_selftest(c) : nb_copy_wait_selftest(c);
}

int nbody_last_timestep(nbody_ctx* c, double* dt) {
    if (!c || !dt) return NBODY_ERR_INVALID;
    *dt = c->dt_last > 0.0 ? c->dt_last : c->prm.dt;
    return NBODY_OK;
}

int nbody_get_time(nbody_ctx* c, double* t) {
    if (!c || !t) return NBODY_ERR_INVALID;
    *t = c->time;
    return NBODY_OK;
}

int nbody_debug_bounds(void) {
#ifdef NBODY_DEBUG_BOUNDS
    return 1;
#else
    return 0;
#endif
}

const char* nbody_last_error(nbody_ctx* c) { return c ? c->err.c_str() : g_create_err.c_str(); }

}  // extern "C"
