// FP64 softened direct sum on the device (the accuracy reference for the FMM)
// and an FMA-chain microbenchmark for the FP32 / FP64 pipe peaks that the
// roofline of the FMM kernels is reported against.
#include <algorithm>

#include "nbody_internal.cuh"

namespace {

constexpr int DT = 128;   // targets per block
constexpr int DS = 128;   // sources per shared tile

template <typename R>
__global__ void __launch_bounds__(DT) k_direct(int64_t n, const R* __restrict__ x, const R* __restrict__ y,
                                               const R* __restrict__ z, const R* __restrict__ q, int64_t nt,
                                               const int32_t* __restrict__ trow, int nsplit, double eps2,
                                               double* __restrict__ part) {
    __shared__ double sx[DS], sy[DS], sz[DS], sq[DS];
    const int64_t t = (int64_t)blockIdx.x * DT + threadIdx.x;
    const int split = blockIdx.y;
    const int64_t j0 = n * split / nsplit, j1 = n * (split + 1) / nsplit;
    int64_t row = -1;
    double xi = 0, yi = 0, zi = 0;
    if (t < nt) {
        row = trow[t];
        xi = x[row]; yi = y[row]; zi = z[row];
    }
    double ex = 0, ey = 0, ez = 0, ps = 0;
    for (int64_t b = j0; b < j1; b += DS) {
        const int64_t j = b + threadIdx.x;
        if (j < j1) { sx[threadIdx.x] = x[j]; sy[threadIdx.x] = y[j]; sz[threadIdx.x] = z[j]; sq[threadIdx.x] = q[j]; }
        __syncthreads();
        const int cnt = (int)(j1 - b < DS ? j1 - b : DS);
        for (int k = 0; k < cnt; ++k) {
            if (b + k == row) continue;
            const double dx = sx[k] - xi, dy = sy[k] - yi, dz = sz[k] - zi;
            const double s = dx * dx + dy * dy + dz * dz + eps2;
            if (s == 0.0) continue;
            const double inv = 1.0 / sqrt(s), w = sq[k] * inv * inv * inv;
            ex += w * dx; ey += w * dy; ez += w * dz; ps += sq[k] * inv;
        }
        __syncthreads();
    }
    if (t < nt) {
        double* o = part + ((int64_t)t * nsplit + split) * 4;
        o[0] = ex; o[1] = ey; o[2] = ez; o[3] = ps;
    }
}

template <typename R>
__global__ void k_direct_final(int64_t nt, const int32_t* __restrict__ trow, int nsplit, const double* __restrict__ part,
                               const R* __restrict__ m, const R* __restrict__ q, double G, double* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double e[4] = {0, 0, 0, 0};
    for (int s = 0; s < nsplit; ++s)
        for (int k = 0; k < 4; ++k) e[k] += part[((int64_t)t * nsplit + s) * 4 + k];
    const int64_t row = trow[t];
    const double f = G * (double)q[row] / (double)m[row];
    out[4 * t] = f * e[0]; out[4 * t + 1] = f * e[1]; out[4 * t + 2] = f * e[2]; out[4 * t + 3] = -G * e[3];
}

__global__ void k_rows(int64_t n, const uint32_t* __restrict__ id, int32_t* __restrict__ row_of) {
    const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (i < n) row_of[id[i]] = (int32_t)i;
}

__global__ void k_pick(int64_t nt, const int64_t* __restrict__ tgt, const int32_t* __restrict__ row_of,
                       int32_t* __restrict__ trow) {
    const int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (t < nt) trow[t] = row_of[tgt[t]];
}

template <typename R>
int direct_t(nbody_ctx* c, int64_t nt, const int64_t* tgt_host, double* acc, double* pot) {
    const int64_t n = c->n;
    const int k = c->cur;
    const int nsplit = (int)std::max<int64_t>(1, std::min<int64_t>(256, (4 * 152 * 8 * DT) / std::max<int64_t>(nt, 1)));
    NB_TRY(nb_grow(c, c->stage, sizeof(double) * 13 * (size_t)n));
    const size_t need = sizeof(int64_t) * nt + sizeof(int32_t) * (n + nt) + sizeof(double) * 4 * nt * (nsplit + 1);
    DevBuf& scratch = c->diag;
    NB_TRY(nb_grow(c, scratch, need + 64));
    char* base = (char*)scratch.p;
    int64_t* tgt = (int64_t*)base;
    int32_t* row_of = (int32_t*)(tgt + nt);
    int32_t* trow = row_of + n;
    double* part = (double*)(((uintptr_t)(trow + nt) + 15) & ~(uintptr_t)15);
    double* out = part + 4 * nt * nsplit;
    NB_CU(c, cudaMemcpyAsync(tgt, tgt_host, sizeof(int64_t) * nt, cudaMemcpyHostToDevice, c->st));
    k_rows<<<(unsigned)((n + 255) / 256), 256, 0, c->st>>>(n, DP<uint32_t>(c->id[k]), row_of);
    k_pick<<<(unsigned)((nt + 255) / 256), 256, 0, c->st>>>(nt, tgt, row_of, trow);
    dim3 g((unsigned)((nt + DT - 1) / DT), (unsigned)nsplit);
    k_direct<R><<<g, DT, 0, c->st>>>(n, DP<R>(c->x[k]), DP<R>(c->y[k]), DP<R>(c->z[k]), DP<R>(c->q[k]), nt, trow,
                                     nsplit, c->prm.eps * c->prm.eps, part);
    k_direct_final<R><<<(unsigned)((nt + 127) / 128), 128, 0, c->st>>>(nt, trow, nsplit, part, DP<R>(c->m[k]),
                                                                         DP<R>(c->q[k]), c->prm.G, out);
    NB_LAUNCHED(c, "direct");
    std::vector<double> h(4 * nt);
    NB_CU(c, cudaMemcpyAsync(h.data(), out, sizeof(double) * 4 * nt, cudaMemcpyDeviceToHost, c->st));
    NB_CU(c, cudaStreamSynchronize(c->st));
    for (int64_t t = 0; t < nt; ++t) {
        if (acc) { acc[3 * t] = h[4 * t]; acc[3 * t + 1] = h[4 * t + 1]; acc[3 * t + 2] = h[4 * t + 2]; }
        if (pot) pot[t] = h[4 * t + 3];
    }
    return NBODY_OK;
}

// FMA throughput: NC independent chains per thread, all in registers
template <typename T, int NC>
__global__ void k_fma_chain(T* out, int iters, T a, T b) {
    T v[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k) v[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < NC; ++k) v[k] = fma(v[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < NC; ++k) s += v[k];
    if (s == (T)-1.2345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T, int NC>
double time_fma(int blocks, int threads, int iters, T* scratch) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_chain<T, NC><<<blocks, threads>>>(scratch, iters / 4, (T)0.999999, (T)1e-7);
    cudaEventRecord(e0);
    k_fma_chain<T, NC><<<blocks, threads>>>(scratch, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 2.0 * NC * (double)iters * blocks * threads / (ms * 1e-3) / 1e9;
}

}  // namespace

extern "C" int nbody_direct_forces(nbody_ctx* c, int64_t nt, const int64_t* targets, double* acc, double* pot) {
    if (!c || !targets || nt < 0) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    for (int64_t t = 0; t < nt; ++t)
        if (targets[t] < 0 || targets[t] >= c->n) return nb_fail(c, NBODY_ERR_INVALID, "target index out of range");
    if (nt == 0) return NBODY_OK;
    NB_CU(c, cudaSetDevice(c->device));
    return c->rsz == 4 ? direct_t<float>(c, nt, targets, acc, pot) : direct_t<double>(c, nt, targets, acc, pot);
}

extern "C" int nbody_measure_peaks(int device, double* out) {
    if (!out) return NBODY_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return NBODY_ERR_NO_DEVICE;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    void* scratch = nullptr;
    if (cudaMalloc(&scratch, (size_t)sms * 64 * 256 * sizeof(double)) != cudaSuccess) return NBODY_ERR_NOMEM;
    out[0] = time_fma<float, 16>(sms * 8, 256, 1 << 16, (float*)scratch);
    out[1] = time_fma<double, 8>(sms * 8, 256, 1 << 12, (double*)scratch);
    cudaFree(scratch);
    return cudaGetLastError() == cudaSuccess ? NBODY_OK : NBODY_ERR_CUDA;
}
