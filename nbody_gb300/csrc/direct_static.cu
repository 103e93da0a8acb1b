// nbody_direct_forces_static: the FP64 softened direct sum of direct.cu for
// callers that cannot allocate device memory.
//
// Some callers must not call cudaMalloc: code that runs under a host
// framework which owns the device memory budget (its caching allocator would
// be bypassed and its accounting broken), and code on latency-critical paths
// where an allocation's implicit synchronization or failure under memory
// pressure is not acceptable.  This entry point takes device-resident inputs
// and outputs from the caller and keeps its only scratch -- the per-split
// partial sums -- in the file-scope array below, which every GPU that loads
// the library holds until the process exits.
//
// Limits and sharing:
//   - at most NB_STATIC_TARGETS targets per call (larger calls are rejected
//     with NBODY_ERR_INVALID; nbody_last_error(NULL) gives the message);
//   - target indices outside [0, n) give NaN for that target, with no
//     out-of-bounds access;
//   - every call on a device uses the same array, which keeps the previous
//     call's contents; the kernels overwrite every slot they read, so nothing
//     has to start at zero;
//   - two calls whose kernels overlap on the GPU (different streams without
//     ordering, or different host threads) race on the array and corrupt
//     each other's results: callers must order them.
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before any stream capture on the device.  A later call
//     checks that the cached address still belongs to that device (after a
//     cudaDeviceReset the module is loaded again and the address is looked up
//     again);
//   - the call selects `device` for its own launches and gives the calling
//     thread back the device that was current before, on every return path.
#include <mutex>

#include "nbody_internal.cuh"

#define NB_STATIC_TARGETS 131072             // targets per call
#define NB_STATIC_SLOTS NB_STATIC_TARGETS    // (target, split) partial-sum slots
#define NB_STATIC_MAX_DEVICES 64

static __device__ __align__(256) double g_direct_scratch[(size_t)NB_STATIC_SLOTS * 4];

namespace {

std::mutex g_static_mu;
double* g_static_ptr[NB_STATIC_MAX_DEVICES] = {nullptr};

constexpr int ST = 128;   // targets per block and sources per tile

__global__ void __launch_bounds__(ST) k_direct_aos(int64_t n, const double* __restrict__ pos,
                                                   const double* __restrict__ q, int64_t nt,
                                                   const int64_t* __restrict__ tgt, int nsplit, double eps2,
                                                   double* __restrict__ part) {
    __shared__ double sx[ST], sy[ST], sz[ST], sq[ST];
    const int64_t t = (int64_t)blockIdx.x * ST + threadIdx.x;
    const int split = blockIdx.y;
    const int64_t j0 = n * split / nsplit, j1 = n * (split + 1) / nsplit;
    int64_t row = -1;
    double xi = 0, yi = 0, zi = 0;
    if (t < nt) {
        row = tgt[t];
        if (row < 0 || row >= n) row = -1;   // out-of-range target: no access, NaN result
        else { xi = pos[3 * row]; yi = pos[3 * row + 1]; zi = pos[3 * row + 2]; }
    }
    double ex = 0, ey = 0, ez = 0, ps = 0;
    for (int64_t b = j0; b < j1; b += ST) {
        const int64_t j = b + threadIdx.x;
        if (j < j1) {
            sx[threadIdx.x] = pos[3 * j]; sy[threadIdx.x] = pos[3 * j + 1]; sz[threadIdx.x] = pos[3 * j + 2];
            sq[threadIdx.x] = q[j];
        }
        __syncthreads();
        const int cnt = (int)(j1 - b < ST ? j1 - b : ST);
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

__global__ void k_direct_aos_final(int64_t n, int64_t nt, const int64_t* __restrict__ tgt, int nsplit,
                                   const double* __restrict__ part, const double* __restrict__ m,
                                   const double* __restrict__ q, double G, double* __restrict__ acc,
                                   double* __restrict__ pot) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double e[4] = {0, 0, 0, 0};
    for (int s = 0; s < nsplit; ++s)
        for (int k = 0; k < 4; ++k) e[k] += part[((int64_t)t * nsplit + s) * 4 + k];
    const int64_t row = tgt[t];
    if (row < 0 || row >= n) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        acc[3 * t] = nan; acc[3 * t + 1] = nan; acc[3 * t + 2] = nan;
        if (pot) pot[t] = nan;
        return;
    }
    const double f = G * q[row] / m[row];
    acc[3 * t] = f * e[0]; acc[3 * t + 1] = f * e[1]; acc[3 * t + 2] = f * e[2];
    if (pot) pot[t] = -G * e[3];
}

// failures are reported like nbody_create's: nbody_last_error(NULL) returns the message
int fail(int code, const char* msg) { return nb_fail(nullptr, code, msg); }


// the device address of the scratch array on the current device (`device`), looked up once per
// device and checked again on later calls: after a cudaDeviceReset the cached address is stale
double* scratch_on(int device) {
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (g_static_ptr[device]) {
        cudaPointerAttributes at;
        const cudaError_t e = cudaPointerGetAttributes(&at, g_static_ptr[device]);
        if (e == cudaSuccess && at.type == cudaMemoryTypeDevice && at.device == device) return g_static_ptr[device];
        cudaGetLastError();
        g_static_ptr[device] = nullptr;
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_direct_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return nullptr;
    }
    g_static_ptr[device] = (double*)p;
    return g_static_ptr[device];
}

int direct_static(int device, int64_t n, const double* pos, const double* mass, const double* charge, double eps,
                  double G, int64_t nt, const int64_t* targets, double* acc, double* pot, void* stream) {
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return fail(NBODY_ERR_NO_DEVICE, "nbody_direct_forces_static: cannot select the device");
    }
    double* scratch = scratch_on(device);
    if (!scratch) return fail(NBODY_ERR_CUDA, "nbody_direct_forces_static: cudaGetSymbolAddress failed");
    int64_t ns = NB_STATIC_SLOTS / nt;
    const int nsplit = (int)(ns > 64 ? 64 : (ns < 1 ? 1 : ns));
    cudaStream_t st = (cudaStream_t)stream;
    dim3 g((unsigned)((nt + ST - 1) / ST), (unsigned)nsplit);
    k_direct_aos<<<g, ST, 0, st>>>(n, pos, charge ? charge : mass, nt, targets, nsplit, eps * eps, scratch);
    k_direct_aos_final<<<(unsigned)((nt + 127) / 128), 128, 0, st>>>(n, nt, targets, nsplit, scratch, mass,
                                                                       charge ? charge : mass, G, acc, pot);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(NBODY_ERR_CUDA, cudaGetErrorString(e));
    return NBODY_OK;
}

}  // namespace

extern "C" int nbody_direct_forces_static(int device, int64_t n, const double* pos, const double* mass,
                                          const double* charge, double eps, double G, int64_t nt,
                                          const int64_t* targets, double* acc, double* pot, void* stream) {
    if (n < 1 || !pos || !mass || nt < 0 || (nt > 0 && (!targets || !acc)))
        return fail(NBODY_ERR_INVALID, "nbody_direct_forces_static: n >= 1 and non-null pos, mass, targets, acc");
    if (nt > NB_STATIC_TARGETS)
        return fail(NBODY_ERR_INVALID, "nbody_direct_forces_static: more than 131072 targets in one call");
    if (device < 0 || device >= NB_STATIC_MAX_DEVICES)
        return fail(NBODY_ERR_INVALID, "nbody_direct_forces_static: device ordinal out of range");
    if (nt == 0) return NBODY_OK;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        prev = -1;
    }
    const int rc = direct_static(device, n, pos, mass, charge, eps, G, nt, targets, acc, pot, stream);
    if (prev >= 0 && prev != device) {
        cudaSetDevice(prev);
        cudaGetLastError();
    }
    return rc;
}
