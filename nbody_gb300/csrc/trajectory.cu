// Trajectory output: the reference's per-step CSV dump (src/main.cpp:77-101:
// one row per step, the time then x, y, z of every particle) written from the
// library every `every` steps, without stalling the step loop.  Positions are
// gathered on the device (input or leaf order) and copied into one of a few
// pinned host slots; a writer thread formats the rows while the GPU keeps
// stepping, and a step only waits when every slot is still being written.
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <new>
#include <thread>

#include "nbody_internal.cuh"

struct nb_traj {
    static constexpr int SLOTS = 3;
    std::FILE* f = nullptr;
    int every = 1, order = 0, digits = 6, device = 0;
    int64_t n = 0, steps = 0;
    double* slot[SLOTS] = {};
    double slot_time[SLOTS] = {};
    cudaEvent_t ready[SLOTS] = {};
    bool busy[SLOTS] = {};
    int next = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int> queue;
    bool stop = false;
    bool io_error = false;
    std::thread writer;
};

namespace {

constexpr int TB = 256;

// positions in input order (order = 1, through the ids) or in the current leaf order
template <typename R>
__global__ void k_traj_positions(int64_t n, int order, const R* __restrict__ x, const R* __restrict__ y,
                                 const R* __restrict__ z, const uint32_t* __restrict__ id, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * TB + threadIdx.x;
    if (i >= n) return;
    const int64_t o = order ? (int64_t)id[i] : i;
    out[3 * o] = (double)x[i];
    out[3 * o + 1] = (double)y[i];
    out[3 * o + 2] = (double)z[i];
}

void writer_loop(nb_traj* T) {
    cudaSetDevice(T->device);
    for (;;) {
        int k;
        {
            std::unique_lock<std::mutex> lk(T->mu);
            T->cv.wait(lk, [&] { return !T->queue.empty() || T->stop; });
            if (T->queue.empty()) return;
            k = T->queue.front();
            T->queue.pop_front();
        }
        cudaEventSynchronize(T->ready[k]);
        bool ok = std::fprintf(T->f, "%.*g", T->digits, T->slot_time[k]) > 0;
        const double* p = T->slot[k];
        for (int64_t i = 0; i < 3 * T->n && ok; ++i) ok = std::fprintf(T->f, ",%.*g", T->digits, p[i]) > 0;
        ok = ok && std::fputc('\n', T->f) != EOF;
        {
            std::lock_guard<std::mutex> lk(T->mu);
            if (!ok) T->io_error = true;
            T->busy[k] = false;
        }
        T->cv.notify_all();
    }
}

void traj_free(nb_traj* T) {
    for (int k = 0; k < nb_traj::SLOTS; ++k) {
        if (T->slot[k]) cudaFreeHost(T->slot[k]);
        if (T->ready[k]) cudaEventDestroy(T->ready[k]);
    }
    if (T->f) std::fclose(T->f);
    delete T;
}

}  // namespace

// called by nbody_step after each step
int nb_traj_capture(nbody_ctx* c) {
    nb_traj* T = c->traj;
    if (!T || ++T->steps % T->every) return NBODY_OK;
    const int k = T->next;
    {
        std::unique_lock<std::mutex> lk(T->mu);
        T->cv.wait(lk, [&] { return !T->busy[k]; });
        T->busy[k] = true;
    }
    T->next = (k + 1) % nb_traj::SLOTS;
    // slot k is ours until it is queued: on a failure below, hand it back before returning so a
    // later capture does not wait for a row that will never be written
    auto release_slot = [&](int rc) {
        {
            std::lock_guard<std::mutex> lk(T->mu);
            T->busy[k] = false;
        }
        T->cv.notify_all();
        return rc;
    };
    double* st = DP<double>(c->stage);
    const int cur = c->cur;
    const unsigned g = (unsigned)((c->n + TB - 1) / TB);
    if (c->rsz == 4)
        k_traj_positions<float><<<g, TB, 0, c->st>>>(c->n, T->order, DP<float>(c->x[cur]), DP<float>(c->y[cur]),
                                                     DP<float>(c->z[cur]), DP<uint32_t>(c->id[cur]), st);
    else
        k_traj_positions<double><<<g, TB, 0, c->st>>>(c->n, T->order, DP<double>(c->x[cur]), DP<double>(c->y[cur]),
                                                      DP<double>(c->z[cur]), DP<uint32_t>(c->id[cur]), st);
    if (int rc = nb_cuda(c, cudaGetLastError(), "trajectory positions")) return release_slot(rc);
    if (int rc = nb_cuda(c, cudaMemcpyAsync(T->slot[k], st, sizeof(double) * 3 * c->n, cudaMemcpyDeviceToHost, c->st),
                         "trajectory copy"))
        return release_slot(rc);
    if (int rc = nb_cuda(c, cudaEventRecord(T->ready[k], c->st), "trajectory event")) return release_slot(rc);
    T->slot_time[k] = c->time;
    {
        std::lock_guard<std::mutex> lk(T->mu);
        T->queue.push_back(k);
    }
    T->cv.notify_all();
    return NBODY_OK;
}

// flushes and closes the writer (also called by nbody_destroy); the first I/O error is reported
int nb_traj_close(nbody_ctx* c) {
    nb_traj* T = c->traj;
    if (!T) return NBODY_OK;
    c->traj = nullptr;
    {
        std::lock_guard<std::mutex> lk(T->mu);
        T->stop = true;
    }
    T->cv.notify_all();
    if (T->writer.joinable()) T->writer.join();
    const bool err = T->io_error || std::fflush(T->f) != 0;
    traj_free(T);
    return err ? nb_fail(c, NBODY_ERR_STATE, "trajectory file write failed") : NBODY_OK;
}

extern "C" {

int nbody_trajectory_open(nbody_ctx* c, const char* path, int every, int order, int digits) {
    if (!c || !path) return NBODY_ERR_INVALID;
    if (c->n == 0) return nb_fail(c, NBODY_ERR_STATE, "no particles");
    if (every < 1 || (order != 0 && order != 1) || digits < 1 || digits > 17)
        return nb_fail(c, NBODY_ERR_INVALID, "every >= 1, order 0 or 1, digits 1..17");
    NB_TRY(nb_traj_close(c));
    NB_CU(c, cudaSetDevice(c->device));
    nb_traj* T = new (std::nothrow) nb_traj();
    if (!T) return nb_fail(c, NBODY_ERR_NOMEM, "host allocation failed");
    T->every = every;
    T->order = order;
    T->digits = digits;
    T->device = c->device;
    T->n = c->n;
    T->f = std::fopen(path, "w");
    if (!T->f) {
        traj_free(T);
        return nb_fail(c, NBODY_ERR_INVALID, std::string("cannot open ") + path);
    }
    for (int k = 0; k < nb_traj::SLOTS; ++k) {
        int rc = nb_cuda(c, cudaMallocHost(&T->slot[k], sizeof(double) * 3 * (size_t)c->n), "cudaMallocHost");
        if (!rc) rc = nb_cuda(c, cudaEventCreateWithFlags(&T->ready[k], cudaEventDisableTiming), "cudaEventCreate");
        if (rc) {
            traj_free(T);
            return rc;
        }
    }
    T->writer = std::thread(writer_loop, T);
    c->traj = T;
    return NBODY_OK;
}

int nbody_trajectory_close(nbody_ctx* c) {
    if (!c) return NBODY_ERR_INVALID;
    NB_CU(c, cudaSetDevice(c->device));
    return nb_traj_close(c);
}

}  // extern "C"
