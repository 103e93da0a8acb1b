/*
 * nbody/cuda_simulation.h -- nbody::CudaSimulation, the GB300 drop-in for
 * nbody::OpenClSimulation (include/nbody/open_cl_simulation.h:19-203 of
 * duanebyer/nbody).  Header-only; link with libnbody_gb300.so.
 *
 * Same constructor as the reference, (bounds, particles, timeStep, log), with
 * the reference's defaults (order-1 expansion, leaf capacity 8, theta 0.5,
 * softening 0.01, G = 1, single precision, explicit Euler, root box
 * [0, bounds)); an overload takes an nbody_params for the other forms.
 * step() returns the new time; particles() returns the particles in octree
 * leaf (Morton) order like the reference's (src/open_cl_simulation.cpp:53-68).
 * Failures throw std::runtime_error carrying the library's message, as the
 * reference throws std::runtime_error (src/open_cl_simulation.cpp:630,648,767).
 *
 * A program written against the reference switches by changing its typedef:
 *     using Simulation = nbody::CudaSimulation;
 */
#ifndef NBODY_CUDA_SIMULATION_H
#define NBODY_CUDA_SIMULATION_H

#include <algorithm>
#include <initializer_list>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "nbody/simulation.h"
#include "nbody_gb300.h"

namespace nbody {
namespace cuda {

/* 4-float vector indexed like the reference's device::vector_t
   (include/nbody/device/types.h:49-74): brace-initialised, operator[]. */
class alignas(16) vector_t final {
    float _v[4];

public:
    vector_t() : _v{0, 0, 0, 0} {}
    vector_t(std::initializer_list<float> list) : _v{0, 0, 0, 0} {
        unsigned i = 0;
        for (float x : list) {
            if (i < 4) _v[i++] = x;
        }
    }
    float& operator[](unsigned i) { return _v[i]; }
    float const& operator[](unsigned i) const { return _v[i]; }
};

}  // namespace cuda

class CudaSimulation final : public Simulation<float, cuda::vector_t> {
    nbody_ctx* _ctx = nullptr;
    std::ostream& _log;
    int64_t _n = 0;

    void check(int rc, const char* what) const {
        if (rc != NBODY_OK) {
            const char* msg = nbody_last_error(_ctx);
            throw std::runtime_error(std::string(what) + ": " + (msg ? msg : ""));
        }
    }

    static nbody_params defaults(Vector bounds) {
        nbody_params p;
        nbody_default_params(&p);
        p.fixed_box = 1;
        p.box_min[0] = p.box_min[1] = p.box_min[2] = 0.0;
        p.box_size = std::max(std::max(bounds[0], bounds[1]), bounds[2]);
        return p;
    }

    void init(nbody_params p, std::vector<Particle> const& particles, Scalar timeStep) {
        p.dt = timeStep;
        int rc = nbody_create(&p, &_ctx);
        if (rc != NBODY_OK) throw std::runtime_error(std::string("nbody_create: ") + nbody_last_error(nullptr));
        _n = (int64_t)particles.size();
        std::vector<double> pos(3 * _n), vel(3 * _n), mass(_n), charge(_n);
        for (int64_t i = 0; i < _n; ++i) {
            for (int d = 0; d < 3; ++d) {
                pos[3 * i + d] = particles[i].position[d];
                vel[3 * i + d] = particles[i].velocity[d];
            }
            mass[i] = particles[i].mass;
            charge[i] = particles[i].charge;
        }
        if (_n > 0)
            check(nbody_set_state(_ctx, _n, pos.data(), vel.data(), mass.data(), charge.data(), nullptr),
                  "nbody_set_state");
    }

    std::vector<Particle> fetch(int order) const {
        std::vector<Particle> out;
        if (_n == 0) return out;
        std::vector<double> pos(3 * _n), vel(3 * _n), mass(_n), charge(_n);
        check(nbody_get_state(_ctx, order, pos.data(), vel.data(), mass.data(), charge.data(), nullptr, nullptr),
              "nbody_get_state");
        out.reserve(_n);
        for (int64_t i = 0; i < _n; ++i) {
            Vector p = {(float)pos[3 * i], (float)pos[3 * i + 1], (float)pos[3 * i + 2], 0.0f};
            Vector v = {(float)vel[3 * i], (float)vel[3 * i + 1], (float)vel[3 * i + 2], 0.0f};
            out.push_back(Particle(p, v, (Scalar)mass[i], (Scalar)charge[i]));
        }
        return out;
    }

public:
    CudaSimulation(Vector bounds, std::vector<Particle> particles, Scalar timeStep, std::ostream& log) : _log(log) {
        _log << "Initializing CUDA.\n";
        init(defaults(bounds), particles, timeStep);
    }

    CudaSimulation(Vector bounds, std::vector<Particle> particles, Scalar timeStep, std::ostream& log,
                   nbody_params params)
        : _log(log) {
        if (params.fixed_box) {
            nbody_params d = defaults(bounds);
            params.box_size = d.box_size;
            params.box_min[0] = params.box_min[1] = params.box_min[2] = 0.0;
        }
        init(params, particles, timeStep);
    }

    CudaSimulation(CudaSimulation const&) = delete;
    CudaSimulation& operator=(CudaSimulation const&) = delete;

    ~CudaSimulation() { nbody_destroy(_ctx); }

    Scalar step() override {
        double t = 0.0;
        check(nbody_step(_ctx, 1, &t), "nbody_step");
        return (Scalar)t;
    }

    std::vector<Particle> particles() const override { return fetch(0); }

    /* additions beyond the reference interface */
    std::vector<Particle> particlesInInputOrder() const { return fetch(1); }

    /* accelerations (n x 3, input order) at the current positions */
    std::vector<double> computeForces() {
        std::vector<double> acc(3 * _n);
        check(nbody_compute_forces(_ctx, acc.data(), nullptr), "nbody_compute_forces");
        return acc;
    }

    /* FP64 diagnostics of the current state (nbody_diagnostics: kinetic and potential energy,
       momentum, angular momentum, mass) */
    std::vector<double> diagnostics() {
        std::vector<double> out(9);
        check(nbody_diagnostics(_ctx, out.data()), "nbody_diagnostics");
        return out;
    }

    /* adjoint of one force evaluation: for S = sum_i mu_i . a_i (mu n x 3, input order) fills
       dS/dx (n x 3), dS/dq and dS/dm (n) */
    void forceVjp(std::vector<double> const& mu, std::vector<double>& gx, std::vector<double>& gq,
                  std::vector<double>& gm) {
        gx.assign(3 * _n, 0.0);
        gq.assign(_n, 0.0);
        gm.assign(_n, 0.0);
        check(nbody_force_vjp(_ctx, mu.data(), gx.data(), gq.data(), gm.data()), "nbody_force_vjp");
    }

    /* nsteps leapfrog steps recorded for backward(): snapshots every `every` steps, or every
       evaluation kept whole with every = 0; returns the time after the last step */
    Scalar forwardCheckpointed(int nsteps, int every) {
        double t = 0.0;
        check(nbody_forward_checkpointed(_ctx, nsteps, every, &t), "nbody_forward_checkpointed");
        return (Scalar)t;
    }

    /* reverse sweep of the recorded run: from dL/dx_N and dL/dv_N (n x 3, input order; empty =
       zero) to dL/dx_0, dL/dv_0 (n x 3), dL/dq and dL/dm (n) */
    void backward(std::vector<double> const& gxT, std::vector<double> const& gvT, std::vector<double>& gx0,
                  std::vector<double>& gv0, std::vector<double>& gq, std::vector<double>& gm) {
        gx0.assign(3 * _n, 0.0);
        gv0.assign(3 * _n, 0.0);
        gq.assign(_n, 0.0);
        gm.assign(_n, 0.0);
        check(nbody_backward(_ctx, gxT.empty() ? nullptr : gxT.data(), gvT.empty() ? nullptr : gvT.data(),
                             gx0.data(), gv0.data(), gq.data(), gm.data()),
              "nbody_backward");
    }

    /* trajectory file in the row format of the reference's particles.csv, one row every `every`
       steps (order 0: leaf order as particles(), 1: input order) */
    void writeTrajectory(const char* path, int every = 1, int order = 0, int digits = 6) {
        check(nbody_trajectory_open(_ctx, path, every, order, digits), "nbody_trajectory_open");
    }
    void closeTrajectory() { check(nbody_trajectory_close(_ctx), "nbody_trajectory_close"); }

    /* adaptive global step, dt = clamp(eta * sqrt(length / max|a|), dtMin, dtMax) each step
       (length <= 0: the softening); setFixedTimestep() returns to the constructor's dt */
    void setAdaptiveTimestep(double eta, double length, double dtMin, double dtMax) {
        check(nbody_set_timestep_control(_ctx, NBODY_DT_ADAPTIVE, eta, length, dtMin, dtMax),
              "nbody_set_timestep_control");
    }
    /* individual steps dtMax / 2^k per particle (dtMax / dtMin = 2^K), each from eta sqrt(length / |a_i|) */
    void setBlockTimesteps(double eta, double length, double dtMin, double dtMax) {
        check(nbody_set_timestep_control(_ctx, NBODY_DT_BLOCK, eta, length, dtMin, dtMax),
              "nbody_set_timestep_control");
    }
    void setFixedTimestep() {
        check(nbody_set_timestep_control(_ctx, NBODY_DT_FIXED, 0.0, 0.0, 0.0, 0.0), "nbody_set_timestep_control");
    }
    double lastTimestep() const {
        double dt = 0.0;
        check(nbody_last_timestep(_ctx, &dt), "nbody_last_timestep");
        return dt;
    }
    /* block steps: each particle's level k (its last step was dtMax / 2^k), in the order particles were
       given to the constructor */
    std::vector<int32_t> levels() const {
        std::vector<int32_t> k((size_t)_n);
        check(nbody_get_levels(_ctx, k.data()), "nbody_get_levels");
        return k;
    }

    /* particles leaving the fixed root box [0, bounds): NBODY_ESCAPE_GROW (default) steps on the
       smallest grown box that keeps [0, bounds) as one of its cells, NBODY_ESCAPE_ERROR makes
       step() throw; grownBoxes() counts the evaluations that took a grown box */
    void setEscapePolicy(int policy) { check(nbody_set_escape_policy(_ctx, policy), "nbody_set_escape_policy"); }
    int64_t grownBoxes() const {
        int64_t s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        check(nbody_get_stats(_ctx, s, 10), "nbody_get_stats");
        return s[7];
    }

    nbody_ctx* handle() const { return _ctx; }
};

}  // namespace nbody

#endif
