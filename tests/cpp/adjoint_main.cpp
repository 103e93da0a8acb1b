// The adjoint through the C++ drop-in: a recorded leapfrog run and its reverse
// sweep for the loss L = sum_i |x_i(T)|^2 / 2 (so dL/dx_T = x_T, dL/dv_T = 0).
// Reads N x 8 float32 particles (position xyz, velocity xyz, mass, charge);
// prints checksums of dL/dx_0, dL/dv_0, dL/dq and dL/dm.
// Usage: adjoint_main N steps every particles.f32
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <vector>

#include "nbody/cuda_simulation.h"

using Simulation = nbody::CudaSimulation;

int main(int argc, char** argv) {
    if (argc < 5) return 2;
    const unsigned n = (unsigned)std::atoi(argv[1]);
    const int steps = std::atoi(argv[2]), every = std::atoi(argv[3]);
    std::vector<float> buf(8 * (size_t)n);
    std::FILE* f = std::fopen(argv[4], "rb");
    if (!f || std::fread(buf.data(), sizeof(float), buf.size(), f) != buf.size()) return 2;
    std::fclose(f);
    std::vector<Simulation::Particle> particles;
    for (unsigned i = 0; i < n; ++i) {
        const float* r = &buf[8 * (size_t)i];
        particles.push_back(Simulation::Particle({r[0], r[1], r[2], 0.0f}, {r[3], r[4], r[5], 0.0f}, r[6], r[7]));
    }
    nbody_params p;
    nbody_default_params(&p);
    p.precision = NBODY_PREC_FP64;
    p.order = 6;
    p.leaf_capacity = 16;
    p.eps = 0.01;
    p.integrator = NBODY_INTEG_LEAPFROG;
    p.fixed_box = 0;
    std::ostringstream log;
    try {
        Simulation sim({1.0f, 1.0f, 1.0f, 0.0f}, particles, 1e-3f, log, p);
        sim.forwardCheckpointed(steps, every);
        std::vector<Simulation::Particle> fin = sim.particlesInInputOrder();
        std::vector<double> gxT(3 * (size_t)n), gvT, gx0, gv0, gq, gm;
        for (unsigned i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) gxT[3 * i + d] = fin[i].position[d];
        sim.backward(gxT, gvT, gx0, gv0, gq, gm);
        double cx = 0, cv = 0, cq = 0, cm = 0;
        for (unsigned i = 0; i < n; ++i) {
            for (int d = 0; d < 3; ++d) {
                cx += (d + 1) * gx0[3 * i + d];
                cv += (d + 1) * gv0[3 * i + d];
            }
            cq += gq[i];
            cm += gm[i];
        }
        std::printf("gx %.15e gv %.15e gq %.15e gm %.15e\n", cx, cv, cq, cm);
    } catch (std::runtime_error const& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
