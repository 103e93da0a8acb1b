/*
 * ref_naive_driver.cpp -- C entry point around the reference's CPU path
 * (src/naive_simulation.cpp, compiled unmodified from where it lies).
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle's port of that path and,
 * where this object exists, as the timed CPU baseline.
 */
#include <vector>

#include "nbody/naive_simulation.h"

using nbody::NaiveSimulation;

extern "C" float ref_naive_steps(int n, float* pos4, float* vel4, const float* mass, const float* charge, float G,
                                 float dt, int steps) {
    std::vector<NaiveSimulation::Particle> ps;
    ps.reserve(n);
    for (int i = 0; i < n; ++i) {
        NaiveSimulation::Vector p = {pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], pos4[4 * i + 3]};
        NaiveSimulation::Vector v = {vel4[4 * i], vel4[4 * i + 1], vel4[4 * i + 2], vel4[4 * i + 3]};
        ps.push_back(NaiveSimulation::Particle(p, v, mass[i], charge[i]));
    }
    NaiveSimulation sim(ps, G, dt);
    float t = 0.0f;
    for (int s = 0; s < steps; ++s) t = sim.step();
    std::vector<NaiveSimulation::Particle> out = sim.particles();
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 4; ++d) {
            pos4[4 * i + d] = out[i].position[d];
            vel4[4 * i + d] = out[i].velocity[d];
        }
    return t;
}
