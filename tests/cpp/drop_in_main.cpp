// A program written like the reference's src/main.cpp (uniform cube, random
// velocities, masses and charges, fixed time step, step() then particles()
// every step), with `using Simulation = nbody::CudaSimulation;` as its only
// change of backend.  Deterministic seed and a small N so it runs in a test;
// prints the final time, the particle count, a position checksum and the
// number of evaluations that took a grown root box (particles that left
// [0, bounds)).
// Usage: drop_in_main [N] [steps] [particles.f32|-] [dt] [final.f32]
//   particles.f32  N x 8 float32 (position xyz, velocity xyz, mass, charge)
//                  replacing the generated particles ("-": generate them)
//   dt             time step (default 1e-3, the reference's src/main.cpp:69)
//   final.f32      receives the final particles() (leaf order), N x 8 float32
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "nbody/cuda_simulation.h"

using Simulation = nbody::CudaSimulation;

int main(int argc, char** argv) {
    unsigned numParticles = argc > 1 ? (unsigned)std::atoi(argv[1]) : 20000;
    int numSteps = argc > 2 ? std::atoi(argv[2]) : 5;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    Simulation::Vector bounds = {1.0, 1.0, 1.0, 0.0};
    float velocityMax = 0.1f;
    std::vector<Simulation::Particle> particles;
    particles.reserve(numParticles);
    for (unsigned i = 0; i < numParticles; ++i) {
        Simulation::Vector position = {bounds[0] * U(rng), bounds[1] * U(rng), bounds[2] * U(rng), 0.0f};
        float theta = 2.0f * (float)M_PI * U(rng);
        float phi = std::acos(2.0f * (U(rng) - 0.5f));
        Simulation::Vector velocity = {velocityMax * std::sin(phi) * std::cos(theta),
                                       velocityMax * std::sin(phi) * std::sin(theta), velocityMax * std::cos(phi),
                                       0.0f};
        float mass = 1.0f + 9.0f * U(rng);
        float charge = 0.1f + 0.9f * U(rng);
        particles.push_back(Simulation::Particle(position, velocity, mass, charge));
    }
    const float timeStep = argc > 4 ? (float)std::atof(argv[4]) : 0.001f;
    if (argc > 3 && std::string(argv[3]) != "-") {
        std::FILE* f = std::fopen(argv[3], "rb");
        if (!f) { std::fprintf(stderr, "cannot open %s\n", argv[3]); return 2; }
        std::vector<float> buf(8 * (size_t)numParticles);
        size_t got = std::fread(buf.data(), sizeof(float), buf.size(), f);
        std::fclose(f);
        if (got != buf.size()) { std::fprintf(stderr, "short read\n"); return 2; }
        particles.clear();
        for (unsigned i = 0; i < numParticles; ++i) {
            const float* r = &buf[8 * (size_t)i];
            Simulation::Vector position = {r[0], r[1], r[2], 0.0f};
            Simulation::Vector velocity = {r[3], r[4], r[5], 0.0f};
            particles.push_back(Simulation::Particle(position, velocity, r[6], r[7]));
        }
    }
    std::ostringstream log;
    try {
        Simulation simulation(bounds, particles, timeStep, log);
        float time = 0.0f;
        double checksum = 0.0;
        size_t count = 0;
        std::vector<Simulation::Particle> ps;
        for (int s = 0; s < numSteps; ++s) {
            time = simulation.step();
            ps = simulation.particles();
            count = ps.size();
            checksum = 0.0;
            for (auto const& p : ps) checksum += p.position[0] + 2.0 * p.position[1] + 3.0 * p.position[2];
        }
        std::printf("time %.9g count %zu checksum %.12e grown %lld\n", time, count, checksum,
                    (long long)simulation.grownBoxes());
        if (argc > 5) {
            std::FILE* f = std::fopen(argv[5], "wb");
            if (!f) { std::fprintf(stderr, "cannot open %s\n", argv[5]); return 2; }
            for (auto const& p : ps) {
                const float r[8] = {p.position[0], p.position[1], p.position[2], p.velocity[0],
                                    p.velocity[1], p.velocity[2], p.mass, p.charge};
                std::fwrite(r, sizeof(float), 8, f);
            }
            std::fclose(f);
        }
    } catch (std::runtime_error const& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
