/*
 * nbody/simulation.h -- the simulation interface of duanebyer/nbody
 * (include/nbody/simulation.h:6-37 there), restated so that this library and
 * programs written against the reference compile without the reference tree.
 * Names, template parameters and member signatures are kept identical because
 * callers (the reference's src/main.cpp) use them directly; the include guard
 * is the reference's own, so a project that also has the reference header uses
 * whichever is included first and both declare the same class.
 */
#ifndef __NBODY_SIMULATION_H_
#define __NBODY_SIMULATION_H_

#include <vector>

namespace nbody {

template <typename TScalar, typename TVector>
class Simulation {
public:
    using Scalar = TScalar;
    using Vector = TVector;

    struct Particle final {
        Vector position;
        Vector velocity;
        Scalar mass;
        Scalar charge;

        Particle(Vector position, Vector velocity, Scalar mass, Scalar charge)
            : position(position), velocity(velocity), mass(mass), charge(charge) {}
    };

    /* advances one time step and returns the new time */
    virtual Scalar step() = 0;
    /* the particles, in the simulation's internal (octree leaf) order */
    virtual std::vector<Particle> particles() const = 0;
};

}  // namespace nbody

#endif
