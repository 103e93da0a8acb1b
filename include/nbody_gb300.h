/*
 * nbody_gb300.h -- C ABI of the GB300 FMM step (libnbody_gb300.so).
 *
 * This is the drop-in boundary below the reference's Simulation interface
 * (include/nbody/simulation.h:6-37 of duanebyer/nbody).  The C++ class
 * nbody::CudaSimulation (include/nbody/cuda_simulation.h) implements that
 * interface on top of these calls, the way OpenClSimulation
 * (include/nbody/open_cl_simulation.h:19-203) implements it on top of OpenCL.
 *
 * Conventions
 *   - every call returns an int status (NBODY_OK = 0); no exception crosses it;
 *     nbody_last_error() gives a one-line message for the last failure;
 *   - plain pointers and sizes only; host arrays are row-major, positions and
 *     velocities as n x 3 doubles;
 *   - one context = one CUDA stream on one device; a context is not
 *     thread-safe, distinct contexts are independent;
 *   - particle state stays resident on the device between calls; host copies
 *     happen only in nbody_set_state / nbody_get_state / nbody_compute_forces.
 */
#ifndef NBODY_GB300_H
#define NBODY_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define NBODY_OK 0
#define NBODY_ERR_INVALID 1      /* bad argument */
#define NBODY_ERR_CUDA 2         /* CUDA runtime error */
#define NBODY_ERR_NOMEM 3        /* device allocation failed */
#define NBODY_ERR_CAPACITY 4     /* a bounded device structure overflowed */
#define NBODY_ERR_STATE 5        /* call not valid in the current state */
#define NBODY_ERR_NO_DEVICE 6    /* no CUDA device */
#define NBODY_ERR_RANGE 7        /* a particle left the fixed root box (policy NBODY_ESCAPE_ERROR), or no
                                    representable root box covers the particles */

/* precision forms */
#define NBODY_PREC_FP32 0        /* state and arithmetic in FP32 */
#define NBODY_PREC_MIXED 1       /* FP64 state and shifts, FP32 offsets and bulk work, compensated sums */
#define NBODY_PREC_FP64 2        /* everything in FP64 */

/* integrators */
#define NBODY_INTEG_LEAPFROG 0   /* kick-drift-kick */
#define NBODY_INTEG_EULER 1      /* v += F/m dt, x += v_old dt (src/open_cl_simulation.cpp:600-607) */

typedef struct nbody_params {
    int precision;        /* NBODY_PREC_* */
    int order;            /* Cartesian expansion order 1..8; 1 = the reference's (monopole, constant local field) */
    int leaf_capacity;    /* bucket capacity (reference: 8, src/open_cl_simulation.cpp:41-47); 1..64 */
    int max_level;        /* depth cap, <= 21 */
    double theta;         /* opening angle of the MAC 3/4 (wA+wB)^2/d^2 < theta^2 (src/interaction.cl:3-5,64-79) */
    double eps;           /* Plummer softening (PARTICLE_RADIUS, src/field.cl:3-5) */
    double G;             /* coupling (-FORCE_CONSTANT, src/field.cl:7-9) */
    double dt;            /* time step */
    int integrator;       /* NBODY_INTEG_* */
    int fixed_box;        /* 1: root box [box_min, box_min + box_size)^3 as the reference's bounds; 0: data cube per step */
    double box_min[3];
    double box_size;
    int device;           /* CUDA device ordinal */
} nbody_params;

typedef struct nbody_ctx nbody_ctx;

/* Fills the reference's defaults: FP32, order 1, capacity 8, theta 0.5,
   eps 0.01, G 1, dt 1e-3, explicit Euler, box [0,1)^3
   (src/main.cpp:23-27,69, src/interaction.cl:3-5, src/field.cl:3-9). */
void nbody_default_params(nbody_params* p);

/* Creates a context (replaces OpenClSimulation::initialize,
   src/open_cl_simulation.cpp:618-681: device selection and setup). */
int nbody_create(const nbody_params* p, nbody_ctx** out);

/* Releases every device resource of the context. */
int nbody_destroy(nbody_ctx* c);

/* Uploads particles; arrays are n x 3 (pos, vel, acc) and n (mass, charge);
   vel and charge may be NULL (zero velocity, charge = mass).  acc, if not
   NULL, are the accelerations at these positions (as returned by
   nbody_get_state), which lets a leapfrog run resume without an extra force
   evaluation.  Replaces the particle packing and octree construction of the
   OpenClSimulation constructor (src/open_cl_simulation.cpp:15-51). */
int nbody_set_state(nbody_ctx* c, int64_t n, const double* pos, const double* vel, const double* mass,
                    const double* charge, const double* acc);

/* Downloads the state.  order = 0: current Morton (leaf) order, the order
   the reference's particles() returns (src/open_cl_simulation.cpp:53-68);
   order = 1: input order.  Any pointer may be NULL.  ids receives, per row,
   the input index of that particle; acc the last accelerations. */
int nbody_get_state(nbody_ctx* c, int order, double* pos, double* vel, double* mass, double* charge, int64_t* ids,
                    double* acc);

/* Advances nsteps steps of dt (replaces OpenClSimulation::step,
   src/open_cl_simulation.cpp:70-106); *t_out (may be NULL) receives the
   time after the last step. */
int nbody_step(nbody_ctx* c, int nsteps, double* t_out);

/* Step-size control.  The reference integrates with one fixed dt and lists a
   variable time step among its goals (TODO: "variable timestep"); this is a
   global adaptive step on top of the fused integrator.
   mode NBODY_DT_FIXED: every step takes params.dt (the default).
   mode NBODY_DT_ADAPTIVE: each step takes
       dt = clamp(eta * sqrt(length / max_i |a_i|), dt_min, dt_max)
   from the accelerations of the last force evaluation: for the leapfrog
   those at the start of the step (so each kick-drift-kick step uses one dt),
   for explicit Euler those of the previous step.  length <= 0 takes the
   softening eps (which must then be > 0).  max |a_i|^2 is reduced on the
   device with the evaluation and read at the step's existing
   synchronisation.  The recorded run of the adjoint
   (nbody_forward_checkpointed) needs mode NBODY_DT_FIXED.  Returning to
   NBODY_DT_FIXED restores the dt the context had before. */
#define NBODY_DT_FIXED 0
#define NBODY_DT_ADAPTIVE 1
#define NBODY_DT_BLOCK 2
int nbody_set_timestep_control(nbody_ctx* c, int mode, double eta, double length, double dt_min, double dt_max);

/* mode NBODY_DT_BLOCK (leapfrog only): individual time steps in a power-of-two
   hierarchy.  dt_max / dt_min must be 2^K (K <= 20).  Each nbody_step
   advances dt_max in 2^K substeps of dt_min: every particle drifts every
   substep; particle i takes steps of dt_i = dt_max / 2^k_i, with k_i the
   smallest level whose step is no longer than eta sqrt(length / |a_i|)
   (length <= 0: eps), chosen at the start of each of its steps from its
   acceleration there (a step may only start where the substep grid allows
   it), and receives its half kicks at the start and the end of each of its
   steps.  A substep at which some step ends evaluates the forces (near
   field only for leaves holding such a particle); the others only drift.
   At the end of nbody_step all particles are synchronous.  K = 0 is the fixed-step kick-drift-kick
   leapfrog.  nbody_get_levels gives each particle's k (input order) of its
   last step; nbody_last_timestep returns dt_max. */
int nbody_get_levels(nbody_ctx* c, int32_t* levels);

/* Particles that leave a fixed root box (params.fixed_box = 1).  The
   reference builds its octree over [0, bounds) (src/open_cl_simulation.cpp:
   20,43-47) and re-inserts moved particles with the external octree's move()
   (:120-123), whose handling of a particle outside the bounds is not part of
   the reference.  Here:
   NBODY_ESCAPE_GROW (the default): an evaluation whose particles do not all
     lie in the box takes the smallest box of side box_size * 2^j that has
     the fixed box as one of its level-j cells and covers every particle (so
     particles inside the fixed box keep their cells below level j); the
     count of such evaluations since nbody_set_state is nbody_get_stats
     entry 7;
   NBODY_ESCAPE_ERROR: such an evaluation fails with NBODY_ERR_RANGE before
     any force is computed (with the leapfrog the opening kick and drift of
     that step have already been applied; with explicit Euler the state is
     the one before the step). */
#define NBODY_ESCAPE_GROW 0
#define NBODY_ESCAPE_ERROR 1
int nbody_set_escape_policy(nbody_ctx* c, int policy);

/* The dt of the last step taken (params.dt before any step). */
int nbody_last_timestep(nbody_ctx* c, double* dt);

/* Accelerations (n x 3) and, if pot != NULL, potential per unit charge (n) at
   the current positions, in input order, without advancing.  This is the
   force evaluation that the reference keeps private
   (computeForceBuffers, src/open_cl_simulation.cpp:486-570). */
int nbody_compute_forces(nbody_ctx* c, double* acc, double* pot);

/* Adjoint (no counterpart in the reference, which has no gradients).
   Arrays are in input order; pointers may be host or device memory; any
   output may be NULL.  Derivatives are those of the FMM forces with the tree
   and interaction lists of each evaluation held fixed (the lists change only
   where a particle crosses a cell boundary or a cell pair crosses the
   acceptance threshold, where the force itself jumps).

   nbody_force_vjp: one force evaluation at the current positions and, for
   S = sum_i mu_i . a_i with mu (n x 3), gx = dS/dx (n x 3), gq = dS/dq (n),
   gm = dS/dm (n).  A zero-charge particle's gq omits the term
   G/m_i mu_i . E_i (its acceleration does not carry E_i). */
int nbody_force_vjp(nbody_ctx* c, const double* mu, double* gx, double* gq, double* gm);

/* Advances nsteps leapfrog (KDK) steps like nbody_step, recording for
   nbody_backward.
   every >= 1: the sorted state every `every` steps (plus the final state):
   (ceil(nsteps / every) + 1) snapshots of about 92 bytes per particle in
   the FP64 and mixed forms, 48 in FP32.  The reverse sweep recomputes each
   checkpoint interval forward from its snapshot (the checkpoint's far field
   only: the snapshot holds its accelerations; then every - 1 full steps) and
   records those evaluations whole, so it holds the records of one interval
   (about 370 bytes per particle per time point at order 5 and leaf capacity
   64).  The last interval, the first one the reverse sweep needs, is
   recorded by this call as it runs and is not recomputed, so this call
   already holds those records.
   every = 0: every time point's whole evaluation (tree, lists, local
   expansions, particle offsets), so the reverse sweep evaluates nothing:
   about 370 bytes per particle per time point at order 5 and leaf capacity
   64 (most of it the far-field lists), plus one state snapshot. */
int nbody_forward_checkpointed(nbody_ctx* c, int nsteps, int every, double* t_out);

/* Reverse sweep of the run recorded by the last nbody_forward_checkpointed:
   given gxT = dL/dx_N and gvT = dL/dv_N (n x 3 each; NULL = zero), returns
   gx0 = dL/dx_0, gv0 = dL/dv_0 (n x 3), gq = dL/dq and gm = dL/dm (n).  The
   context's state is that run's final state again on return.  The recording
   is dropped by nbody_set_state and nbody_step. */
int nbody_backward(nbody_ctx* c, const double* gxT, const double* gvT, double* gx0, double* gv0, double* gq,
                   double* gm);

/* Frozen-structure replay of the run recorded by nbody_forward_checkpointed
   with every = 0: from the initial state given here (input order; vel and
   charge may be NULL = zero velocity, charge = mass) it advances nsteps
   (<= the recorded steps; < 0: all of them) leapfrog steps in which the
   force evaluation at time point k reuses the tree, interaction lists and
   near-field plan recorded at time point k, recomputing everything that
   depends on the particle data.  That is the function whose derivative
   nbody_backward returns, so central finite differences of the replay check
   the adjoint without the jumps a rebuilt tree makes when a perturbed
   particle crosses a cell boundary.  pos_out / vel_out (n x 3, input order,
   may be NULL) receive the final state.  The recording and the context's
   state are those of the recorded run again on return.  (No counterpart in
   the reference.) */
int nbody_forward_replay(nbody_ctx* c, const double* pos, const double* vel, const double* mass,
                         const double* charge, int nsteps, double* pos_out, double* vel_out);

/* Trajectory file (replaces the CSV dump of src/main.cpp:77-101, same row
   format: the time, then x,y,z of every particle, comma separated, one row per
   written step).  After nbody_trajectory_open, every `every`-th step taken by
   nbody_step appends a row; order = 0 writes particles in the current leaf
   order (what the reference's particles() returns), order = 1 in input order;
   digits = significant digits (the reference's stream default is 6).
   Positions are copied asynchronously and formatted by a writer thread; a
   step waits only when three rows are still being written.
   nbody_trajectory_close (also done by nbody_set_state and nbody_destroy)
   flushes and closes the file and reports a failed write. */
int nbody_trajectory_open(nbody_ctx* c, const char* path, int every, int order, int digits);
int nbody_trajectory_close(nbody_ctx* c);

/* FP64 diagnostics of the current state: out[0] kinetic energy, out[1]
   potential energy, out[2..4] momentum, out[5..7] angular momentum,
   out[8] total mass.  (The reference computes none.) */
int nbody_diagnostics(nbody_ctx* c, double* out);

/* FP64 softened direct sum at the current positions for nt targets (input
   indices), on the device: acc (nt x 3) and pot (nt, may be NULL).  The
   accuracy reference for the FMM (there is no such call in the reference;
   its CPU path src/naive_simulation.cpp is a direct sum without softening). */
int nbody_direct_forces(nbody_ctx* c, int64_t nt, const int64_t* targets, double* acc, double* pot);

/* Allocation-free form of nbody_direct_forces, for callers that must not
   allocate device memory (code under a host framework that owns the device
   memory budget, or on a path where cudaMalloc's synchronization or failure
   under memory pressure is unacceptable).  No counterpart in the reference.
   Inputs and outputs are the caller's device-accessible arrays: pos (n x 3),
   mass and charge (n; charge may be NULL = mass), targets (nt indices into
   them), acc (nt x 3) and pot (nt, may be NULL).  Work is enqueued on
   `stream` (a cudaStream_t, NULL = default stream) and the call returns
   without waiting; outputs are valid once the stream is synchronized.
   Scratch is a fixed 4 MiB device array inside the library, so nt is limited
   to 131072 per call (larger requests fail with NBODY_ERR_INVALID).  Every
   call on a device shares that array: calls that overlap on the GPU race and
   must be ordered by the caller.  The first call on a device looks up the
   array's device address; make it before any stream capture on that device
   (after a cudaDeviceReset the next call looks it up again).  The call makes
   `device` current for its launches and restores the calling thread's
   previous current device before it returns.  Target indices outside
   [0, n) give NaN results.  Errors: nbody_last_error(NULL). */
int nbody_direct_forces_static(int device, int64_t n, const double* pos, const double* mass, const double* charge,
                               double eps, double G, int64_t nt, const int64_t* targets, double* acc, double* pot,
                               void* stream);

/* Work counters of the last force evaluation: out[0] far-field (M2L)
   cell pairs, out[1] near-field particle pairs, out[2] near-field leaf
   pairs, out[3] nodes, out[4] leaves, out[5] depth, out[6] kernel launches
   of the last step, out[7] evaluations since nbody_set_state whose fixed
   root box was grown (nbody_set_escape_policy), out[8] near-field leaves
   over the substeps of the last block step and out[9] how many of them
   held a particle closing its step (the others' near field was skipped),
   out[10] the force evaluations of the last block step (substeps at which
   no step can end only drift).  n = number of entries wanted (<= 11). */
int nbody_get_stats(nbody_ctx* c, int64_t* out, int n);

/* Floating-point operations this build counts per far-field cell pair
   (derivative tensor + contraction, FMA = 2) and per near-field particle
   pair (20, the GPU Gems 3 ch. 31 convention) at expansion order p. */
int64_t nbody_flops_per_m2l(int order);
int64_t nbody_flops_per_p2p(void);

/* Measured FMA throughput of this device: out[0] FP32 and out[1] FP64
   GFLOP/s (FMA = 2 flops), from a register-resident FMA chain kernel
   timed with CUDA events. */
int nbody_measure_peaks(int device, double* out);

/* Number of particles, nodes, leaves and the depth of the last tree. */
int nbody_tree_info(nbody_ctx* c, int64_t* n, int64_t* nnodes, int64_t* nleaves, int* depth);

/* Copies the last tree for inspection: keys (n, sorted Morton keys), perm
   (n, input index of each sorted row), nodes (nnodes x 9 int32 rows:
   level, ix, iy, iz, begin, count, parent, child_begin, nchild; breadth-first).
   Any pointer may be NULL. */
int nbody_get_tree(nbody_ctx* c, uint64_t* keys, int64_t* perm, int32_t* nodes);

/* Sizes and contents of the last interaction lists, as (target, source)
   node pairs.  which = 0: far field (M2L), 1: near field (P2P).  Pass
   pairs = NULL to get the size only.  Replaces the interaction buffers of
   computeInteractionBuffers (src/open_cl_simulation.cpp:176-369). */
int nbody_get_interactions(nbody_ctx* c, int which, int64_t* npairs, int32_t* pairs);

/* Per-phase device times (ms) of the last force evaluation: 0 kick/drift +
   keys, 1 sort + gather, 2 tree, 3 upward pass (P2M, M2M), 4 interaction
   lists, 5 far field (M2L, L2L), 6 near field + L2P + integration; and of the
   last nbody_force_vjp: 7 adjoint seeds + L2P transpose, 8 L2L transpose,
   9 M2L transpose, 10 M2M transpose (the near field runs alongside 7-10 on
   side streams), 11 the rest of the near field + the P2M/L2P adjoints.
   n <= 12.  Timing is enabled by nbody_set_timing(c, 1). */
int nbody_set_timing(nbody_ctx* c, int on);
int nbody_phase_times(nbody_ctx* c, float* ms, int n);

/* The context's CUDA stream (a cudaStream_t), for callers that order their
   own work after the step. */
void* nbody_stream(nbody_ctx* c);

/* Device memory held by the context (its grow-only work buffers, snapshots and
   records) and its high-water mark since nbody_create, in bytes. */
int nbody_device_memory(nbody_ctx* c, int64_t* current, int64_t* peak);

/* Time limits of the device-side waits.  Every wait in a kernel of this
   library is bounded; one that runs out raises an error word and the kernel
   returns (it never traps or hangs), and the host turns the word into
   NBODY_ERR_CUDA at its next synchronisation.  scan_polls bounds the polls of
   one status word in the single-pass scans' look-back (default about a
   second's worth); copy_cycles bounds, in SM clock cycles, the far-field
   kernel's wait for its own bulk copies (default 2e9, about a second).  A
   value <= 0 restores the default.  A scan that gives up leaves the context
   failed for good (its state may be inconsistent): create a new one.  A
   far-field wait that gives up fails that evaluation only. */
int nbody_set_wait_limits(nbody_ctx* c, int64_t scan_polls, int64_t copy_cycles);

/* Runs one of the bounded device waits on something that never completes and
   reports it the way a step does, so the give-up path can be checked on a
   GPU without a fault or a hang (no counterpart in the reference):
   which = 0: the scans' look-back wait on a tile status word that nothing
     publishes (context's scan_polls limit): NBODY_ERR_CUDA "a device scan did
     not complete in time", which leaves the context failed like a real one;
   which = 1: the far-field kernel's wait on an mbarrier that expects bytes no
     copy delivers (context's copy_cycles limit): NBODY_ERR_CUDA "a far-field
     copy did not complete in time"; the context stays usable. */
int nbody_selftest_wait(nbody_ctx* c, int which);

/* 1 in the NBODY_DEBUG_BOUNDS build of the library (libnbody_gb300_debug.so),
   0 otherwise.  That build checks every index read from device data (sorted
   order, node ids of the interaction lists, particle ranges): an index out
   of range is replaced by an in-bounds one and the failing site is reported
   as NBODY_ERR_CUDA at the end of the evaluation, so a bug shows as an error
   instead of a fault.  (No counterpart in the reference.) */
int nbody_debug_bounds(void);

/* Simulated time. */
int nbody_get_time(nbody_ctx* c, double* t);

/* Message of the last failure on this context (or of the last failed
   nbody_create when c is NULL). */
const char* nbody_last_error(nbody_ctx* c);

#ifdef __cplusplus
}
#endif

#endif
