/*
 * dpg.h -- C ABI of the GB300-native (sm_103a) granular contact library.
 *
 * Drop-in boundary for the hot path of mmccraw98/dpCUDA-v2: the cell-list and
 * Verlet neighbour build, harmonic disk contacts, and the NVE, FIRE and Adam
 * updates, plus the stress / box-scaling / last-state pieces the jamming
 * drivers use.  Each entry point names the reference interface it replaces
 * (file:line in the reference tree).  Plain C types only: pointers, sizes,
 * doubles, status codes.
 *
 * Conventions
 *  - Every function returns an int status (DPG_OK = 0).  dpg_last_error()
 *    gives a message for the calling thread's last failure.
 *  - A handle owns its device memory and a CUDA stream; there is no global
 *    state, so several handles may coexist.  A handle is not thread-safe.
 *  - Arrays crossing the boundary are in STATIC order (the order the
 *    particles were given at setup), like the reference's state files
 *    (src/io/state_log.cu:30-32).  Internally particles are kept cell-sorted.
 *  - `where` arguments say whether a pointer is host (DPG_HOST) or device
 *    (DPG_DEVICE) memory.
 *  - Arithmetic of the plain form is IEEE FP64 without FMA contraction, in the
 *    reference's operation order: per-particle results are bit-identical to
 *    the reference kernels given identical inputs and neighbour lists.
 */
#ifndef DPG_H
#define DPG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------- */
#define DPG_OK 0
#define DPG_ERR_ARG 1          /* bad argument */
#define DPG_ERR_CUDA 2         /* CUDA runtime error */
#define DPG_ERR_OVERFLOW 3     /* neighbour capacity exceeded and could not grow */
#define DPG_ERR_NOT_CONVERGED 4
#define DPG_ERR_STATE 5        /* call out of order (e.g. forces before neighbours) */
#define DPG_ERR_TIMEOUT 6      /* a bounded device wait ran out */

#define DPG_HOST 0
#define DPG_DEVICE 1

/* neighbour methods (src/particles/base/particle.cu:237-265) */
#define DPG_NEIGH_CELL 0
#define DPG_NEIGH_VERLET 1
#define DPG_NEIGH_ALL 2

/* precision forms */
#define DPG_FP64 0  /* plain all-FP64 drop-in */
#define DPG_MIXED 1 /* FP64 cell origin + FP32 offsets, FP32 pair maths, FP64 accumulation */
#define DPG_DWORD 2 /* dpg_ensemble_compute_forces only: the double-word FP32 pair
                       arithmetic of the mixed form's refinement stage */

typedef struct dpg_system *dpg_handle;

/* Particle parameters: Particle::setEnergyScale / setExponent
 * (src/particles/base/particle.cu:729-825) and the box. */
typedef struct {
    int64_t n_particles;
    double box_x, box_y;
    double e_c; /* contact energy scale */
    double n_c; /* contact exponent (2 = harmonic) */
    int precision; /* DPG_FP64 or DPG_MIXED */
    int reserved;
} dpg_params;

/* Neighbour configuration: Particle::setupNeighbors config keys
 * (src/particles/base/particle.cu:71-100, include/particles/standard_configs.h:135-141). */
typedef struct {
    int method;                 /* DPG_NEIGH_* (requested; fallbacks as in the reference) */
    double cutoff_multiplier;   /* r_c = multiplier * max diameter */
    double displacement_multiplier;
    double particles_per_cell;
    double cell_displacement_multiplier;
} dpg_neighbor_config;

/* What setup chose (Particle members neighbor_cutoff, n_cells_dim, ...). */
typedef struct {
    int method;
    int capacity;  /* max_neighbors_allocated */
    int n_cells_dim;
    int reserved;
    double cutoff;
    double neighbor_threshold_sq;
    double cell_size;
    double cell_threshold_sq;
    int64_t n_rebuilds;
    int64_t n_cell_rebuilds;
} dpg_neighbor_info;

/* FIRE parameters: Fire (include/integrator/fire.h:15-35) + minimizeFire
 * (src/routines/minimization.cu:75-112).  fmax_target > 0 adds a
 * max_i |F_i| <= fmax_target stop (not in the reference). */
typedef struct {
    double alpha_init;
    double dt;
    double avg_pe_target;
    double avg_pe_diff_target;
    int64_t max_steps;
    double fmax_target;
} dpg_fire_params;

typedef struct {
    int64_t steps;   /* loop index at exit, as minimizeFire's `step` */
    int stopped;     /* Fire::stopped */
    int converged;   /* left through a stop criterion (not max_steps) */
    double avg_pe;   /* PE / N at exit */
    double max_force;
    double alpha, dt;
} dpg_fire_result;

/* ---- lifetime ------------------------------------------------------- */
/* Disk::initializeFromConfig / Particle::setNumParticles + setBoxSize
 * (src/particles/disk/disk.cu:98-170).  stream may be NULL (own stream). */
int dpg_create(const dpg_params *p, void *cuda_stream, dpg_handle *out);
int dpg_destroy(dpg_handle h);
/* the parameters the handle was created with, box updated (Particle::n_particles, e_c, n_c) */
int dpg_get_params(dpg_handle h, dpg_params *p);
const char *dpg_last_error(void);
int dpg_version(void);

/* ---- state ---------------------------------------------------------- */
/* Particle::setData on positions, velocities, radii, masses (static order).
 * Any pointer may be NULL to leave that array unchanged. */
int dpg_set_state(dpg_handle h, const double *x, const double *y, const double *vx,
                  const double *vy, const double *radii, const double *masses, int where);
/* Particle::getArrayData (src/particles/base/particle.cu:480-692), un-permuted
 * to static order like the reference IO.  NULL pointers are skipped. */
int dpg_get_state(dpg_handle h, double *x, double *y, double *vx, double *vy, double *fx,
                  double *fy, double *pe, int where);
int dpg_set_forces(dpg_handle h, const double *fx, const double *fy, int where);
/* radii and masses in static order to host arrays (getArrayData "radii", "masses") */
int dpg_get_static_params(dpg_handle h, double *radii, double *masses);
/* Disk::load (src/particles/disk/disk.cu:35-96): replace positions,
 * velocities, radii and masses from static-order arrays AND reset the internal
 * slot order to the static order (forces and PE zeroed).  Call
 * dpg_setup_neighbors afterwards, as load() does. */
int dpg_load_state(dpg_handle h, const double *x, const double *y, const double *vx,
                   const double *vy, const double *radii, const double *masses, int where);
/* Particle::setBoxSize / getBoxSize (src/particles/base/particle.cu:694-709) */
int dpg_set_box(dpg_handle h, double box_x, double box_y);
int dpg_get_box(dpg_handle h, double *box_x, double *box_y);
int dpg_synchronize(dpg_handle h);

/* ---- neighbours ----------------------------------------------------- */
/* Particle::setupNeighbors (src/particles/base/particle.cu:71-100): method
 * fallbacks, cell size, initial lists, then calculateForces (+= semantics). */
int dpg_setup_neighbors(dpg_handle h, const dpg_neighbor_config *cfg, dpg_neighbor_info *info);
/* Particle::updateNeighborList (src/particles/base/particle.cu:1167-1169) */
int dpg_build_neighbors(dpg_handle h);
/* Particle::checkForNeighborUpdate (src/particles/base/particle.cu:1137-1161);
 * *rebuilt = 0 none, 1 neighbour list, 2 cell list + neighbour list. */
int dpg_check_neighbors(dpg_handle h, int *rebuilt);
int dpg_neighbor_info_get(dpg_handle h, dpg_neighbor_info *info);
/* Neighbour list in STATIC indices, row-major [n * cap] padded with -1, and
 * counts[n]; cap in/out: capacity of `list` rows in, used capacity out. */
int dpg_get_neighbors(dpg_handle h, int32_t *list, int32_t *counts, int *cap);
/* Cell list in the reference's representation: cell_index[n] of the particle
 * in each sorted slot, cell_start[n_cells + 1] with -1 for empty cells, and
 * static_index[n] of each slot (src/particles/base/kernels.cu:309-438). */
int dpg_get_cells(dpg_handle h, int64_t *cell_index, int64_t *cell_start, int64_t *static_index);

/* ---- forces and integration ----------------------------------------- */
/* kernelZeroForceAndPotentialEnergy (src/particles/base/kernels.cu:150-161) */
int dpg_zero_forces(dpg_handle h);
/* Disk::calculateForces -> kernelCalcDiskForces, accumulates into F and PE
 * (src/particles/disk/disk.cu:218-221, src/particles/disk/kernels.cu:11-57) */
int dpg_compute_forces(dpg_handle h);
/* Particle::updateVelocities (src/particles/base/particle.cu:1090-1092) */
int dpg_kick(dpg_handle h, double dt);
/* Particle::updatePositions (src/particles/base/particle.cu:1086-1088) */
int dpg_drift(dpg_handle h, double dt);
/* n_steps of NVE::step (src/integrator/nve.cu:15-25), device-resident loop */
int dpg_nve_steps(dpg_handle h, double dt, int64_t n_steps);

/* ---- state files in the reference's on-disk layout ---------------------- */
/* One text file per array in `dir` (created if missing): positions.dat,
 * velocities.dat, forces.dat ("x<TAB>y" lines), radii.dat, masses.dat,
 * potential_energy.dat, box_size.dat (one value per line), "%.17e", static
 * order -- the layout of the reference's StateLog (src/io/state_log.cu:27-41,
 * include/io/io_utils.h:81-108, include/constants.h:11); step.dat too when
 * step >= 0 (a restart directory). */
int dpg_write_state(dpg_handle h, const char *dir, int64_t step);
/* Reads positions, radii, masses, box_size (required) and velocities (optional,
 * else zero) from `dir` into the system, as Particle::loadDataFromPath
 * (src/particles/base/particle.cu:180-215); the slot order is reset. */
int dpg_read_state(dpg_handle h, const char *dir);
/* number of particles in a state directory (values in radii.dat) */
int dpg_state_count(const char *dir, int64_t *n_particles);

/* ---- damped NVE and gradient descent ----------------------------------- */
/* calculateDampedForces: F -= damping * v (src/particles/base/particle.cu:1363-1365,
 * kernel src/particles/base/kernels.cu:83-89) */
int dpg_damped_forces(dpg_handle h, double damping);
/* n DampedNVE::step (src/integrator/damped_nve.cu:15-27): kick dt/2, drift,
 * neighbour check, F = -damping v + pair forces, kick dt/2; one device loop */
int dpg_damped_nve_steps(dpg_handle h, double dt, double damping, int64_t n_steps);
/* Disk::calculateForceDistancePairs (src/particles/disk/disk.cu:228-255, kernel
 * src/particles/disk/kernels.cu:73-175): per neighbour-list entry, arrays of
 * n * cap (cap from dpg_neighbor_info_get) laid out as the reference's,
 * [slot * cap + k] in the current (cell-sorted) slot order, with the
 * reference's fill values where an entry is unused.  out[16] (NULL entries
 * skipped): pair energy, force x, force y, separation x, y, overlap (distance -
 * radius sum), radius sum, separation angle, pair Hessian xx, xy, yx, yy,
 * self Hessian xx, xy, yx, yy; this_id / other_id: static indices. */
int dpg_pair_dump(dpg_handle h, double *const *out, int64_t *this_id, int64_t *other_id,
                  int where);
/* Disk::calculateWallForces: += the hard-wall force and energy of walls at 0
 * and the box length on both axes (src/particles/disk/disk.cu:257-259,
 * include/particles/base/kernels.cuh:185-235) */
int dpg_wall_forces(dpg_handle h);
/* n NVE::wall_step (src/integrator/nve.cu:27-38): NVE with the wall forces
 * added before the pair forces; one device loop */
int dpg_nve_wall_steps(dpg_handle h, double dt, int64_t n_steps);
/* updatePositionsGradDesc: x += alpha F (src/particles/base/particle.cu:267-269) */
int dpg_grad_desc_step(dpg_handle h, double alpha);
/* n GradDesc::step (src/integrator/grad_desc.cu:11-17): zero, neighbour check,
 * forces, x += alpha F */
int dpg_grad_desc_steps(dpg_handle h, double alpha, int64_t n_steps);

/* ---- FIRE / Adam ------------------------------------------------------ */
/* Particle::getPowerFire (src/particles/base/particle.cu:993-1009) */
int dpg_power_fire(dpg_handle h, double *power);
/* Particle::mixVelocitiesAndForces (src/particles/base/particle.cu:895-897) */
int dpg_mix(dpg_handle h, double alpha);
/* Particle::setVelocitiesToZero (src/particles/base/particle.cu:871-873) */
int dpg_zero_velocities(dpg_handle h);
/* Fire::Fire (src/integrator/fire.cu:3-7) */
int dpg_fire_init(dpg_handle h, double alpha_init, double dt);
/* Fire::step (src/integrator/fire.cu:13-46); *stopped = Fire::stopped */
int dpg_fire_step(dpg_handle h, int *stopped);
int dpg_fire_get(dpg_handle h, double *alpha, double *dt, int64_t *n_good, int64_t *n_bad,
                 int *stopped);
/* minimizeFire (src/routines/minimization.cu:75-112), device-resident loop */
int dpg_fire_minimize(dpg_handle h, const dpg_fire_params *p, dpg_fire_result *r);
/* DPG_MIXED systems (no reference counterpart): pair forces are FP32 from
 * per-particle offsets to grid-cell centres, summed in FP64.  In
 * dpg_fire_minimize the system switches to the FP64 pair arithmetic once
 * max|F| <= switch_fmax (default 1e-6), FIRE goes uphill 6 times running, or
 * max|F|, once below 100 switch_fmax, stops falling for 2000 iterations; the
 * PE-change and fmax_target stop tests only pass in FP64. */
int dpg_set_mixed_switch(dpg_handle h, double switch_fmax);
/* Particle::initAdamVariables (src/particles/base/particle.cu:319-322) */
int dpg_adam_init(dpg_handle h);
/* Particle::updatePositionsAdam (src/particles/base/particle.cu:329-333) */
int dpg_adam_step(dpg_handle h, int64_t step, double alpha, double beta1, double beta2,
                  double epsilon);
/* minimizeAdam (src/routines/minimization.cu:3-33); *steps as its `step` */
int dpg_adam_minimize(dpg_handle h, double alpha, double beta1, double beta2, double epsilon,
                      double avg_pe_target, double avg_pe_diff_target, int64_t max_steps,
                      int64_t *steps);

/* ---- observables ---------------------------------------------------- */
/* totalPotentialEnergy / totalKineticEnergy (src/particles/base/particle.cu:1074-1080) */
int dpg_reduce_energies(dpg_handle h, double *pe, double *ke);
/* max_i |F_i| and |sum_i F_i| (getForceBalance, src/particles/base/particle.cu:231-235) */
int dpg_force_stats(dpg_handle h, double *max_force, double *force_balance);
/* calculateStressTensor + getStressTensor + getPressure
 * (src/particles/disk/disk.cu:281-285, src/particles/base/particle.cu:1371-1384) */
int dpg_pressure(dpg_handle h, double *pressure, double stress[4]);
/* countContacts + getContactCount (src/particles/disk/disk.cu:250-255) */
int dpg_contact_count(dpg_handle h, double *contacts);
/* getPackingFraction (src/particles/base/particle.cu:1011-1015) */
int dpg_packing_fraction(dpg_handle h, double *phi);

/* ---- box scaling and snapshots ---------------------------------------- */
/* Particle::scaleBox (src/particles/base/particle.cu:1057-1064) */
int dpg_scale_box(dpg_handle h, double factor);
/* Particle::scaleToPackingFractionFull (src/particles/base/particle.cu:1047-1055) */
int dpg_scale_to_packing_fraction(dpg_handle h, double phi);
/* setLastState / revertToLastState as device-side snapshots
 * (src/particles/base/particle.cu:956-991) */
int dpg_save_state(dpg_handle h);
int dpg_restore_state(dpg_handle h);

/* ---- jamming drivers (host control flow over the entry points above) ----- */
/* Pressure-band jamming by bisection on the box length:
 * scripts/runArthurJamWithFire.cpp:36-106.  Decompress (scaleBox by
 * decompress_factor) until P < pressure_low; then minimise, measure P, and
 * compress by compression_rate while unjammed, bisect on L once jammed
 * (P > pressure_high), reloading the last unjammed state; stop when
 * pressure_low <= P <= pressure_high and contacts > 2N. */
typedef struct {
    double pressure_low, pressure_high;
    double compression_rate;        /* L <- L * rate while unjammed without a bracket */
    double length_tolerance;        /* |L_low / L_high - 1| below this: give up */
    double decompress_factor;       /* initial scaleBox factor (1.01 in the reference) */
    int64_t max_compression_steps;
    dpg_fire_params fire;           /* each minimisation (minimizeFire defaults in the reference) */
    dpg_neighbor_config neighbors;  /* used to reload the saved state */
} dpg_jam_params;

typedef struct {
    double packing_fraction;
    double pressure;
    double box_length;
    double contacts;
    int64_t compression_steps;
    int64_t fire_steps_total;
    int status;  /* 0 final state reached, 1 length tolerance hit, 2 out of steps */
    int reserved;
} dpg_jam_result;

int dpg_jam_pressure(dpg_handle h, const dpg_jam_params *p, dpg_jam_result *r);

/* Energy-criterion jamming by bisection on phi: scripts/runJam.cpp:25-106
 * (decompress until PE/N < avg_pe_tolerance; compress by compression_increment;
 * jammed when PE/N > tolerance after FIRE; revertToLastState; bisect until
 * |phi_high / phi_low - 1| < phi_tolerance, then the stability check
 * scripts/runJam.cpp:15-23). */
typedef struct {
    double avg_pe_tolerance, avg_pe_diff_tolerance;
    double phi_tolerance, compression_increment, delta_phi_stability;
    int64_t max_compression_steps;
} dpg_jam_phi_params;

int dpg_jam_phi(dpg_handle h, const dpg_jam_phi_params *p, dpg_jam_result *r);

/* ======================================================================
 *  Rigid bumpy bodies (src/particles/rigid_bumpy/, include/particles/rigid_bumpy/)
 *  Bodies carry n_vertices_per_body vertex disks of one radius on a circle
 *  of radius R - r_v; vertex-vertex harmonic contacts are reduced to body
 *  force, torque and energy.
 * ====================================================================== */
typedef struct dpg_bumpy_system *dpg_bumpy_handle;

typedef struct {
    int64_t n_bodies;
    int64_t n_vertices;  /* sum of the per-body vertex counts */
    double box_x, box_y;
    double e_c;          /* vertex contact energy scale (the reference's d_e_c after
                            RigidBumpy's geometric rescaling, rigid_bumpy.cu:218-222) */
    double n_c;
    double vertex_radius;                      /* d_vertex_radius */
    double segment_length_per_vertex_diameter; /* sets the rebuild threshold */
    int rotation;                              /* RigidBumpy::rotation */
    int precision;                             /* DPG_FP64 */
} dpg_bumpy_params;

/* RigidBumpy construction (rigid_bumpy.cu:138-230, allocation part) */
int dpg_bumpy_create(const dpg_bumpy_params *p, void *cuda_stream, dpg_bumpy_handle *out);
int dpg_bumpy_destroy(dpg_bumpy_handle h);
/* Bodies in static order: positions, angles, velocities, angular velocities
 * (may be NULL = 0), radii and vertex counts; places the vertices on each
 * body (kernelInitializeVerticesOnParticles, kernels.cu:1137-1162). */
int dpg_bumpy_set_bodies(dpg_bumpy_handle h, const double *x, const double *y,
                         const double *angle, const double *vx, const double *vy,
                         const double *omega, const double *radii,
                         const int32_t *n_vertices_per_body);
/* explicit vertex positions in static vertex order (vertex_positions setData) */
int dpg_bumpy_set_vertices(dpg_bumpy_handle h, const double *vx, const double *vy);
/* RigidBumpy::setMass (rigid_bumpy.cu:1068-1080): body mass, vertex masses, moments of inertia */
int dpg_bumpy_set_mass(dpg_bumpy_handle h, double mass);
/* bodies back in static order; any pointer may be NULL */
int dpg_bumpy_get_bodies(dpg_bumpy_handle h, double *x, double *y, double *angle, double *vx,
                         double *vy, double *omega, double *fx, double *fy, double *torque,
                         double *pe, double *inertia);
int dpg_bumpy_get_vertices(dpg_bumpy_handle h, double *vx, double *vy);
/* setupNeighbors with RigidBumpy::setNeighborSize (rigid_bumpy.cu:1229-1250):
 * body list + vertex list, then calculateForces (+=). */
int dpg_bumpy_setup_neighbors(dpg_bumpy_handle h, const dpg_neighbor_config *cfg,
                              dpg_neighbor_info *info);
int dpg_bumpy_neighbor_info_get(dpg_bumpy_handle h, dpg_neighbor_info *info, int *vertex_capacity);
/* checkForNeighborUpdate (body displacement only, as the reference) */
int dpg_bumpy_check_neighbors(dpg_bumpy_handle h, int *rebuilt);
/* vertex neighbour list in static vertex indices, row-major [n_vertices * cap] */
int dpg_bumpy_get_vertex_neighbors(dpg_bumpy_handle h, int32_t *list, int32_t *counts, int *cap);
/* zeroForceAndPotentialEnergy / calculateForces (rigid_bumpy.cu:1088-1105,1378-1381) */
int dpg_bumpy_zero_forces(dpg_bumpy_handle h);
int dpg_bumpy_compute_forces(dpg_bumpy_handle h);
/* updateVelocities / updatePositions (rigid_bumpy.cu:1107-1130) */
int dpg_bumpy_kick(dpg_bumpy_handle h, double dt);
int dpg_bumpy_drift(dpg_bumpy_handle h, double dt);
/* mixVelocitiesAndForces / setVelocitiesToZero (rigid_bumpy.cu:1192-1196,1256-1260) */
int dpg_bumpy_mix(dpg_bumpy_handle h, double alpha);
int dpg_bumpy_zero_velocities(dpg_bumpy_handle h);
/* totals: PE, KE (translational + rotational), FIRE power (with tau.omega),
 * max |F_b| and max |tau_b| */
int dpg_bumpy_observables(dpg_bumpy_handle h, double *pe, double *ke, double *power,
                          double *max_force, double *max_torque);
int dpg_bumpy_nve_steps(dpg_bumpy_handle h, double dt, int64_t n_steps);
int dpg_bumpy_fire_init(dpg_bumpy_handle h, double alpha_init, double dt);
int dpg_bumpy_fire_step(dpg_bumpy_handle h, int *stopped);
/* minimizeFire with the rigid overrides; p->fmax_target > 0 stops at
 * max|F_b| <= fmax_target and max|tau_b| <= tmax_target */
/* DPG_MIXED bodies (no reference counterpart): FP32 vertex-pair forces, FP64
 * vertex torques and body sums; FIRE switches to FP64 vertex pairs once
 * max(|F|, |tau|) <= switch_fmax (default 1e-6) or stops falling, and only an
 * FP64 state passes the stop tests */
int dpg_bumpy_set_mixed_switch(dpg_bumpy_handle h, double switch_fmax);
int dpg_bumpy_fire_minimize(dpg_bumpy_handle h, const dpg_fire_params *p, double tmax_target,
                            dpg_fire_result *r);
/* scalePositionsFull (rigid_bumpy.cu:1044-1048) with the box: Particle::scaleBox */
int dpg_bumpy_scale_box(dpg_bumpy_handle h, double factor);
/* RigidBumpy::initAdamVariables / updatePositionsAdam (rigid_bumpy.cu:1461-1486,
 * kernels.cu:1004-1093): translational and angular moments; the translational
 * ones follow the reference's re-sort (swapped with never-gathered twins), the
 * angular ones stay with their slot */
int dpg_bumpy_adam_init(dpg_bumpy_handle h);
int dpg_bumpy_adam_step(dpg_bumpy_handle h, int64_t step, double alpha, double beta1,
                        double beta2, double epsilon);
/* minimizeAdam (src/routines/minimization.cu:3-33) with dof = 3 N (rotation) or 2 N;
 * *steps = the final step index */
int dpg_bumpy_adam_minimize(dpg_bumpy_handle h, double alpha, double beta1, double beta2,
                            double epsilon, double avg_pe_target, double avg_pe_diff_target,
                            int64_t max_steps, int64_t *steps);
/* Rigid gradient descent, GradDesc::step (src/integrator/grad_desc.cu:11-17) with
 * a rigid update the reference lacks (its GradDesc runs the disk
 * kernelGradDescStep, src/particles/base/kernels.cu:613-637, on the body
 * centres only): x += alpha F, theta += alpha tau (rotation), vertices move
 * with their body */
int dpg_bumpy_grad_desc_step(dpg_bumpy_handle h, double alpha);
int dpg_bumpy_grad_desc_steps(dpg_bumpy_handle h, double alpha, int64_t n_steps);
/* RigidBumpy::calculateDampedForces (rigid_bumpy.cu:1501-1503): F -= g v, tau -= g omega */
int dpg_bumpy_damped_forces(dpg_bumpy_handle h, double damping);
/* DampedNVE::step (src/integrator/damped_nve.cu:15-25) n times, device-resident */
int dpg_bumpy_damped_nve_steps(dpg_bumpy_handle h, double dt, double damping, int64_t n_steps);
/* with_pairs = 0: calculateWallForces_onlyWallContacts (rigid_bumpy.cu:1495-1499);
 * with_pairs = 1: calculateWallForces then calculateForces (the pair NVE::wall_step
 * calls); += into the body arrays.  Walls at 0 and L on both axes
 * (calcWallInteraction, include/particles/base/kernels.cuh:185-235) act on vertices */
int dpg_bumpy_wall_forces(dpg_bumpy_handle h, int with_pairs);
/* NVE::wall_step (src/integrator/nve.cu:27-38) n times, device-resident */
int dpg_bumpy_nve_wall_steps(dpg_bumpy_handle h, double dt, int64_t n_steps);
/* calculateStressTensor + getPressure / getStressTensor (rigid_bumpy.cu:1513-1519,
 * kernels.cu:705-789, particle.cu:1371-1385).  stress = {xx, xy, yx, yy} sums;
 * per_body (nullable, host, 4 * n_bodies: [component][body], static order) */
int dpg_bumpy_stress(dpg_bumpy_handle h, double *stress, double *pressure, double *per_body);
/* countContacts + getContactCount / getVertexContactCount (rigid_bumpy.cu:1505-1511,
 * 779-781, kernels.cu:924-997); per-body arrays nullable, host, static order */
int dpg_bumpy_contacts(dpg_bumpy_handle h, double *contacts, double *vertex_contacts,
                       int32_t *per_body, int32_t *vertex_per_body);
/* RigidBumpy::calculateForceDistancePairs (rigid_bumpy.cu:1383-1459, kernel
 * kernels.cu:482-703): arrays of n_bodies * cap (cap from
 * dpg_bumpy_neighbor_info_get), [slot * cap + k] in the current (cell-sorted)
 * slot order, the reference's fill values where an entry is unused.  out[30]
 * (NULL entries skipped): pair energy, force x, force y, separation x, y,
 * overlap (distance - radius sum), radius sum, separation angle, angle i,
 * angle j, friction coefficient, summed vertex overlap, pair Hessian xx, xy,
 * xt, yx, yy, yt, tx, ty, tt, self Hessian xx, xy, xt, yx, yy, yt, tx, ty, tt.
 * this_id / other_id: static body indices; vertex_contacts: this body's
 * vertices touching the other body.  where: DPG_HOST or DPG_DEVICE pointers. */
int dpg_bumpy_pair_dump(dpg_bumpy_handle h, double *const *out, int64_t *this_id,
                        int64_t *other_id, int64_t *vertex_contacts, int where);
/* sizes, static arrays (static body / vertex order) and the box */
int dpg_bumpy_counts(dpg_bumpy_handle h, int64_t *n_bodies, int64_t *n_vertices);
int dpg_bumpy_get_static(dpg_bumpy_handle h, double *radii, double *masses,
                         int32_t *n_vertices_per_body, double *vertex_masses, double *box);
/* body masses, moments of inertia and vertex masses as given (static order),
 * as RigidBumpy::loadDataFromPath sets them from a state directory */
int dpg_bumpy_set_inertia(dpg_bumpy_handle h, const double *masses, const double *inertia,
                          const double *vertex_masses);
/* Particle::setBoxSize; the cell size follows the box (updateCellSize) */
int dpg_bumpy_set_box(dpg_bumpy_handle h, double box_x, double box_y);
/* State directory in the reference's layout (one "%.17e" text file per array,
 * static order): the disk files (positions, velocities, forces, radii, masses,
 * potential_energy, box_size) plus angles, angular_velocities, torques,
 * moments_of_inertia, num_vertices_in_particle (integers), vertex_positions
 * and vertex_masses (static vertex order) -- RigidBumpy's fundamental values
 * (include/particles/rigid_bumpy/rigid_bumpy.h:32); step.dat when step >= 0.
 * The reader follows RigidBumpy::loadDataFromPath (rigid_bumpy.cu:310-371):
 * positions, radii, masses, box_size, num_vertices_in_particle and
 * vertex_positions required; velocities, angles, angular velocities optional
 * (zero); moments of inertia and vertex masses computed as setMass does when
 * absent.  The handle's body and vertex counts must match the directory's
 * (dpg_bumpy_state_count). */
int dpg_bumpy_write_state(dpg_bumpy_handle h, const char *dir, int64_t step);
int dpg_bumpy_read_state(dpg_bumpy_handle h, const char *dir);
int dpg_bumpy_state_count(const char *dir, int64_t *n_bodies, int64_t *n_vertices);
/* getPackingFraction for rigid bodies: pi sum R^2 of the body radii over the
 * box area (RigidBumpy::getParticleArea, rigid_bumpy.cu:1026-1030) */
int dpg_bumpy_packing_fraction(dpg_bumpy_handle h, double *phi);
/* scripts/runArthurJamWithFire.cpp:36-106 on rigid bodies (dpg_jam_pressure's
 * control flow with the rigid calls); minimisations stop on p->fire's tests
 * plus max|tau| <= tmax_target when p->fire.fmax_target > 0; the saved
 * unjammed state is reloaded as RigidBumpy::load does, then setupNeighbors */
int dpg_bumpy_jam_pressure(dpg_bumpy_handle h, const dpg_jam_params *p, double tmax_target,
                           dpg_jam_result *r);
/* setLastState / revertToLastState (rigid_bumpy.cu:1144-1179, particle.cu:956-991):
 * device-side snapshot; the revert restores the box and rebuilds the body and
 * vertex lists from the cell arrays as they are */
int dpg_bumpy_save_state(dpg_bumpy_handle h);
int dpg_bumpy_restore_state(dpg_bumpy_handle h);

/* ======================================================================
 *  Ensembles: the batched form.  Many independent disk systems of uneven
 *  size (each with its own box, neighbour list, FIRE dt/alpha/counters and
 *  convergence state) advanced together: every kernel launch covers all
 *  systems, finished systems are masked out, and the whole loop is one CUDA
 *  graph.  No reference counterpart as an API: the reference runs one system
 *  per process (its state lives in __constant__ symbols); an ensemble runs
 *  the same per-system algorithms (minimizeFire, the pressure-band jamming of
 *  scripts/runArthurJamWithFire.cpp) for S systems at once.
 * ====================================================================== */
typedef struct dpg_ensemble_system *dpg_ensemble;

typedef struct {
    int64_t n_systems;
    double e_c, n_c;
    double cutoff;      /* neighbour cutoff (absolute, e.g. d_max + skin) */
    double skin;        /* lists rebuilt when a particle moved more than skin / 2 */
    int precision;      /* DPG_FP64, or DPG_MIXED (FP32 pair forces, then FP64 refinement) */
    int reserved;
    double switch_fmax; /* DPG_MIXED: FP32 pair forces until max|F| <= switch_fmax (0: 1e-6)
                           or until max|F| stops falling within 100 switch_fmax;
                           FP64 pair forces after */
} dpg_ensemble_params;

typedef struct {
    double avg_pe, max_force, pressure, packing_fraction, box_length, contacts;
    int64_t fire_steps;     /* force passes over the whole run */
    int64_t minimizations;
    int64_t rebuilds;
    int status;             /* jamming: 0 final state, 1 length tolerance, 2 out of steps */
    int converged;
    int64_t fp64_steps;     /* force passes with FP64 pair arithmetic (mixed: the final check) */
    int64_t dw_steps;       /* force passes with double-word FP32 pairs (mixed: the refinement) */
} dpg_ensemble_result;

/* n_particles[s], box[s] (square boxes) */
int dpg_ensemble_create(const dpg_ensemble_params *p, const int64_t *n_particles, const double *box,
                        void *cuda_stream, dpg_ensemble *out);
int dpg_ensemble_destroy(dpg_ensemble e);
/* host arrays, system after system (sum of n_particles entries each) */
int dpg_ensemble_set_state(dpg_ensemble e, const double *x, const double *y, const double *radii,
                           const double *masses);
int dpg_ensemble_get_state(dpg_ensemble e, double *x, double *y, double *fx, double *fy);
/* minimizeFire on every system (p->fmax_target > 0 adds the max|F_i| stop) */
int dpg_ensemble_fire_minimize(dpg_ensemble e, const dpg_fire_params *p, dpg_ensemble_result *per_system);
/* One force pass on every system at its current positions (cell and neighbour
 * lists rebuilt first): forces readable with dpg_ensemble_get_state, and
 * per-system avg_pe, max_force, pressure and contacts in per_system (may be
 * NULL).  precision DPG_FP64 uses the reference pair arithmetic, DPG_MIXED
 * the FP32 pair forces, DPG_DWORD the double-word FP32 pairs of the
 * refinement (systems with fewer than 3 cells a side use FP64).
 * Disk::calculateForces (src/particles/disk/disk.cu:218-221) for a batch. */
int dpg_ensemble_compute_forces(dpg_ensemble e, int precision, dpg_ensemble_result *per_system);
/* pressure-band jamming of every system (the dpg_jam_pressure control flow) */
int dpg_ensemble_jam(dpg_ensemble e, const dpg_jam_params *p, dpg_ensemble_result *per_system);

/* Execution forms of an ensemble run (the same FIRE / jamming algorithm; the
 * grid and persistent forms share the per-slot arithmetic, the resident form
 * keeps positions as FP64 cell centres plus double-word FP32 offsets; totals
 * round differently in each):
 *  DPG_FORM_GRID     every stage is one launch over all systems, the loop a
 *                    CUDA graph (best for few large systems);
 *  DPG_FORM_PERSIST  one persistent block per system runs its whole
 *                    minimisation / jamming protocol with no further launches
 *                    (no grid-wide synchronisation; each system at its own pace);
 *  DPG_FORM_RESIDENT one block or cluster per system holds the system on chip (packed
 *                    offsets and cell lists in shared memory, per-particle
 *                    dynamics in registers) for time-sliced persistent launches;
 *                    FP64 pair arithmetic only verifies double-word states and
 *                    measures finished minimisations; systems of at most 16384
 *                    particles, in size classes that run side by side, each
 *                    launch carrying as many clusters of a class as the GPU
 *                    holds at once (the class's systems take turns);
 *  DPG_FORM_AUTO     the resident form when it holds every system, else the
 *                    grid form, or the form dpg_ensemble_autotune chose. */
#define DPG_FORM_AUTO 0
#define DPG_FORM_GRID 1
#define DPG_FORM_PERSIST 2
#define DPG_FORM_RESIDENT 3
/* threads: persistent form's threads per system block (128, 256 or 512; 0 = by size) */
int dpg_ensemble_set_form(dpg_ensemble e, int form, int threads);
/* Launches the host has issued for this ensemble so far (no reference
 * counterpart; a measurement hook): every kernel launch, and a CUDA-graph
 * launch as one (the grid form's loop runs its kernels inside one graph). */
int dpg_ensemble_launch_count(dpg_ensemble e, int64_t *count);

typedef struct {
    int form;                  /* chosen form (DPG_FORM_GRID / _PERSIST / _RESIDENT) */
    int threads;               /* chosen threads per system block (persistent form) */
    double skin;               /* chosen Verlet skin (the cutoff moves with it) */
    int n_candidates;
    int cand_form[16], cand_threads[16];
    double cand_skin[16];
    double cand_rate[16];      /* particle-iterations per second of each candidate */
} dpg_ensemble_tuning;

/* Autotuner (no reference counterpart): times `iters` FIRE iterations from
 * the current positions for each execution form, persistent block size (128,
 * 256, 512) and Verlet skin (1, 0.75, 0.5 x the current skin; the cutoff
 * shrinks with it, the cell grid stays), restoring the positions after each
 * trial, and keeps the fastest by particle-iterations per second. */
int dpg_ensemble_autotune(dpg_ensemble e, const dpg_fire_params *p, int iters, dpg_ensemble_tuning *out);

/* ---- threads per particle of the FP64 force kernels ------------------- */
/* Lanes per particle (1, 2, 4, 8) of the FP64 force kernels: lane g sums
 * neighbour slots g, g + G, ... and the pair terms are added in slot order
 * through shuffles, so every group gives bit-identical forces.  The default
 * is chosen from the particle count; DPG_MIXED systems use one lane. */
int dpg_set_force_group(dpg_handle h, int lanes);
/* Autotuner (no reference counterpart): times `iters` force passes for each
 * group on the current positions and lists, keeps the fastest (*chosen) and
 * restores the forces and energies; us_per_pass[4] (nullable): mean device
 * time per pass for 1, 2, 4, 8 lanes. */
int dpg_autotune_force_group(dpg_handle h, int iters, int *chosen, double *us_per_pass);

/* ---- measurement ------------------------------------------------------ */
/* Runs `iters` iterations of a device loop (kind 0 = FIRE from the current
 * state, as dpg_fire_minimize's body; kind 1 = NVE with step dt) as plain
 * stream launches with a CUDA-event pair around each phase, and returns the
 * mean device time per iteration of each phase in avg_us[3] (0 = move /
 * first half, 1 = neighbour check + rebuild kernels, 2 = forces + kick) and
 * counts[3] = {iterations, neighbour-list builds, cell-list builds}.  No
 * reference counterpart: this is the measurement hook bench.py uses for the
 * per-kernel roofline. */
int dpg_profile_loop(dpg_handle h, int kind, int iters, double dt, double *avg_us, int64_t *counts);
/* The ensemble's FIRE loop from a fresh start (the dpg_ensemble_fire_minimize
 * parameters), `iters` iterations as plain stream launches with events around
 * each phase: avg_us[4] = mean device time per iteration of move, cell/list
 * rebuild kernels, forces (+ per-system reductions and FIRE decisions),
 * transition; counts[3] = {iterations, list rebuilds summed over systems,
 * force passes summed over systems}.  Leaves the systems mid-minimisation
 * (set the state again before a solve).  No reference counterpart. */
int dpg_ensemble_profile_loop(dpg_ensemble e, const dpg_fire_params *p, int iters, double *avg_us,
                              int64_t *counts);

/* Measured multiply-add throughput of the current GPU (no reference
 * counterpart; the roofline denominator of arithmetic-bound kernels): fp64 = 1
 * for the FP64 pipe, 0 for FP32; `iters` rounds of 8 independent FMA chains
 * per thread over 8 blocks of 256 threads per SM, one launch timed with CUDA
 * events.  *tflops = 2 x FMAs / time; *ms (nullable) = the launch's time. */
int dpg_measure_fma_peak(int fp64, int iters, double *tflops, double *ms);

/* ---- forces without device allocation --------------------------------- */
/* No counterpart in the reference.  Harmonic forces fx, fy and per-particle
 * energies pe of n disks (device arrays, any order, square box of side
 * box_x == box_y), the same values as dpg_setup_neighbors + dpg_compute_forces
 * up to summation order, for callers that cannot call cudaMalloc: hosts that
 * give all device memory to their own fixed pool up front, and real-time
 * loops that cannot wait on the allocator's locks and synchronisation.  The
 * cell list lives in one fixed array inside the library (about 1 MiB on every
 * GPU that loads it, held until exit), so n is at most 65536 and
 * box_x / max_diameter below 257; larger inputs return DPG_ERR_ARG.
 * max_diameter must be at least the largest 2 * radius.  The first call on a
 * device (and the first after its context was reset) looks the array's
 * address up; make that first call before any stream capture.  Calls share
 * the array: calls that overlap on the GPU race, so serialise them on one
 * stream.  Work is queued on cuda_stream (NULL = legacy default stream); the
 * function does not synchronise. */
int dpg_disk_forces_noalloc(const double *x, const double *y, const double *radii, int64_t n,
                            double box_x, double box_y, double e_c, double n_c,
                            double max_diameter, double *fx, double *fy, double *pe,
                            void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
