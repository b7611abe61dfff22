/*
 * dpg_oracle.h -- CPU oracle for the 2D granular contact hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64 restatement of the
 * reference (mmccraw98/dpCUDA-v2) disk and rigid-bumpy algorithms, used by the
 * test-suite as the parity checker and by bench.py as the timed CPU baseline.
 * Nothing in the product library links or calls it.
 *
 * Every function cites the reference file:line it restates.  Arithmetic is
 * written operation-for-operation in the reference's order and the file is
 * compiled with -ffp-contract=off, so per-particle results are bit-identical
 * to the reference kernels compiled on the host (oracle/ref) and to the
 * product's FP64 CUDA kernels (which are compiled with --fmad=false).
 *
 * Array conventions follow the reference: "current" order is the cell-sorted
 * order; static_index[i] is the original (input) index of the particle
 * stored at slot i; neighbour lists are row-major [n * cap] int64 padded with
 * -1 (src/particles/base/particle.cu:1320-1331).
 */
#ifndef DPG_ORACLE_H
#define DPG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* neighbour methods, src/particles/base/particle.cu:237-265 */
enum { ORC_NEIGH_CELL = 0, ORC_NEIGH_VERLET = 1, ORC_NEIGH_ALL = 2 };

typedef struct orc_sys orc_sys;

/* ---- lifetime / state ------------------------------------------------- */
orc_sys *orc_create(int64_t n, double box_x, double box_y, double e_c, double n_c);
void orc_destroy(orc_sys *s);
/* arrays in static (input) order; any pointer may be NULL (left unchanged) */
void orc_set_arrays(orc_sys *s, const double *x, const double *y, const double *vx,
                    const double *vy, const double *r, const double *m);
void orc_set_forces(orc_sys *s, const double *fx, const double *fy);
/* arrays back in static order (reference IO un-permutes by static index) */
void orc_get_arrays(const orc_sys *s, double *x, double *y, double *vx, double *vy,
                    double *fx, double *fy, double *pe, double *r, double *m);
/* raw current-order views (for bit-level comparisons) */
void orc_get_current(const orc_sys *s, double *x, double *y, double *vx, double *vy,
                     double *fx, double *fy, double *pe, int64_t *static_index);
void orc_set_box(orc_sys *s, double bx, double by);
void orc_get_box(const orc_sys *s, double *bx, double *by);
void orc_set_threads(int nthreads);

/* ---- neighbours -------------------------------------------------------- */
int orc_setup_neighbors(orc_sys *s, int method, double cutoff_mult, double disp_mult,
                        double particles_per_cell, double cell_disp_mult);
void orc_update_neighbor_list(orc_sys *s);
int orc_check_for_neighbor_update(orc_sys *s); /* returns 1 if rebuilt */
void orc_neighbor_info(const orc_sys *s, int *method, double *cutoff, double *thr2,
                       int64_t *n_cells_dim, double *cell_size, double *cell_thr2,
                       int64_t *cap);
/* list in current order (row-major, -1 padded); counts[n] */
void orc_get_neighbors(const orc_sys *s, int64_t *list, int64_t *counts);
void orc_get_cells(const orc_sys *s, int64_t *cell_index, int64_t *cell_start);
int64_t orc_num_rebuilds(const orc_sys *s, int64_t *n_cell_rebuilds);

/* ---- forces / dynamics ------------------------------------------------- */
void orc_zero_force_and_pe(orc_sys *s);
void orc_calculate_forces(orc_sys *s); /* += into F, PE (reference semantics) */
void orc_update_velocities(orc_sys *s, double dt);
void orc_update_positions(orc_sys *s, double dt);
void orc_mix_velocities_and_forces(orc_sys *s, double alpha);
void orc_set_velocities_zero(orc_sys *s);
double orc_power_fire(orc_sys *s);
double orc_total_pe(orc_sys *s);
double orc_total_ke(orc_sys *s); /* computes per-particle KE first */
double orc_max_force(orc_sys *s);
double orc_force_balance(orc_sys *s);
void orc_nve_steps(orc_sys *s, double dt, int64_t n_steps);
void orc_damped_forces(orc_sys *s, double gamma);                    /* F -= gamma v */
void orc_damped_nve_steps(orc_sys *s, double dt, double gamma, int64_t n_steps);
void orc_update_positions_grad_desc(orc_sys *s, double alpha);       /* x += alpha F */
void orc_grad_desc_steps(orc_sys *s, double alpha, int64_t n_steps);
void orc_wall_forces(orc_sys *s);                                    /* += wall force / energy */
void orc_pair_dump(orc_sys *s, double *const *d, int64_t *this_id, int64_t *other_id);
void orc_nve_wall_steps(orc_sys *s, double dt, int64_t n_steps);

/* ---- FIRE -------------------------------------------------------------- */
void orc_fire_init(orc_sys *s, double alpha_init, double dt);
int orc_fire_step(orc_sys *s); /* returns stopped flag */
void orc_fire_state(const orc_sys *s, double *alpha, double *dt, int64_t *n_good,
                    int64_t *n_bad, int *stopped);
/* minimizeFire; fmax_target > 0 adds a max|F_i| <= fmax_target stop */
int64_t orc_minimize_fire(orc_sys *s, double alpha_init, double dt, double pe_target,
                          double pe_diff_target, int64_t num_steps, double fmax_target,
                          int *stopped_out);

/* ---- Adam -------------------------------------------------------------- */
void orc_init_adam(orc_sys *s);
void orc_adam_step(orc_sys *s, int64_t step, double alpha, double beta1, double beta2,
                   double eps);
int64_t orc_minimize_adam(orc_sys *s, double alpha, double beta1, double beta2, double eps,
                          double pe_target, double pe_diff_target, int64_t num_steps);

/* ---- jamming pieces ---------------------------------------------------- */
void orc_stress_tensor(orc_sys *s, double out[4]);
double orc_pressure(orc_sys *s);
double orc_contact_count(orc_sys *s);
double orc_particle_area(const orc_sys *s);
double orc_packing_fraction(const orc_sys *s);
void orc_scale_to_packing_fraction(orc_sys *s, double phi); /* ...Full variant */
void orc_scale_box(orc_sys *s, double factor);
void orc_set_last_state(orc_sys *s);
void orc_revert_to_last_state(orc_sys *s);

/* ---- jamming drivers (scripts/runArthurJamWithFire.cpp, scripts/runJam.cpp) */
void orc_load_state(orc_sys *s, const double *x, const double *y, const double *r,
                    const double *m); /* Disk::load: static order, slot order reset */
typedef struct {
    double packing_fraction, pressure, box_length, contacts;
    int64_t compression_steps, fire_steps_total;
    int status;
} orc_jam_result;
void orc_jam_pressure(orc_sys *s, double p_low, double p_high, double compression_rate,
                      double length_tol, double decompress_factor, int64_t max_steps,
                      double fire_alpha, double fire_dt, double pe_target, double pe_diff_target,
                      int64_t fire_max_steps, int method, double cm, double dm, double ppc,
                      double cdm, orc_jam_result *r);
void orc_jam_phi(orc_sys *s, double tol, double dtol, double phi_tol, double increment,
                 double dphi_stab, int64_t max_steps, orc_jam_result *r);

/* ---- seeded initialisation (include/functors.h:17-50) ------------------ */
void orc_fill_uniform(double *out, int64_t n, double lo, double hi, int64_t seed_offset,
                      int64_t seed);
void orc_fill_normal(double *out, int64_t n, double mean, double stddev,
                     int64_t seed_offset, int64_t seed);
double orc_erfcinv(double z);

#ifdef __cplusplus
}
#endif
#endif
