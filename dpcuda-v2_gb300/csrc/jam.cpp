// jam.cpp -- jamming drivers over the C ABI: the control flow of the
// reference's run scripts (scripts/runArthurJamWithFire.cpp,
// scripts/runJam.cpp), restated as host C++, for disks and (the pressure-band
// driver) rigid bumpy bodies.  Every particle operation goes through the
// dpg_* / dpg_bumpy_* entry points, so the drivers run the GPU hot path.
#include <cmath>
#include <vector>

#include "host_common.h"

using dpg::set_error;

namespace {

struct Saved {
    std::vector<double> x, y, r, m;
    double bx = 0, by = 0;
};

double box_length(dpg_handle h) {
    double bx, by;
    dpg_get_box(h, &bx, &by);
    return std::pow(1.0 * bx * by, 1.0 / 2);
}

// write_restart_file("last_state"): positions, velocities, radii, masses,
// box, all in static order (src/io/state_log.cu:27-66)
int save(dpg_handle h, int64_t n, Saved &s) {
    s.x.resize(n); s.y.resize(n); s.r.resize(n); s.m.resize(n);
    DPG_TRY(dpg_get_state(h, s.x.data(), s.y.data(), nullptr, nullptr, nullptr, nullptr, nullptr, DPG_HOST));
    DPG_TRY(dpg_get_static_params(h, s.r.data(), s.m.data()));
    DPG_TRY(dpg_get_box(h, &s.bx, &s.by));
    return DPG_OK;
}

// Disk::load("last_state") (src/particles/disk/disk.cu:35-96): arrays in
// static order, box, then setupNeighbors (full neighbour initialisation)
int load(dpg_handle h, const Saved &s, const dpg_neighbor_config &cfg) {
    std::vector<double> z(s.x.size(), 0.0);
    DPG_TRY(dpg_set_box(h, s.bx, s.by));
    DPG_TRY(dpg_load_state(h, s.x.data(), s.y.data(), z.data(), z.data(), s.r.data(), s.m.data(), DPG_HOST));
    DPG_TRY(dpg_setup_neighbors(h, &cfg, nullptr));
    return DPG_OK;
}

}  // namespace

extern "C" int dpg_jam_pressure(dpg_handle h, const dpg_jam_params *p, dpg_jam_result *r) {
    if (!h || !p || !r) return set_error(DPG_ERR_ARG, "dpg_jam_pressure: null argument");
    dpg_params prm;
    DPG_TRY(dpg_get_params(h, &prm));
    const int64_t np = prm.n_particles;
    dpg_fire_result fr;
    int64_t fire_total = 0;
    // decompress until P < pressure_low (scripts/runArthurJamWithFire.cpp:36-45):
    // minimizeFire(1e-16, 0) then pressure
    dpg_fire_params dec = p->fire;
    dec.avg_pe_target = 1e-16;
    dec.avg_pe_diff_target = 0.0;
    double P = 0.0;
    for (int guard = 0;; guard++) {
        if (guard > 10000) return set_error(DPG_ERR_NOT_CONVERGED, "decompression did not end");
        DPG_TRY(dpg_fire_minimize(h, &dec, &fr));
        fire_total += fr.steps + 1;
        DPG_TRY(dpg_pressure(h, &P, nullptr));
        if (P < p->pressure_low) break;
        DPG_TRY(dpg_scale_box(h, p->decompress_factor));
    }
    Saved last;
    double L_low = -1, L_high = -1, L_last = -1;
    int64_t step = 0;
    int status = 2;
    double contacts = 0;
    while (step < p->max_compression_steps) {
        DPG_TRY(dpg_fire_minimize(h, &p->fire, &fr));
        fire_total += fr.steps + 1;
        DPG_TRY(dpg_pressure(h, &P, nullptr));
        DPG_TRY(dpg_contact_count(h, &contacts));
        double L = box_length(h);
        double L_prior = L;
        if (P < p->pressure_low) {
            L_low = L;
            DPG_TRY(save(h, np, last));
            L_last = L;
            if (L_high != -1) {
                L = (L_high + L_low) / 2;
                L_high = -1;
            } else {
                L = L * p->compression_rate;
            }
        } else {
            if (P > p->pressure_high) {
                L_high = L;
                if (L_last < 0) return set_error(DPG_ERR_STATE, "jammed before any unjammed state was saved");
                DPG_TRY(load(h, last, p->neighbors));
                L_prior = L_last;
                L = (L_high + L_low) / 2;
            } else if (contacts > 2 * np) {
                status = 0;
                break;
            }
        }
        if (L_low > 0 && L_high > 0 && std::abs(L_low / L_high - 1) < p->length_tolerance) {
            status = 1;
            break;
        }
        DPG_TRY(dpg_scale_box(h, L / L_prior));
        step++;
    }
    DPG_TRY(dpg_pressure(h, &P, nullptr));
    DPG_TRY(dpg_contact_count(h, &contacts));
    DPG_TRY(dpg_packing_fraction(h, &r->packing_fraction));
    r->pressure = P;
    r->box_length = box_length(h);
    r->contacts = contacts;
    r->compression_steps = step;
    r->fire_steps_total = fire_total;
    r->status = status;
    return DPG_OK;
}

// minimizeFire(particle, tol, difftol[, steps]) with the defaults alpha 0.1, dt 1e-2
static int fire_pe(dpg_handle h, double tol, double dtol, int64_t steps, int64_t *total) {
    dpg_fire_params fp = {0.1, 1e-2, tol, dtol, steps, 0.0};
    dpg_fire_result fr;
    DPG_TRY(dpg_fire_minimize(h, &fp, &fr));
    *total += fr.steps + 1;
    return DPG_OK;
}

static int avg_pe(dpg_handle h, int64_t n, double *pe) {
    double ke;
    DPG_TRY(dpg_reduce_energies(h, pe, &ke));
    *pe /= (double)n;
    return DPG_OK;
}

extern "C" int dpg_jam_phi(dpg_handle h, const dpg_jam_phi_params *p, dpg_jam_result *r) {
    if (!h || !p || !r) return set_error(DPG_ERR_ARG, "dpg_jam_phi: null argument");
    dpg_params prm;
    DPG_TRY(dpg_get_params(h, &prm));
    const int64_t np = prm.n_particles;
    int64_t total = 0;
    const double tol = p->avg_pe_tolerance, dtol = p->avg_pe_diff_tolerance;
    double pe = 0;
    // start with no contacts (scripts/runJam.cpp:42-49)
    for (int guard = 0;; guard++) {
        if (guard > 10000) return set_error(DPG_ERR_NOT_CONVERGED, "decompression did not end");
        DPG_TRY(fire_pe(h, tol, dtol, 100000, &total));
        DPG_TRY(avg_pe(h, np, &pe));
        if (pe < tol) break;
        DPG_TRY(dpg_scale_box(h, 1.1));
    }
    DPG_TRY(dpg_save_state(h));
    double phi_low, phi, phi_high = -1.0;
    DPG_TRY(dpg_packing_fraction(h, &phi_low));
    int64_t step = 0;
    int status = 2;
    while (step < p->max_compression_steps) {
        DPG_TRY(dpg_packing_fraction(h, &phi));
        DPG_TRY(fire_pe(h, tol, dtol, 1000000, &total));
        DPG_TRY(avg_pe(h, np, &pe));
        if (pe > tol) {  // jammed
            phi_high = phi;
            phi = (phi_high + phi_low) / 2.0;
            DPG_TRY(dpg_restore_state(h));
        } else {
            DPG_TRY(dpg_save_state(h));
            phi_low = phi;
            if (phi_high > 0) phi = (phi_high + phi_low) / 2.0;
            else phi += p->compression_increment;
        }
        if (std::abs(phi_high / phi_low - 1) < p->phi_tolerance) {
            // is_stable_configuration (scripts/runJam.cpp:15-23)
            double cur;
            DPG_TRY(dpg_save_state(h));
            DPG_TRY(dpg_packing_fraction(h, &cur));
            DPG_TRY(dpg_scale_to_packing_fraction(h, cur + p->delta_phi_stability));
            DPG_TRY(fire_pe(h, tol, dtol, 100000, &total));
            double fin;
            DPG_TRY(avg_pe(h, np, &fin));
            DPG_TRY(dpg_restore_state(h));
            bool stable = fin > 1e-1 * std::pow(p->delta_phi_stability, prm.n_c);
            if (stable) { status = 0; break; }
            phi_low = phi;
            phi_high = -1.0;
            DPG_TRY(dpg_packing_fraction(h, &phi));
            DPG_TRY(dpg_save_state(h));
        }
        DPG_TRY(dpg_scale_to_packing_fraction(h, phi));
        step++;
    }
    double P, contacts;
    DPG_TRY(dpg_pressure(h, &P, nullptr));
    DPG_TRY(dpg_contact_count(h, &contacts));
    DPG_TRY(dpg_packing_fraction(h, &r->packing_fraction));
    r->pressure = P;
    r->box_length = box_length(h);
    r->contacts = contacts;
    r->compression_steps = step;
    r->fire_steps_total = total;
    r->status = status;
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// rigid bumpy bodies
// ---------------------------------------------------------------------------
namespace {

// write_restart_file("last_state") for rigid bodies: RigidBumpy's fundamental
// values (include/particles/rigid_bumpy/rigid_bumpy.h:32) in static order
struct SavedBumpy {
    std::vector<double> x, y, th, vx, vy, w, r, m, I, px, py, vm;
    std::vector<int32_t> nvb;
    double box[2] = {0, 0};
};

int bsave(dpg_bumpy_handle h, SavedBumpy &s) {
    int64_t nb = 0, nv = 0;
    DPG_TRY(dpg_bumpy_counts(h, &nb, &nv));
    for (auto *v : {&s.x, &s.y, &s.th, &s.vx, &s.vy, &s.w, &s.r, &s.m, &s.I}) v->resize(nb);
    s.nvb.resize(nb);
    s.px.resize(nv); s.py.resize(nv); s.vm.resize(nv);
    DPG_TRY(dpg_bumpy_get_bodies(h, s.x.data(), s.y.data(), s.th.data(), s.vx.data(), s.vy.data(),
                                 s.w.data(), nullptr, nullptr, nullptr, nullptr, s.I.data()));
    DPG_TRY(dpg_bumpy_get_vertices(h, s.px.data(), s.py.data()));
    DPG_TRY(dpg_bumpy_get_static(h, s.r.data(), s.m.data(), s.nvb.data(), s.vm.data(), s.box));
    return DPG_OK;
}

// RigidBumpy::load("last_state") (loadDataFromPath, rigid_bumpy.cu:310-371),
// then setupNeighbors
int bload(dpg_bumpy_handle h, const SavedBumpy &s, const dpg_neighbor_config &cfg) {
    DPG_TRY(dpg_bumpy_set_box(h, s.box[0], s.box[1]));
    DPG_TRY(dpg_bumpy_set_bodies(h, s.x.data(), s.y.data(), s.th.data(), s.vx.data(), s.vy.data(),
                                 s.w.data(), s.r.data(), s.nvb.data()));
    DPG_TRY(dpg_bumpy_set_vertices(h, s.px.data(), s.py.data()));
    DPG_TRY(dpg_bumpy_set_inertia(h, s.m.data(), s.I.data(), s.vm.data()));
    DPG_TRY(dpg_bumpy_zero_forces(h));
    DPG_TRY(dpg_bumpy_setup_neighbors(h, &cfg, nullptr));
    return DPG_OK;
}

double bbox_length(dpg_bumpy_handle h) {
    double box[2] = {1, 1};
    dpg_bumpy_get_static(h, nullptr, nullptr, nullptr, nullptr, box);
    return std::pow(1.0 * box[0] * box[1], 1.0 / 2);
}

}  // namespace

// RigidBumpy::getParticleArea (rigid_bumpy.cu:1026-1030: pi sum R^2 of the body
// radii) over the box area: Particle::getPackingFraction (particle.cu:1011-1015)
extern "C" int dpg_bumpy_packing_fraction(dpg_bumpy_handle h, double *phi) {
    if (!h || !phi) return set_error(DPG_ERR_ARG, "null argument");
    int64_t nb = 0, nv = 0;
    DPG_TRY(dpg_bumpy_counts(h, &nb, &nv));
    std::vector<double> r(nb);
    double box[2];
    DPG_TRY(dpg_bumpy_get_static(h, r.data(), nullptr, nullptr, nullptr, box));
    double a = 0.0;
    for (double v : r) a += v * v;
    *phi = a * 3.141592653589793238462643383279502884197 / (1.0 * box[0] * box[1]);
    return DPG_OK;
}

// scripts/runArthurJamWithFire.cpp:36-106 on rigid bumpy bodies
extern "C" int dpg_bumpy_jam_pressure(dpg_bumpy_handle h, const dpg_jam_params *p, double tmax_target,
                                      dpg_jam_result *r) {
    if (!h || !p || !r) return set_error(DPG_ERR_ARG, "dpg_bumpy_jam_pressure: null argument");
    int64_t nb = 0, nv = 0;
    DPG_TRY(dpg_bumpy_counts(h, &nb, &nv));
    dpg_fire_result fr;
    int64_t fire_total = 0;
    dpg_fire_params dec = p->fire;
    dec.avg_pe_target = 1e-16;
    dec.avg_pe_diff_target = 0.0;
    double P = 0.0, contacts = 0.0;
    for (int guard = 0;; guard++) {
        if (guard > 10000) return set_error(DPG_ERR_NOT_CONVERGED, "decompression did not end");
        DPG_TRY(dpg_bumpy_fire_minimize(h, &dec, tmax_target, &fr));
        fire_total += fr.steps + 1;
        DPG_TRY(dpg_bumpy_stress(h, nullptr, &P, nullptr));
        if (P < p->pressure_low) break;
        DPG_TRY(dpg_bumpy_scale_box(h, p->decompress_factor));
    }
    SavedBumpy last;
    double L_low = -1, L_high = -1, L_last = -1;
    int64_t step = 0;
    int status = 2;
    while (step < p->max_compression_steps) {
        DPG_TRY(dpg_bumpy_fire_minimize(h, &p->fire, tmax_target, &fr));
        fire_total += fr.steps + 1;
        DPG_TRY(dpg_bumpy_stress(h, nullptr, &P, nullptr));
        DPG_TRY(dpg_bumpy_contacts(h, &contacts, nullptr, nullptr, nullptr));
        double L = bbox_length(h);
        double L_prior = L;
        if (P < p->pressure_low) {
            L_low = L;
            DPG_TRY(bsave(h, last));
            L_last = L;
            if (L_high != -1) {
                L = (L_high + L_low) / 2;
                L_high = -1;
            } else {
                L = L * p->compression_rate;
            }
        } else {
            if (P > p->pressure_high) {
                L_high = L;
                if (L_last < 0) return set_error(DPG_ERR_STATE, "jammed before any unjammed state was saved");
                DPG_TRY(bload(h, last, p->neighbors));
                L_prior = L_last;
                L = (L_high + L_low) / 2;
            } else if (contacts > 2 * nb) {
                status = 0;
                break;
            }
        }
        if (L_low > 0 && L_high > 0 && std::abs(L_low / L_high - 1) < p->length_tolerance) {
            status = 1;
            break;
        }
        DPG_TRY(dpg_bumpy_scale_box(h, L / L_prior));
        step++;
    }
    DPG_TRY(dpg_bumpy_stress(h, nullptr, &P, nullptr));
    DPG_TRY(dpg_bumpy_contacts(h, &contacts, nullptr, nullptr, nullptr));
    DPG_TRY(dpg_bumpy_packing_fraction(h, &r->packing_fraction));
    r->pressure = P;
    r->box_length = bbox_length(h);
    r->contacts = contacts;
    r->compression_steps = step;
    r->fire_steps_total = fire_total;
    r->status = status;
    return DPG_OK;
}
