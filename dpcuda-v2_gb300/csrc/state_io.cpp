// state_io.cpp -- system state in the reference's on-disk layout.
//
// The reference writes one text file per array into a state directory
// (system/init, system/restart, trajectories/t<step>): 2-D arrays as
// "x<TAB>y" lines, 1-D arrays one value per line, all in std::scientific with
// 17 digits (include/io/io_utils.h:81-108, include/constants.h:11,
// src/io/state_log.cu:27-41), in static (input) order, plus step.dat in a
// restart directory.  It loads positions, velocities, forces, radii, masses and
// box_size from such a directory (src/particles/base/particle.cu:102-148,
// 180-215).  These entry points read and write the same layout, so runs of the
// reference and of this library can start from each other's states.  Rigid
// bumpy bodies add the RigidBumpy fundamental values (include/particles/
// rigid_bumpy/rigid_bumpy.h:32): angles, angular velocities, vertex counts,
// vertex positions (static vertex order), moments of inertia and vertex
// masses, loaded as RigidBumpy::loadDataFromPath does
// (src/particles/rigid_bumpy/rigid_bumpy.cu:310-371).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "host_common.h"

namespace {

std::string join(const char *dir, const char *name) {
    std::string p(dir);
    if (!p.empty() && p.back() != '/') p += '/';
    return p + name;
}

int make_dirs(const std::string &path) {
    std::string cur;
    size_t pos = 0;
    while (pos != std::string::npos) {
        pos = path.find('/', pos + 1);
        cur = path.substr(0, pos);
        if (cur.empty()) continue;
        if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST)
            return dpg::set_error(DPG_ERR_ARG, "cannot create directory %s: %s", cur.c_str(), strerror(errno));
    }
    return DPG_OK;
}

int write_cols(const std::string &path, const double *a, const double *b, int64_t n) {
    FILE *f = fopen(path.c_str(), "w");
    if (!f) return dpg::set_error(DPG_ERR_ARG, "cannot write %s: %s", path.c_str(), strerror(errno));
    for (int64_t i = 0; i < n; i++) {
        if (b) fprintf(f, "%.17e\t%.17e\n", a[i], b[i]);
        else fprintf(f, "%.17e\n", a[i]);
    }
    int bad = ferror(f);
    fclose(f);
    if (bad) return dpg::set_error(DPG_ERR_ARG, "write error on %s", path.c_str());
    return DPG_OK;
}

// whitespace-separated numbers, as read_array_from_file reads them
int read_values(const std::string &path, int64_t count, std::vector<double> &out, bool required,
                bool *found) {
    *found = false;
    FILE *f = fopen(path.c_str(), "r");
    if (!f) {
        if (required) return dpg::set_error(DPG_ERR_ARG, "cannot read %s", path.c_str());
        return DPG_OK;
    }
    out.resize((size_t)count);
    char tok[128];
    for (int64_t i = 0; i < count; i++) {
        if (fscanf(f, "%127s", tok) != 1) {
            fclose(f);
            return dpg::set_error(DPG_ERR_ARG, "%s: expected %lld values, found %lld", path.c_str(),
                                  (long long)count, (long long)i);
        }
        char *end = nullptr;
        out[(size_t)i] = strtod(tok, &end);
        if (end == tok || *end != '\0') {
            fclose(f);
            return dpg::set_error(DPG_ERR_ARG, "%s: bad number '%s'", path.c_str(), tok);
        }
    }
    fclose(f);
    *found = true;
    return DPG_OK;
}

}  // namespace

namespace {

int write_ints(const std::string &path, const int32_t *a, int64_t n) {
    FILE *f = fopen(path.c_str(), "w");
    if (!f) return dpg::set_error(DPG_ERR_ARG, "cannot write %s: %s", path.c_str(), strerror(errno));
    for (int64_t i = 0; i < n; i++) fprintf(f, "%lld\n", (long long)a[i]);
    int bad = ferror(f);
    fclose(f);
    if (bad) return dpg::set_error(DPG_ERR_ARG, "write error on %s", path.c_str());
    return DPG_OK;
}

int write_step(const char *dir, int64_t step) {
    if (step < 0) return DPG_OK;
    std::string path = join(dir, "step.dat");
    FILE *f = fopen(path.c_str(), "w");
    if (!f) return dpg::set_error(DPG_ERR_ARG, "cannot write %s", path.c_str());
    fprintf(f, "%lld", (long long)step);
    fclose(f);
    return DPG_OK;
}

int count_values(const std::string &path, int64_t *n) {
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return dpg::set_error(DPG_ERR_ARG, "cannot read %s", path.c_str());
    char tok[128];
    int64_t c = 0;
    while (fscanf(f, "%127s", tok) == 1) c++;
    fclose(f);
    *n = c;
    return DPG_OK;
}

}  // namespace

extern "C" int dpg_state_count(const char *dir, int64_t *n_particles) {
    if (!dir || !n_particles) return dpg::set_error(DPG_ERR_ARG, "null argument");
    std::string path = join(dir, "radii.dat");
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return dpg::set_error(DPG_ERR_ARG, "cannot read %s", path.c_str());
    char tok[128];
    int64_t n = 0;
    while (fscanf(f, "%127s", tok) == 1) n++;
    fclose(f);
    *n_particles = n;
    return DPG_OK;
}

extern "C" int dpg_write_state(dpg_handle h, const char *dir, int64_t step) {
    if (!h || !dir) return dpg::set_error(DPG_ERR_ARG, "null argument");
    dpg_params p;
    DPG_TRY(dpg_get_params(h, &p));
    const int64_t n = p.n_particles;
    std::vector<double> x(n), y(n), vx(n), vy(n), fx(n), fy(n), pe(n), r(n), m(n);
    DPG_TRY(dpg_get_state(h, x.data(), y.data(), vx.data(), vy.data(), fx.data(), fy.data(),
                          pe.data(), DPG_HOST));
    DPG_TRY(dpg_get_static_params(h, r.data(), m.data()));
    double box[2];
    DPG_TRY(dpg_get_box(h, &box[0], &box[1]));
    DPG_TRY(make_dirs(dir));
    DPG_TRY(write_cols(join(dir, "positions.dat"), x.data(), y.data(), n));
    DPG_TRY(write_cols(join(dir, "velocities.dat"), vx.data(), vy.data(), n));
    DPG_TRY(write_cols(join(dir, "forces.dat"), fx.data(), fy.data(), n));
    DPG_TRY(write_cols(join(dir, "radii.dat"), r.data(), nullptr, n));
    DPG_TRY(write_cols(join(dir, "masses.dat"), m.data(), nullptr, n));
    DPG_TRY(write_cols(join(dir, "potential_energy.dat"), pe.data(), nullptr, n));
    DPG_TRY(write_cols(join(dir, "box_size.dat"), box, nullptr, 2));
    if (step >= 0) {
        std::string path = join(dir, "step.dat");
        FILE *f = fopen(path.c_str(), "w");
        if (!f) return dpg::set_error(DPG_ERR_ARG, "cannot write %s", path.c_str());
        fprintf(f, "%lld", (long long)step);
        fclose(f);
    }
    return DPG_OK;
}

extern "C" int dpg_read_state(dpg_handle h, const char *dir) {
    if (!h || !dir) return dpg::set_error(DPG_ERR_ARG, "null argument");
    dpg_params p;
    DPG_TRY(dpg_get_params(h, &p));
    const int64_t n = p.n_particles;
    std::vector<double> xy, vxy, r, m, box;
    bool have_xy, have_v, have_r, have_m, have_box;
    DPG_TRY(read_values(join(dir, "positions.dat"), 2 * n, xy, true, &have_xy));
    DPG_TRY(read_values(join(dir, "velocities.dat"), 2 * n, vxy, false, &have_v));
    DPG_TRY(read_values(join(dir, "radii.dat"), n, r, true, &have_r));
    DPG_TRY(read_values(join(dir, "masses.dat"), n, m, true, &have_m));
    DPG_TRY(read_values(join(dir, "box_size.dat"), 2, box, true, &have_box));
    std::vector<double> x(n), y(n), vx(n, 0.0), vy(n, 0.0);
    for (int64_t i = 0; i < n; i++) {
        x[i] = xy[2 * i];
        y[i] = xy[2 * i + 1];
        if (have_v) { vx[i] = vxy[2 * i]; vy[i] = vxy[2 * i + 1]; }
    }
    DPG_TRY(dpg_set_box(h, box[0], box[1]));
    return dpg_load_state(h, x.data(), y.data(), vx.data(), vy.data(), r.data(), m.data(), DPG_HOST);
}

// ---------------------------------------------------------------------------
// rigid bumpy bodies
// ---------------------------------------------------------------------------
extern "C" int dpg_bumpy_state_count(const char *dir, int64_t *n_bodies, int64_t *n_vertices) {
    if (!dir || !n_bodies || !n_vertices) return dpg::set_error(DPG_ERR_ARG, "null argument");
    DPG_TRY(count_values(join(dir, "radii.dat"), n_bodies));
    int64_t v = 0;
    DPG_TRY(count_values(join(dir, "vertex_positions.dat"), &v));
    *n_vertices = v / 2;
    return DPG_OK;
}

extern "C" int dpg_bumpy_write_state(dpg_bumpy_handle h, const char *dir, int64_t step) {
    if (!h || !dir) return dpg::set_error(DPG_ERR_ARG, "null argument");
    int64_t nb = 0, nv = 0;
    DPG_TRY(dpg_bumpy_counts(h, &nb, &nv));
    std::vector<double> x(nb), y(nb), th(nb), vx(nb), vy(nb), w(nb), fx(nb), fy(nb), tq(nb), pe(nb),
        I(nb), r(nb), m(nb), px(nv), py(nv), vm(nv);
    std::vector<int32_t> nvb(nb);
    double box[2];
    DPG_TRY(dpg_bumpy_get_bodies(h, x.data(), y.data(), th.data(), vx.data(), vy.data(), w.data(),
                                 fx.data(), fy.data(), tq.data(), pe.data(), I.data()));
    DPG_TRY(dpg_bumpy_get_vertices(h, px.data(), py.data()));
    DPG_TRY(dpg_bumpy_get_static(h, r.data(), m.data(), nvb.data(), vm.data(), box));
    DPG_TRY(make_dirs(dir));
    DPG_TRY(write_cols(join(dir, "positions.dat"), x.data(), y.data(), nb));
    DPG_TRY(write_cols(join(dir, "velocities.dat"), vx.data(), vy.data(), nb));
    DPG_TRY(write_cols(join(dir, "forces.dat"), fx.data(), fy.data(), nb));
    DPG_TRY(write_cols(join(dir, "radii.dat"), r.data(), nullptr, nb));
    DPG_TRY(write_cols(join(dir, "masses.dat"), m.data(), nullptr, nb));
    DPG_TRY(write_cols(join(dir, "potential_energy.dat"), pe.data(), nullptr, nb));
    DPG_TRY(write_cols(join(dir, "box_size.dat"), box, nullptr, 2));
    DPG_TRY(write_cols(join(dir, "angles.dat"), th.data(), nullptr, nb));
    DPG_TRY(write_cols(join(dir, "angular_velocities.dat"), w.data(), nullptr, nb));
    DPG_TRY(write_cols(join(dir, "torques.dat"), tq.data(), nullptr, nb));
    DPG_TRY(write_cols(join(dir, "moments_of_inertia.dat"), I.data(), nullptr, nb));
    DPG_TRY(write_ints(join(dir, "num_vertices_in_particle.dat"), nvb.data(), nb));
    DPG_TRY(write_cols(join(dir, "vertex_positions.dat"), px.data(), py.data(), nv));
    DPG_TRY(write_cols(join(dir, "vertex_masses.dat"), vm.data(), nullptr, nv));
    return write_step(dir, step);
}

extern "C" int dpg_bumpy_read_state(dpg_bumpy_handle h, const char *dir) {
    if (!h || !dir) return dpg::set_error(DPG_ERR_ARG, "null argument");
    int64_t nb = 0, nv = 0;
    DPG_TRY(dpg_bumpy_counts(h, &nb, &nv));
    std::vector<double> xy, vxy, r, m, box, th, w, I, nvbd, pxy, vm;
    bool f_xy, f_v, f_r, f_m, f_box, f_th, f_w, f_I, f_nvb, f_pxy, f_vm;
    DPG_TRY(read_values(join(dir, "positions.dat"), 2 * nb, xy, true, &f_xy));
    DPG_TRY(read_values(join(dir, "velocities.dat"), 2 * nb, vxy, false, &f_v));
    DPG_TRY(read_values(join(dir, "radii.dat"), nb, r, true, &f_r));
    DPG_TRY(read_values(join(dir, "masses.dat"), nb, m, true, &f_m));
    DPG_TRY(read_values(join(dir, "box_size.dat"), 2, box, true, &f_box));
    DPG_TRY(read_values(join(dir, "angles.dat"), nb, th, false, &f_th));
    DPG_TRY(read_values(join(dir, "angular_velocities.dat"), nb, w, false, &f_w));
    DPG_TRY(read_values(join(dir, "moments_of_inertia.dat"), nb, I, false, &f_I));
    DPG_TRY(read_values(join(dir, "num_vertices_in_particle.dat"), nb, nvbd, true, &f_nvb));
    DPG_TRY(read_values(join(dir, "vertex_positions.dat"), 2 * nv, pxy, true, &f_pxy));
    DPG_TRY(read_values(join(dir, "vertex_masses.dat"), nv, vm, false, &f_vm));
    std::vector<double> x(nb), y(nb), vx(nb, 0.0), vy(nb, 0.0), ang(nb, 0.0), om(nb, 0.0);
    std::vector<int32_t> nvb(nb);
    for (int64_t b = 0; b < nb; b++) {
        x[b] = xy[2 * b];
        y[b] = xy[2 * b + 1];
        if (f_v) { vx[b] = vxy[2 * b]; vy[b] = vxy[2 * b + 1]; }
        if (f_th) ang[b] = th[b];
        if (f_w) om[b] = w[b];
        nvb[b] = (int32_t)nvbd[b];
    }
    std::vector<double> px(nv), py(nv);
    for (int64_t v = 0; v < nv; v++) { px[v] = pxy[2 * v]; py[v] = pxy[2 * v + 1]; }
    DPG_TRY(dpg_bumpy_set_box(h, box[0], box[1]));
    DPG_TRY(dpg_bumpy_set_bodies(h, x.data(), y.data(), ang.data(), vx.data(), vy.data(), om.data(),
                                 r.data(), nvb.data()));
    DPG_TRY(dpg_bumpy_set_vertices(h, px.data(), py.data()));
    if (!f_vm) {  // kernelGetVertexMasses: the body mass shared by its vertices
        vm.resize(nv);
        int64_t v = 0;
        for (int64_t b = 0; b < nb; b++)
            for (int32_t k = 0; k < nvb[b]; k++) vm[v++] = m[b] / (double)nvb[b];
    }
    if (!f_I) {
        // kernelGetMomentsOfInertia (kernels.cu:1171-1189): vertex mass times the
        // squared distance from the centre, summed in vertex order
        I.assign(nb, 0.0);
        int64_t v = 0;
        for (int64_t b = 0; b < nb; b++)
            for (int32_t k = 0; k < nvb[b]; k++, v++) {
                double rx = px[v] - x[b], ry = py[v] - y[b];
                I[b] += vm[v] * (rx * rx + ry * ry);
            }
    }
    return dpg_bumpy_set_inertia(h, m.data(), I.data(), vm.data());
}
