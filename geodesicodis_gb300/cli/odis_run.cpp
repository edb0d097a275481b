// odis_run: the GeodesicODIS run driver on libodis_gpu.so.
//
// Reads a run directory the way the reference's main (src/main.cpp) and
// ab3Explicit (src/timeIntegrator.cpp:57-322) do: input.in keys
// (src/globals.cpp:58-203), optional InitialConditions/{vel,pres}_init.txt
// (src/initialConditions.cpp:209-276) when "initial conditions" is LOAD.  It runs
// the time loop on the GPU, prints the reference's "DUMPING DATA AT ... AVG
// DISS: ... GW" line at every output interval (src/timeIntegrator.cpp:190-193)
// to stdout and OUTPUT.txt, and writes the final state back in the
// InitialConditions format.  DATA/power.txt gets one "orbit  W/m^2  GW" line
// per output interval, DATA/final_nodes.txt the final displacement and Cartesian
// velocity (RBF reconstruction) per node; the HDF5 field dumps (src/outFiles.cpp)
// are not written.
//
//   odis_run [--dir D] [--grid FILE | --level N] [--precision fp64|df64|fp32] [--orbits X]
//
// --level is the number of subdivisions (10*4^N+2 cells); without --grid or
// --level the grid is generated for input.in's "geodesic grid level", whose
// count the reference's grid files give as 10*4^(level-1)+2 cells.
#include "odis_gpu.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;

bool read_state(const std::string& path, int n, std::vector<double>& x, std::vector<double>& hist)
{
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    x.assign(n, 0.0);
    hist.assign((size_t)3 * n, 0.0);
    for (int i = 0; i < n; i++) {
        if (std::fscanf(f, " %lf , %lf , %lf , %lf", &x[i], &hist[3 * i], &hist[3 * i + 1], &hist[3 * i + 2]) != 4) {
            std::fclose(f);
            return false;
        }
    }
    std::fclose(f);
    return true;
}

bool write_state(const std::string& path, int n, const std::vector<double>& x, const std::vector<double>& hist)
{
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    for (int i = 0; i < n; i++)
        std::fprintf(f, "%1.6E, %1.6E, %1.6E, %1.6E\n", x[i], hist[3 * i], hist[3 * i + 1], hist[3 * i + 2]);
    std::fclose(f);
    return true;
}

int fail(const char* what, odis_status st)
{
    std::fprintf(stderr, "odis_run: %s failed (status %d)\n", what, st);
    return 2;
}

}  // namespace

int main(int argc, char** argv)
{
    std::string dir = ".", grid, prec = "fp64";
    int level = -1;
    double orbits = -1.0;
    for (int a = 1; a < argc; a++) {
        const std::string k = argv[a];
        auto next = [&]() -> std::string { return a + 1 < argc ? argv[++a] : std::string(); };
        if (k == "--dir") dir = next();
        else if (k == "--grid") grid = next();
        else if (k == "--level") level = std::atoi(next().c_str());
        else if (k == "--precision") prec = next();
        else if (k == "--orbits") orbits = std::atof(next().c_str());
        else {
            std::fprintf(stderr, "usage: odis_run [--dir D] [--grid FILE | --level N] [--precision fp64|df64|fp32] "
                                 "[--orbits X]\n");
            return 2;
        }
    }
    odis_input in;
    odis_status st = odis_params_from_input((dir + "/input.in").c_str(), &in);
    if (st != ODIS_OK) return fail("reading input.in", st);
    odis_params p = in.params;
    p.precision = prec == "fp32" ? ODIS_FP32 : prec == "df64" ? ODIS_DF64 : ODIS_FP64;
    if (p.advection && p.precision != ODIS_FP64) {
        std::fprintf(stderr, "odis_run: advection true runs the nonlinear equations in FP64\n");
        p.precision = ODIS_FP64;
    }
    odis_mesh* mesh = nullptr;
    if (!grid.empty()) st = odis_mesh_from_file(grid.c_str(), p.radius, &mesh);
    else st = odis_mesh_generate(level >= 0 ? level : in.grid_level - 1, p.radius, &mesh);
    if (st != ODIS_OK) return fail("building the mesh", st);
    int N = 0, E = 0;
    odis_mesh_sizes(mesh, &N, &E, nullptr);
    // the check the reference never makes: omega_max * dt <= 6/11
    double w = 0.0;
    int stable = 0;
    if (odis_mesh_gravity_wave_omega(mesh, p.g, p.h, 200, &w) == ODIS_OK &&
        odis_stable_steps_per_orbit(in.period, w, 1.0, &stable) == ODIS_OK && stable > in.steps_per_orbit)
        std::fprintf(stderr, "odis_run: warning: %d steps per orbit put the fastest gravity wave at omega*dt = %.3f, "
                             "beyond the 6/11 limit of the AB3 loop; at least %d are needed\n",
                     in.steps_per_orbit, w * in.period / in.steps_per_orbit, stable);
    odis_ctx* ctx = nullptr;
    st = odis_create(&p, mesh, &ctx);
    if (st != ODIS_OK) return fail("odis_create", st);
    std::vector<double> v, eta, dv, de;
    if (in.init_kind == 1) {
        if (!read_state(dir + "/InitialConditions/vel_init.txt", E, v, dv) ||
            !read_state(dir + "/InitialConditions/pres_init.txt", N, eta, de))
            return fail("reading InitialConditions", ODIS_ERR_IO);
        st = odis_set_state(ctx, 0, v.data(), eta.data(), dv.data(), de.data());
        if (st != ODIS_OK) return fail("odis_set_state", st);
    }
    const double total_orbits = orbits > 0 ? orbits : in.end_time;
    const int out_every = std::max(1, in.steps_per_orbit / std::max(1, in.output_time));
    const long long total_steps = (long long)std::llround(total_orbits * in.steps_per_orbit);
    mkdir((dir + "/DATA").c_str(), 0755);
    FILE* out = std::fopen((dir + "/OUTPUT.txt").c_str(), "a");
    FILE* pw = std::fopen((dir + "/DATA/power.txt").c_str(), "w");
    std::vector<double> power(out_every);
    const double area = 4.0 * kPi * p.radius * p.radius;
    int rc = 0, count = 1;
    for (long long done = 0; done < total_steps; done += out_every, count++) {
        const int n = (int)std::min<long long>(out_every, total_steps - done);
        st = odis_run_steps(ctx, n, power.data(), ODIS_MEM_HOST);
        double avg = 0.0;
        for (int k = 0; k < n; k++) avg += power[k];
        avg /= n;
        const double t_orb = (double)(done + n) / in.steps_per_orbit;
        char line[256];
        std::snprintf(line, sizeof line, "DUMPING DATA AT %f AVG DISS: %e GW%d", t_orb, power[n - 1] * area / 1e9, count);
        std::printf("%s\n", line);
        if (out) std::fprintf(out, "%s\n", line);
        if (pw) std::fprintf(pw, "%.9f %.12e %.12e\n", t_orb, avg, avg * area / 1e9);
        if (st == ODIS_ERR_NONFINITE) {
            std::printf("Terminating ODIS: the state became non-finite\n");
            rc = 1;
            break;
        }
        if (st != ODIS_OK) { rc = fail("odis_run_steps", st); break; }
    }
    if (out) std::fclose(out);
    if (pw) std::fclose(pw);
    int iter = 0;
    v.assign(E, 0.0); eta.assign(N, 0.0); dv.assign((size_t)3 * E, 0.0); de.assign((size_t)3 * N, 0.0);
    if (odis_get_state(ctx, &iter, v.data(), eta.data(), dv.data(), de.data()) == ODIS_OK) {
        mkdir((dir + "/InitialConditions").c_str(), 0755);
        write_state(dir + "/InitialConditions/vel_init.txt", E, v, dv);
        write_state(dir + "/InitialConditions/pres_init.txt", N, eta, de);
        // final displacement and Cartesian velocity at the nodes (the "displacement" and
        // "x/y/z velocity" fields of the reference's output)
        std::vector<double> uxyz((size_t)3 * N);
        if (odis_interpolate_cartesian(ctx, uxyz.data(), v.data(), ODIS_MEM_HOST) == ODIS_OK) {
            FILE* f = std::fopen((dir + "/DATA/final_nodes.txt").c_str(), "w");
            if (f) {
                for (int i = 0; i < N; i++)
                    std::fprintf(f, "%1.9E %1.9E %1.9E %1.9E\n", eta[i], uxyz[3 * i], uxyz[3 * i + 1], uxyz[3 * i + 2]);
                std::fclose(f);
            }
        }
    }
    odis_destroy(ctx);
    odis_mesh_destroy(mesh);
    return rc;
}
