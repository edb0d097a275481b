// odis_run: the GeodesicODIS run driver on libodis_gpu.so.
//
// Reads a run directory the way the reference's main (src/main.cpp) and
// ab3Explicit (src/timeIntegrator.cpp:57-322) do: input.in keys
// (src/globals.cpp:58-203), optional InitialConditions/{vel,pres}_init.txt
// (src/initialConditions.cpp:209-276) when "initial conditions" is LOAD, or the
// closed-form OBLIQ_WEST state when it is ANALYTICAL.  It runs
// the time loop on the GPU, prints the reference's "DUMPING DATA AT ... AVG
// DISS: ... GW" line at every output interval (src/timeIntegrator.cpp:190-193)
// to stdout and OUTPUT.txt, and writes the final state back in the
// InitialConditions format.  DATA/power.txt gets one "orbit  W/m^2  GW" line
// per output interval, DATA/final_nodes.txt the final displacement and Cartesian
// velocity (RBF reconstruction) per node.  DATA/data.h5 holds the reference's
// field dumps (OutFiles::CreateHDF5Framework, DumpGridData, DumpData,
// src/outFiles.cpp:138-823): float32 datasets [dumps][faces or nodes], one row
// per dump, for the outputs input.in switches on.
//
// SIGINT, as in the reference (CatchExit and the loop's flag check,
// src/timeIntegrator.cpp:32-37, 120, 307-316): the handler prints "Caught
// Terminate Signal...", the loop stops after the step chunk in flight (at most
// kCheckSteps steps), writes "Terminate signal caught..." to OUTPUT.txt, saves
// the state and exits with status 1.  Besides the reference's %1.6E text files
// (rounded to 7 digits), the state is saved exactly as
// InitialConditions/state.bin (FP64, with the step count); --resume continues
// from it to the same bits as an uninterrupted run.
//
//   odis_run [--dir D] [--grid FILE | --level N] [--precision fp64|df64|fp32] [--orbits X] [--resume]
//            [--device-mesh]
//
// --level is the number of subdivisions (10*4^N+2 cells); without --grid or
// --level the grid is generated for input.in's "geodesic grid level", whose
// count the reference's grid files give as 10*4^(level-1)+2 cells.
// --device-mesh generates the grid and builds the mesh geometry and TRiSK
// weights on the GPU (the same integers; the geometry to the conditioning of
// the reference's formulas), which is faster at fine levels.
#include "odis_gpu.h"

#include <csignal>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int kCheckSteps = 512;      // steps between two looks at the terminate flag

volatile std::sig_atomic_t g_terminate = 0;

extern "C" void catch_exit(int)
{
    static const char msg[] = "Caught Terminate Signal...\n";
    ssize_t w = write(STDOUT_FILENO, msg, sizeof msg - 1);
    (void)w;
    g_terminate = 1;
}

// Exact checkpoint: "ODISCKP1", int64 steps taken, int32 faces, int32 cells,
// then v[E], eta[N], dvdt[E][3], detadt[N][3] as little-endian FP64.
bool write_checkpoint(const std::string& path, long long iter, int E, int N, const std::vector<double>& v,
                      const std::vector<double>& eta, const std::vector<double>& dv, const std::vector<double>& de)
{
    const std::string tmp = path + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    const int64_t it = iter;
    const int32_t e = E, n = N;
    bool ok = std::fwrite("ODISCKP1", 1, 8, f) == 8 && std::fwrite(&it, 8, 1, f) == 1 && std::fwrite(&e, 4, 1, f) == 1 &&
              std::fwrite(&n, 4, 1, f) == 1 && std::fwrite(v.data(), 8, E, f) == (size_t)E &&
              std::fwrite(eta.data(), 8, N, f) == (size_t)N && std::fwrite(dv.data(), 8, (size_t)3 * E, f) == (size_t)3 * E &&
              std::fwrite(de.data(), 8, (size_t)3 * N, f) == (size_t)3 * N;
    ok = std::fclose(f) == 0 && ok;
    return ok && std::rename(tmp.c_str(), path.c_str()) == 0;      // a reader never sees half a file
}

bool read_checkpoint(const std::string& path, long long* iter, int E, int N, std::vector<double>& v,
                     std::vector<double>& eta, std::vector<double>& dv, std::vector<double>& de)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    char magic[8];
    int64_t it = 0;
    int32_t e = 0, n = 0;
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "ODISCKP1", 8) == 0 && std::fread(&it, 8, 1, f) == 1 &&
              std::fread(&e, 4, 1, f) == 1 && std::fread(&n, 4, 1, f) == 1 && e == E && n == N && it >= 0;
    if (ok) {
        v.resize(E); eta.resize(N); dv.resize((size_t)3 * E); de.resize((size_t)3 * N);
        ok = std::fread(v.data(), 8, E, f) == (size_t)E && std::fread(eta.data(), 8, N, f) == (size_t)N &&
             std::fread(dv.data(), 8, (size_t)3 * E, f) == (size_t)3 * E &&
             std::fread(de.data(), 8, (size_t)3 * N, f) == (size_t)3 * N;
    }
    std::fclose(f);
    *iter = it;
    return ok;
}

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

// DATA/data.h5 in the reference's layout.  Datasets, in CreateHDF5Framework's
// order (src/outFiles.cpp:222-333) and DumpGridData's (:463-521); the dump at
// time level t writes row t-1 (DumpData, :523-823).
struct DataFile {
    enum { kEast, kNorth, kX, kY, kZ, kDisp, kDiss, kDissAvg, kTime, kDummy1, kCount };
    odis_h5* h = nullptr;
    int index[kCount];
    int N = 0, E = 0;

    odis_status open(const std::string& path, int flags, long long T, int n_cells, int n_faces, const odis_mesh* mesh)
    {
        N = n_cells;
        E = n_faces;
        std::vector<const char*> names;
        std::vector<int> ranks;
        std::vector<long long> dims;
        for (int& i : index) i = -1;
        auto add = [&](int id, const char* name, long long rows, long long cols) {
            if (id >= 0) index[id] = (int)names.size();
            names.push_back(name);
            ranks.push_back(cols ? 2 : 1);
            dims.push_back(rows);
            dims.push_back(cols);
        };
        if (flags & 1) { add(kEast, "east velocity", T, E); add(kNorth, "north velocity", T, E); }
        if (flags & 2) { add(kX, "x velocity", T, N); add(kY, "y velocity", T, N); add(kZ, "z velocity", T, N); }
        if (flags & 4) add(kDisp, "displacement", T, N);
        if (flags & 8) add(kDiss, "dissipated energy", T, E);
        if (flags & 16) add(kDissAvg, "dissipation avg output", T, 0);
        if (flags & 32) add(kTime, "kinetic avg output", T, 0);
        if (flags & 64) add(kDummy1, "dummy1 output", T, N);
        add(-1, "face longitude", E, 0);
        add(-1, "face latitude", E, 0);
        odis_status st = odis_h5_create(path.c_str(), (int)names.size(), names.data(), ranks.data(), dims.data(), &h);
        if (st != ODIS_OK) return st;
        // face centres in degrees: (float) of the angle, times 180/pi, to float (src/outFiles.cpp:491-492)
        std::vector<double> lat(E), lon(E);
        std::vector<float> out(E);
        if ((st = odis_mesh_field(mesh, 4, lat.data())) != ODIS_OK || (st = odis_mesh_field(mesh, 5, lon.data())) != ODIS_OK)
            return st;
        for (int i = 0; i < E; i++) out[i] = (float)((double)(float)lon[i] * 180. / kPi);
        if ((st = odis_h5_write_rows(h, (int)names.size() - 2, 0, E, out.data())) != ODIS_OK) return st;
        for (int i = 0; i < E; i++) out[i] = (float)((double)(float)lat[i] * 180. / kPi);
        return odis_h5_write_rows(h, (int)names.size() - 1, 0, E, out.data());
    }

    bool wants(int id) const { return h && index[id] >= 0; }

    odis_status row(int id, long long t, const double* x, int n, int stride)
    {
        if (!wants(id)) return ODIS_OK;
        std::vector<float> r(n);
        for (int i = 0; i < n; i++) r[i] = (float)x[(size_t)i * stride];
        return odis_h5_write_rows(h, index[id], t, 1, r.data());
    }

    // one dump: the state's face velocities (east, north), Cartesian node velocity,
    // displacement, per-face dissipation, mean dissipation, time, and cv_mass
    // (computed by the reference before the initial conditions load, so zero)
    odis_status dump(odis_ctx* ctx, long long t, double time)
    {
        if (!h) return ODIS_OK;
        std::vector<double> v(E), eta(N), uv((size_t)2 * E), e(E), uxyz((size_t)3 * N, 0.0), zero(N, 0.0);
        int iter = 0;
        odis_status st = odis_get_state(ctx, &iter, v.data(), eta.data(), nullptr, nullptr);
        if (st == ODIS_OK) st = odis_interpolate_velocity(ctx, uv.data(), v.data(), ODIS_MEM_HOST);
        double avg = 0.0;
        if (st == ODIS_OK) st = odis_update_energy(ctx, &avg, e.data(), uv.data(), ODIS_MEM_HOST);
        if (st == ODIS_OK && wants(kX)) st = odis_interpolate_cartesian(ctx, uxyz.data(), v.data(), ODIS_MEM_HOST);
        if (st == ODIS_OK) st = row(kEast, t, uv.data(), E, 2);
        if (st == ODIS_OK) st = row(kNorth, t, uv.data() + 1, E, 2);
        if (st == ODIS_OK) st = row(kX, t, uxyz.data(), N, 3);
        if (st == ODIS_OK) st = row(kY, t, uxyz.data() + 1, N, 3);
        if (st == ODIS_OK) st = row(kZ, t, uxyz.data() + 2, N, 3);
        if (st == ODIS_OK) st = row(kDisp, t, eta.data(), N, 1);
        if (st == ODIS_OK) st = row(kDiss, t, e.data(), E, 1);
        if (st == ODIS_OK) st = row(kDissAvg, t, &avg, 1, 1);
        if (st == ODIS_OK) st = row(kTime, t, &time, 1, 1);
        if (st == ODIS_OK) st = row(kDummy1, t, zero.data(), N, 1);
        return st;
    }

    odis_status close()
    {
        odis_status st = h ? odis_h5_close(h) : ODIS_OK;
        h = nullptr;
        return st;
    }
};

}  // namespace

int main(int argc, char** argv)
{
    std::string dir = ".", grid, prec = "fp64";
    int level = -1;
    double orbits = -1.0;
    bool resume = false, device_mesh = false;
    for (int a = 1; a < argc; a++) {
        const std::string k = argv[a];
        auto next = [&]() -> std::string { return a + 1 < argc ? argv[++a] : std::string(); };
        if (k == "--dir") dir = next();
        else if (k == "--grid") grid = next();
        else if (k == "--level") level = std::atoi(next().c_str());
        else if (k == "--precision") prec = next();
        else if (k == "--orbits") orbits = std::atof(next().c_str());
        else if (k == "--resume") resume = true;
        else if (k == "--device-mesh") device_mesh = true;
        else {
            std::fprintf(stderr, "usage: odis_run [--dir D] [--grid FILE | --level N] [--precision fp64|df64|fp32] "
                                 "[--orbits X] [--resume] [--device-mesh]\n");
            return 2;
        }
    }
    odis_input in;
    odis_status st = odis_params_from_input((dir + "/input.in").c_str(), &in);
    if (st != ODIS_OK) return fail("reading input.in", st);
    odis_params p = in.params;
    p.precision = prec == "fp32" ? ODIS_FP32 : prec == "df64" ? ODIS_DF64 : ODIS_FP64;
    if (p.advection && p.precision == ODIS_FP32) {
        std::fprintf(stderr, "odis_run: advection true runs the nonlinear equations in FP64 or df64; using fp64\n");
        p.precision = ODIS_FP64;
    }
    odis_mesh* mesh = nullptr;
    const int gen_level = level >= 0 ? level : in.grid_level - 1;
    if (!grid.empty())
        st = device_mesh ? odis_mesh_from_file_device(grid.c_str(), p.radius, &mesh)
                         : odis_mesh_from_file(grid.c_str(), p.radius, &mesh);
    else
        st = device_mesh ? odis_mesh_generate_device(gen_level, p.radius, &mesh)
                         : odis_mesh_generate(gen_level, p.radius, &mesh);
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
    long long start = 0;          // steps already taken (--resume)
    if (resume) {
        if (!read_checkpoint(dir + "/InitialConditions/state.bin", &start, E, N, v, eta, dv, de))
            return fail("reading InitialConditions/state.bin", ODIS_ERR_IO);
        st = odis_set_state(ctx, (int)start, v.data(), eta.data(), dv.data(), de.data());
        if (st != ODIS_OK) return fail("odis_set_state", st);
    } else if (in.init_kind == 1) {
        if (!read_state(dir + "/InitialConditions/vel_init.txt", E, v, dv) ||
            !read_state(dir + "/InitialConditions/pres_init.txt", N, eta, de))
            return fail("reading InitialConditions", ODIS_ERR_IO);
        st = odis_set_state(ctx, 0, v.data(), eta.data(), dv.data(), de.data());
        if (st != ODIS_OK) return fail("odis_set_state", st);
    } else if (in.init_kind == 2) {
        // analyticalInitialConditions at t = 0 (src/initialConditions.cpp:150-211); the AB3
        // loop still starts with its two Euler steps, as for NONE
        v.assign(E, 0.0); eta.assign(N, 0.0); dv.assign((size_t)3 * E, 0.0); de.assign((size_t)3 * N, 0.0);
        st = odis_analytical_state(&p, mesh, 0.0, v.data(), eta.data(), dv.data(), de.data());
        if (st != ODIS_OK) return fail("initial conditions ANALYTICAL (potential OBLIQ_WEST only)", st);
        st = odis_set_state(ctx, 0, v.data(), eta.data(), dv.data(), de.data());
        if (st != ODIS_OK) return fail("odis_set_state", st);
    }
    const double total_orbits = orbits > 0 ? orbits : in.end_time;
    const int out_every = std::max(1, in.steps_per_orbit / std::max(1, in.output_time));
    const long long total_steps = (long long)std::llround(total_orbits * in.steps_per_orbit);
    std::signal(SIGINT, catch_exit);
    mkdir((dir + "/DATA").c_str(), 0755);
    FILE* out = std::fopen((dir + "/OUTPUT.txt").c_str(), "a");
    FILE* pw = std::fopen((dir + "/DATA/power.txt").c_str(), "w");
    std::vector<double> power(out_every);
    const double area = 4.0 * kPi * p.radius * p.radius;
    // DATA/data.h5: the initial dump and one per output interval
    DataFile data;
    const long long dumps = 1 + (total_steps + out_every - 1) / out_every;
    st = data.open(dir + "/DATA/data.h5", in.out_flags, dumps, N, E, mesh);
    if (st != ODIS_OK) return fail("creating DATA/data.h5", st);
    {   // the dump before the loop (src/timeIntegrator.cpp:186-196)
        std::vector<double> v0(E), uv0((size_t)2 * E);
        double avg0 = 0.0;
        st = odis_get_state(ctx, nullptr, v0.data(), nullptr, nullptr, nullptr);
        if (st == ODIS_OK) st = odis_interpolate_velocity(ctx, uv0.data(), v0.data(), ODIS_MEM_HOST);
        if (st == ODIS_OK) st = odis_update_energy(ctx, &avg0, nullptr, uv0.data(), ODIS_MEM_HOST);
        if (st == ODIS_OK) st = data.dump(ctx, 0, 0.0);
        if (st != ODIS_OK) return fail("the initial dump", st);
        char line[256];
        std::snprintf(line, sizeof line, "DUMPING DATA AT %f AVG DISS: %e GW%d", 0.0, avg0 * area / 1e9, 1);
        std::printf("%s\n", line);
        if (out) std::fprintf(out, "%s\n", line);
    }
    int rc = 0, count = 2 + (int)(start / out_every);
    bool terminated = false;
    // output intervals end where the step count is a multiple of out_every (the reference's
    // iter % out_freq == 0), also after a resume from a mid-interval checkpoint
    for (long long done = start, n = 0; done < total_steps; done += n, count++) {
        n = std::min<long long>(out_every - done % out_every, total_steps - done);
        int ran = 0;
        for (st = ODIS_OK; ran < n && st == ODIS_OK && !g_terminate; ran += (int)std::min<long long>(kCheckSteps, n - ran))
            st = odis_run_steps(ctx, (int)std::min<long long>(kCheckSteps, n - ran), power.data() + ran, ODIS_MEM_HOST);
        if (g_terminate && ran < n) {          // stopped inside the output interval: no dump for it
            terminated = true;
            break;
        }
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
        st = data.dump(ctx, count - 1, p.dt * (double)(done + n));
        if (st != ODIS_OK) { rc = fail("writing DATA/data.h5", st); break; }
        if (g_terminate) { terminated = true; break; }
    }
    if (terminated) {                         // src/timeIntegrator.cpp:307-316
        std::printf("Terminate signal caught...\n");
        if (out) std::fprintf(out, "Terminate signal caught...\n");
        rc = 1;
    }
    if (data.close() != ODIS_OK && rc == 0) rc = fail("closing DATA/data.h5", ODIS_ERR_IO);
    if (out) std::fclose(out);
    if (pw) std::fclose(pw);
    int iter = 0;
    v.assign(E, 0.0); eta.assign(N, 0.0); dv.assign((size_t)3 * E, 0.0); de.assign((size_t)3 * N, 0.0);
    if (odis_get_state(ctx, &iter, v.data(), eta.data(), dv.data(), de.data()) == ODIS_OK) {
        mkdir((dir + "/InitialConditions").c_str(), 0755);
        write_state(dir + "/InitialConditions/vel_init.txt", E, v, dv);
        write_state(dir + "/InitialConditions/pres_init.txt", N, eta, de);
        if (!write_checkpoint(dir + "/InitialConditions/state.bin", iter, E, N, v, eta, dv, de) && rc == 0)
            rc = fail("writing InitialConditions/state.bin", ODIS_ERR_IO);
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
