// input.in reader with the reference's semantics (src/globals.cpp:35-477):
//   * each record is `key; value; comment;` (the comment column is skipped),
//   * keys are matched case-insensitively after leading whitespace is dropped,
//   * unknown keys are skipped, missing keys keep the reference's defaults
//     (src/globals.cpp:479-571),
//   * obliquity is read in degrees and converted to radians (:424),
//   * the orbital period is recomputed from the angular velocity and rounded
//     to an even number of seconds, angvel = 2 pi / period (:209-214),
//   * `time step` is a target: dt = P/n with n the first multiple of 100 such
//     that P/n <= target, and totalIter = n (src/mesh.cpp:1566-1621),
//   * FREE surface sets love reduction = 1 + k2 - h2
//     (src/boundaryConditions.cpp:18-25).
#include "odis_internal.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

namespace odis {

namespace {
constexpr double kPi = 3.1415926535897932384626433832795028841971693993751058;

void copy_str(char* dst, const std::string& s)
{
    std::strncpy(dst, s.c_str(), 31);
    dst[31] = 0;
}
}  // namespace

int parse_input(const char* path, odis_input& out)
{
    std::ifstream in(path);
    if (!in.is_open()) return ODIS_ERR_IO;

    // defaults, src/globals.cpp:479-571
    double radius = 2574.73e3, k2 = .120, h2 = .2, love = 0.920012, h = 400, g = 1.35;
    double e = 0.0288, theta_default = 0.32 * kPi / 180., alpha = 2.28e-7;
    double dt_target = 40., angvel = 4.56e-6, end_time = 80., semimajor = 1221.87e6;
    int lmax = 10, level = 1, output_time = 1, fourier_freq = 0;
    bool advection = false, diss_avg = true, kinetic_avg = false;
    bool out_disp = false, out_vel = false, out_cart = false, out_diss = false, out_dummy1 = false;
    std::string potential = "ECC", friction = "QUADRATIC", surface = "FREE", solver = "AB3", init = "NONE";
    bool theta_given = false;
    double theta_read = 0.0;

    std::string key, val, comment;
    while (std::getline(in >> std::ws, key, ';')) {
        std::transform(key.begin(), key.end(), key.begin(), ::tolower);
        std::getline(in >> std::ws, val, ';');
        std::stringstream vs(val);
        auto rd = [&](double& d) { vs >> d; };
        auto ri = [&](int& i) { vs >> i; };
        auto rb = [&](bool& b) { std::string s; vs >> s; if (s == "false") b = false; else if (s == "true") b = true; };
        auto rs = [&](std::string& s) { vs >> s; };
        if (key == "radius") rd(radius);
        else if (key == "angular velocity") rd(angvel);
        else if (key == "k2") rd(k2);
        else if (key == "h2") rd(h2);
        else if (key == "love reduction factor") rd(love);
        else if (key == "ocean thickness") rd(h);
        else if (key == "surface gravity") rd(g);
        else if (key == "eccentricity") rd(e);
        else if (key == "semimajor axis") rd(semimajor);
        else if (key == "fourier freq") ri(fourier_freq);
        else if (key == "obliquity") { rd(theta_read); theta_given = true; }
        else if (key == "time step") rd(dt_target);
        else if (key == "friction coefficient") rd(alpha);
        else if (key == "sh degree") ri(lmax);
        else if (key == "geodesic grid level") ri(level);
        else if (key == "advection") rb(advection);
        else if (key == "simulation end time") rd(end_time);
        else if (key == "potential") rs(potential);
        else if (key == "friction type") rs(friction);
        else if (key == "surface type") rs(surface);
        else if (key == "solver type") rs(solver);
        else if (key == "initial conditions") rs(init);
        else if (key == "dissipation avg output") rb(diss_avg);
        else if (key == "kinetic avg output") rb(kinetic_avg);
        else if (key == "displacement output") rb(out_disp);
        else if (key == "velocity output") rb(out_vel);
        else if (key == "velocity cartesian output") rb(out_cart);
        else if (key == "dissipation output") rb(out_diss);
        else if (key == "dummy1 output") rb(out_dummy1);
        else if (key == "output time") ri(output_time);
        std::getline(in, comment, ';');
    }
    // obliquity: degrees -> radians (the default is already in radians and is
    // converted again, exactly as the reference does at :424)
    double theta = (theta_given ? theta_read : theta_default) * kPi / 180.;

    odis_params& p = out.params;
    std::memset(&out, 0, sizeof(out));
    double P = 0.0, dt = 0.0;
    int n = 0;
    odis_derive_time(angvel, dt_target, &p.angvel, &P, &dt, &n);
    p.radius = radius;
    p.g = g;
    p.h = h;
    p.alpha = alpha;
    p.ecc = e;
    p.obliq = theta;
    p.love_reduct = (surface == "FREE") ? 1.0 + k2 - h2 : love;
    p.dt = dt;
    // the reference's name -> tide_type mapping (src/globals.cpp:250-266)
    static const char* const kPotNames[] = {"OBLIQ", "OBLIQ_WEST", "OBLIQ_EAST", "ECC_RAD", "ECC_LIB", "ECC",
                                            "ECC_WEST", "ECC_EAST", "FULL", "FULL2", "TOTAL", "ECC_W3",
                                            "OBLIQ_W3", "PLANET", "PLANET_OBL", "GENERAL", "NONE"};
    p.potential = -1;
    for (int k = 0; k <= ODIS_POT_NONE; k++)
        if (potential == kPotNames[k]) p.potential = k;
    p.semimajor_axis = semimajor;
    p.fourier_freq = fourier_freq;
    p.init_load = init == "LOAD" ? 1 : 0;
    p.precision = ODIS_FP64;
    p.sh_lmax = 0;
    p.sh_factors = nullptr;
    out.period = P;
    out.end_time = end_time;
    out.steps_per_orbit = n;
    out.grid_level = level;
    out.output_time = output_time;
    out.sh_degree = lmax;
    out.advection = advection ? 1 : 0;
    p.advection = out.advection;
    out.fric_linear = friction == "LINEAR" ? 1 : 0;
    p.friction = out.fric_linear ? ODIS_FRIC_LINEAR : ODIS_FRIC_QUADRATIC;
    out.surface_free = surface == "FREE" ? 1 : 0;
    out.init_kind = init == "NONE" ? 0 : init == "LOAD" ? 1 : init == "ANALYTICAL" ? 2 : -1;
    out.out_flags = (out_vel ? 1 : 0) | (out_cart ? 2 : 0) | (out_disp ? 4 : 0) | (out_diss ? 8 : 0) |
                    (diss_avg ? 16 : 0) | (kinetic_avg ? 32 : 0) | (out_dummy1 ? 64 : 0);
    copy_str(out.potential_name, potential);
    copy_str(out.friction_name, friction);
    copy_str(out.surface_name, surface);
    copy_str(out.solver_name, solver);
    copy_str(out.init_name, init);
    // the reference terminates on unknown enum strings (src/globals.cpp:233-292)
    if (p.potential < 0 || out.init_kind < 0) return ODIS_ERR_ARG;
    if (!(friction == "LINEAR" || friction == "QUADRATIC")) return ODIS_ERR_ARG;
    if (!(solver == "EULER" || solver == "AB3" || solver == "RK4")) return ODIS_ERR_ARG;
    return ODIS_OK;
}

}  // namespace odis
