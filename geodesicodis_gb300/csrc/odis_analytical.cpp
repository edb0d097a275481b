// Analytical initial conditions ("initial conditions ANALYTICAL" in input.in):
// the reference's analyticalInitialConditions (src/initialConditions.cpp:150-211)
// over its closed-form LTE solution analyticalLTE, case OBLIQ_WEST
// (src/analyticalLTE.cpp:22-44, 62-80, 133-181).  Host code, FP64.
//
// The solution keeps the stream-function coefficient Psi_11 and the velocity
// potential coefficient Phi_21 of the westward obliquity tide (degree 2,
// order 1, frequency -Omega):
//   lam = w / (2 Omega), w = -Omega;  lambs = 4 Omega^2 r^2 / (g h)
//   L_1 = lam + 1/2 + i alpha / (2 Omega)
//   K_2 = lam + 1/6 - 6 / (lambs lam) + i alpha / (2 Omega)
//   Psi_11 = (Omega r^2 obl / 4) / (q_1(1) - K_2 L_1 / p_2(1)),  Phi_21 = -i L_1 / p_2(1) Psi_11
// with p_n(m) = (n+1)(n+m) / (n(2n+1)) and q_n(m) = n(n+1-m) / ((n+1)(2n+1)).
// The east and north velocities are the stream function's and the potential's
// gradients in spherical coordinates; eta follows from continuity.  Without drag
// this solves the continuous equations exactly (Phi_21 = 0); with drag the
// closed form leaves out the coupling to Psi_31, as the reference does.
#include "../../include/odis_gpu.h"
#include "odis_internal.h"

#include <cmath>
#include <complex>

namespace {

using cplx = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;

double pn(double n, double m) { return (n + 1) * (n + m) / (n * (2 * n + 1)); }
double qn(double n, double m) { return n * (n + 1 - m) / ((n + 1) * (2 * n + 1)); }

struct Westward {
    cplx psi, phi;
    double w, r, h;

    Westward(const odis_params& p)
    {
        const cplx I(0.0, 1.0);
        w = -p.angvel;
        r = p.radius;
        h = p.h;
        const double lam = w / (2 * p.angvel);
        const double lambs = 4 * p.angvel * p.angvel * p.radius * p.radius / (p.g * p.h);
        const cplx damp = I * (p.alpha / (2 * p.angvel));
        const cplx L1 = lam + 1.0 / 2.0 + damp;
        const cplx K2 = lam + 1.0 / 6.0 - 6.0 / (lambs * lam) + damp;
        const double U21 = 0.5 * p.angvel * p.angvel * p.radius * p.radius * p.obliq;
        psi = U21 / (2 * p.angvel) / (qn(1, 1) - K2 * L1 / pn(2, 1));
        phi = -I * L1 / pn(2, 1) * psi;
    }

    // (u_east, v_north) and their time derivatives at (lat, lon), time t
    void velocity(double lat, double lon, double t, double out[4]) const
    {
        const cplx I(0.0, 1.0);
        const double th = kPi * 0.5 - lat, st = std::sin(th), ct = std::cos(th);
        const cplx e = std::exp(I * lon), ph = std::exp(-I * w * t);
        const cplx Y11 = st * e, Y21 = 3 * ct * st * e, Y31 = 1.5 * (5 * ct * ct - 1) * st * e;
        const cplx U = (-1.0 / 3.0 * psi * Y21 + I * phi * Y21) * ph;
        const cplx V = -(I * psi * Y11 + phi * (4.0 * Y31 - 9.0 * Y11) / 5.0) * ph;
        const double den = r * st;
        out[0] = U.real() / den;
        out[1] = V.real() / den;
        out[2] = (-I * w * U).real() / den;
        out[3] = (-I * w * V).real() / den;
    }

    // (eta, deta/dt) at (lat, lon), time t
    void height(double lat, double lon, double t, double out[2]) const
    {
        const cplx I(0.0, 1.0);
        const double th = kPi * 0.5 - lat, st = std::sin(th), ct = std::cos(th);
        const cplx Y21 = 3 * ct * st * std::exp(I * lon);
        const cplx E = I * 6.0 / (r * r) * h / w * phi * Y21 * std::exp(-I * w * t);
        out[0] = E.real();
        out[1] = (-I * w * E).real();
    }
};

}  // namespace

extern "C" odis_status odis_analytical_state(const odis_params* p, const odis_mesh* mesh, double t, double* v,
                                             double* eta, double* dvdt, double* detadt)
{
    if (!p || !mesh || p->potential != ODIS_POT_OBLIQ_WEST || !(p->angvel > 0) || !(p->g > 0) || !(p->h > 0) ||
        !(p->radius > 0))
        return ODIS_ERR_ARG;
    const odis::Mesh& m = mesh->m;
    const Westward sol(*p);
    for (int e = 0; e < m.E; e++) {
        const double lat = m.face_centre[(size_t)e * 2], lon = m.face_centre[(size_t)e * 2 + 1];
        const double nx = m.face_normal[(size_t)e * 2], ny = m.face_normal[(size_t)e * 2 + 1];
        for (int k = 0; k < 3; k++) {
            double a[4];
            sol.velocity(lat, lon, t - k * p->dt, a);
            if (k == 0 && v) v[e] = a[0] * nx + a[1] * ny;
            if (dvdt) dvdt[(size_t)e * 3 + k] = a[2] * nx + a[3] * ny;
        }
    }
    for (int i = 0; i < m.N; i++) {
        const double lat = m.node_sph[(size_t)i * 2], lon = m.node_sph[(size_t)i * 2 + 1];
        for (int k = 0; k < 3; k++) {
            double a[2];
            sol.height(lat, lon, t - k * p->dt, a);
            if (k == 0 && eta) eta[i] = a[0];
            if (detadt) detadt[(size_t)i * 3 + k] = a[1];
        }
    }
    return ODIS_OK;
}
