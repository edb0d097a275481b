// Tidal forcing potential of forcing() (src/tidalPotentials.cpp:29-334), split
// into its time-dependent scalars (ForcingTerms, one set per time t) and the
// per-node evaluation, so that the same code serves the per-operator call (terms
// from the host) and the fused time loop (terms per step from a device table).
#pragma once

#include "../../include/odis_gpu.h"

#include <cmath>

namespace odis {

// forcing types with a case in the reference's switch
__host__ __device__ inline bool pot_has_case(int t)
{
    return t == ODIS_POT_ECC || t == ODIS_POT_OBLIQ || t == ODIS_POT_OBLIQ_WEST || t == ODIS_POT_FULL ||
           t == ODIS_POT_FULL2 || t == ODIS_POT_PLANET || t == ODIS_POT_GENERAL;
}
__host__ __device__ inline bool pot_valid(int t) { return t >= ODIS_POT_OBLIQ && t <= ODIS_POT_NONE; }
// single-frequency potentials, U = cos(M) Ua + sin(M) Ub: folded through the
// gradient into two per-face coefficients at setup
__host__ __device__ inline bool pot_single_freq(int t)
{
    return t == ODIS_POT_ECC || t == ODIS_POT_OBLIQ || t == ODIS_POT_OBLIQ_WEST || t == ODIS_POT_FULL;
}
// potentials with several harmonics of M (FULL2) or another period (PLANET,
// GENERAL): evaluated at the nodes every step
__host__ __device__ inline bool pot_nodal(int t)
{
    return t == ODIS_POT_FULL2 || t == ODIS_POT_PLANET || t == ODIS_POT_GENERAL;
}

constexpr int kForcingTerms = 12;     // doubles per ForcingTerms

struct ForcingTerms {
    double cosM, sinM, cos2M, cos3M, cos4M;          // M = Omega t
    double pl_factor, pl_p, pl_cosphi, pl_sinphi;     // PLANET
    double ge_cos, ge_sin;                            // GENERAL
    double pad;
};
static_assert(sizeof(ForcingTerms) == kForcingTerms * sizeof(double), "ForcingTerms layout");

// node trig row: cosLat sinLat cosLon sinLon cos2Lat sin2Lat cos2Lon sin2Lon cos^2Lat sin^2Lat Pbar20 Pbar22
constexpr int kNodeTrig = 12;

struct ForcingConst {
    int type;
    double omega, radius, love, ecc, obl, semimajor, freq;
};

__host__ __device__ inline ForcingTerms forcing_terms(const ForcingConst& k, double t)
{
    ForcingTerms f{};
    const double omega = k.omega;
    f.cosM = cos(omega * t);
    f.sinM = sin(omega * t);
    f.cos2M = cos(2 * omega * t);
    f.cos3M = cos(3 * omega * t);
    f.cos4M = cos(4 * omega * t);
    if (k.type == ODIS_POT_PLANET) {            // src/tidalPotentials.cpp:178-212 (Io-like perturber)
        const double m2 = 8.931938e+22, a1 = 421800000.0, a2 = k.semimajor;
        const double n2 = omega, n1 = n2 * 2.0, nij = n1 - n2;
        const double cosnt = cos(nij * t), sinnt = sin(nij * t);
        f.pl_p = pow(a1, 2.0) + pow(a2, 2.0) - 2. * a1 * a2 * cosnt;
        f.pl_cosphi = (a1 - a2 * cosnt);
        f.pl_sinphi = a2 * sinnt;
        f.pl_factor = 0.5 * 6.67408e-11 * m2 * pow(k.radius / f.pl_p, 2.0) / sqrt(f.pl_p);
    }
    if (k.type == ODIS_POT_GENERAL) {           // :243-258
        const double n2 = omega, n1 = n2 * 2.0, nij = n1 - n2;
        f.ge_cos = cos(k.freq * nij * t);
        f.ge_sin = sin(k.freq * nij * t);
    }
    return f;
}

// U at one node, in the reference's evaluation order per case
__host__ __device__ inline double forcing_node(const ForcingConst& k, const ForcingTerms& f, const double* tr)
{
    const double cosLat = tr[0], sinLat = tr[1], cosLon = tr[2], sinLon = tr[3];
    const double cos2Lat = tr[4], sin2Lat = tr[5], cos2Lon = tr[6], sin2Lon = tr[7];
    const double cosSqLat = tr[8], sinSqLat = tr[9];
    const double lr = k.love, omega = k.omega, radius = k.radius, ecc = k.ecc, obl = k.obl;
    const double cosM = f.cosM, sinM = f.sinM, cos2M = f.cos2M;
    switch (k.type) {
    case ODIS_POT_ECC: {                        // :82-101
        const double factor = 0.75 * lr * pow(omega, 2.0) * pow(radius, 2.0) * ecc;
        return factor * ((1. - 3. * sinSqLat) * cosM + cosSqLat * (3. * cosM * cos2Lon + 4. * sinM * sin2Lon));
    }
    case ODIS_POT_OBLIQ: {                      // :104-116
        const double factor = -3. / 2. * lr * pow(omega, 2.0) * pow(radius, 2.0) * obl;
        return factor * cosM * sin2Lat * cosLon;
    }
    case ODIS_POT_OBLIQ_WEST: {                 // :118-131
        const double factor = 0.5 * lr * pow(omega, 2.0) * pow(radius, 2.0) * obl;
        return 3 * factor * sinLat * cosLat * (cosLon * cosM - sinLon * sinM);
    }
    case ODIS_POT_FULL: {                       // :158-174
        const double factor = 0.75 * lr * pow(omega, 2.0) * pow(radius, 2.0) * ecc;
        const double factor2 = -3. / 2. * lr * pow(omega, 2.0) * pow(radius, 2.0) * obl;
        return factor * ((1 - 3 * sinSqLat) * cosM + cosSqLat * (3 * cosM * cos2Lon + 4 * sinM * sin2Lon)) +
               factor2 * cosM * sin2Lat * cosLon;
    }
    case ODIS_POT_FULL2: {                      // :133-156
        const double factor = 1 / 32. * lr * pow(omega, 2.0) * pow(radius, 2.0);
        double T1 = 3. * ecc * (4. - 7. * obl * obl) * cosM + 6 * (obl * obl + ecc * ecc * (3 - 7 * obl * obl)) * cos2M;
        T1 += 3 * ecc * obl * obl * (7 * f.cos3M + 17 * ecc * f.cos4M);
        T1 *= -(1 - 3 * cos2Lat);
        double T2 = (4 + 15 * ecc * ecc + 20 * ecc * cosM + 43 * ecc * ecc * cos2M) * cosLon;
        T2 += 2 * ecc * (4 + 25 * ecc * cosM) * sinM * sinLon;
        T2 *= 24 * obl * cosLat * sinLat * sinM;
        double T3 = obl * obl * (2 + 3 * ecc * ecc + 6 * ecc * cosM + 9 * ecc * ecc * cos2M) * (cosM * cosLon + sinM * sinLon);
        T3 += -(obl * obl - 2) * ((6 * ecc * cosM + 17 * ecc * ecc * cos2M) * cos2Lon +
                                  2 * ecc * (4 + 17 * ecc * cosM) * sinM * sin2Lon);
        T3 *= 6 * cosSqLat;
        return factor * (T1 + T2 + T3);
    }
    case ODIS_POT_PLANET: {                     // :214-221
        const double cosgam = cosLat * (cosLon * f.pl_cosphi + sinLon * f.pl_sinphi);
        return f.pl_factor * (3. * pow(cosgam, 2.0) - f.pl_p);
    }
    case ODIS_POT_GENERAL: {                    // :250-268 with Pbar_20, Pbar_22 at the node
        const double a20 = -9.991062592506567e-05 * 2.0, a22 = 0.0012049514054640862 * 2.0;
        const double b22 = -0.0012017622891820471 * 2.0;
        const double U20 = (0.0 + a20 * f.ge_cos) * tr[10];
        const double U22a = (0.0 + a22 * f.ge_cos) * tr[11] * cos2Lon;
        const double U22b = (0.0 + b22 * f.ge_sin) * tr[11] * sin2Lon;
        return (U20 + U22a + U22b);
    }
    default:
        return 0.0;
    }
}

// per-operator forcing: U[i] for the node table trig[kNodeTrig][Np]
void launch_forcing(const double* trig, int N, int Np, double* U, const ForcingConst& k, const ForcingTerms& f,
                    cudaStream_t s);
// terms[k] = forcing_terms(dt * (first + k) + dt), k < n (the fused loop's forcing at t^{n+1})
void launch_forcing_terms(double* terms, const ForcingConst& k, long long first, int n, double dt, cudaStream_t s);
// usg[i] (method type: double, float or double-float) = (add ? usg[i] : 0) + U_i / g at the step
// `*iter + offset` of the run that started at `*run_first`, from the run's terms table
void launch_node_forcing(int precision, const double* trig, int N, int Np, void* usg, int add, double inv_g,
                         const ForcingConst& k, const double* terms, const long long* iter, const long long* run_first,
                         int offset, cudaStream_t s);

}  // namespace odis
