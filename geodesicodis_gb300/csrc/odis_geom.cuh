// Spherical geometry of the mesh builder, shared by the host builder
// (odis_mesh.cpp) and the device builder (odis_mesh_dev.cu).
//
// The formulas follow the reference's evaluation order, because several are
// ill-conditioned at fine levels (acos-based arc lengths, spherical excess from
// acos angles) and the per-step kernels must see the coefficients GeodesicODIS
// builds to agree with it to 1e-10:
//   map factor / map coordinates ...... include/mathRoutines.h:29-68
//   arc lengths ....................... include/mathRoutines.h:134-163
//   spherical midpoint ................ include/mathRoutines.h:172-192
//   edge normal in map coordinates .... include/mathRoutines.h:214-248
//   great-circle intersection ......... include/mathRoutines.h:320-383
//   angle about a node ................ include/mathRoutines.h:385-410
//   spherical triangle area ........... include/mathRoutines.h:415-439
// Math calls are unqualified so that host code takes the C library's and
// device code CUDA's; squares the reference takes with pow(x, 2.0) stay pow on
// the host (bit-identical to the reference's build) and are x * x on the device.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define ODIS_HD __host__ __device__
#else
#define ODIS_HD
#endif

namespace odis {
namespace geo {

constexpr double kGeoPi = 3.1415926535897932384626433832795028841971693993751058;

struct LL { double lat, lon; };

ODIS_HD inline double pow2(double x)
{
#ifdef __CUDA_ARCH__
    return x * x;
#else
    return std::pow(x, 2.0);
#endif
}

ODIS_HD inline double mapfac(double lat1, double lat2, double lon1, double lon2)
{
    return 2.0 / (1.0 + sin(lat1) * sin(lat2) + cos(lat1) * cos(lat2) * cos(lon2 - lon1));
}

// stereographic coordinates of q in the plane tangent at c (radius r)
ODIS_HD inline void stereo(LL c, LL q, double r, double& m, double& x, double& y)
{
    m = mapfac(c.lat, q.lat, c.lon, q.lon);
    x = m * r * (cos(q.lat) * sin(q.lon - c.lon));
    y = m * r * (sin(q.lat) * cos(c.lat) - cos(q.lat) * sin(c.lat) * cos(q.lon - c.lon));
}

ODIS_HD inline double arc_acos(LL a, LL b, double r)
{
    return r * acos(sin(a.lat) * sin(b.lat) + cos(a.lat) * cos(b.lat) * cos(b.lon - a.lon));
}

ODIS_HD inline void to_xyz(LL a, double p[3])
{
    // sph2cart with colatitude pi/2 - lat, unit radius
    const double colat = kGeoPi * 0.5 - a.lat;
    p[0] = 1.0 * sin(colat) * cos(a.lon);
    p[1] = 1.0 * sin(colat) * sin(a.lon);
    p[2] = 1.0 * cos(colat);
}

ODIS_HD inline double arc_atan2(LL a, LL b)
{
    double p[3], q[3];
    to_xyz(a, p);
    to_xyz(b, q);
    double c = pow2(p[1] * q[2] - p[2] * q[1]);
    c += pow2(-(p[0] * q[2] - p[2] * q[0]));
    c += pow2(p[0] * q[1] - p[1] * q[0]);
    c = sqrt(c);
    const double d = p[0] * q[0] + p[1] * q[1] + p[2] * q[2];
    return atan2(c, d);
}

ODIS_HD inline void latlon_xyz(LL a, double p[3])
{
    p[0] = cos(a.lat) * cos(a.lon);
    p[1] = cos(a.lat) * sin(a.lon);
    p[2] = sin(a.lat);
}

ODIS_HD inline LL midpoint(LL a, LL b)
{
    double p[3], q[3], c[3];
    latlon_xyz(a, p);
    latlon_xyz(b, q);
    for (int k = 0; k < 3; k++) c[k] = 0.5 * (p[k] + q[k]);
    return {atan2(c[2], sqrt(pow2(c[0]) + pow2(c[1]))), atan2(c[1], c[0])};
}

ODIS_HD inline void map_normal(LL a, LL b, double n[2])
{
    const LL c = midpoint(a, b);
    double m, x1, y1, x2, y2;
    stereo(c, a, 1.0, m, x1, y1);
    stereo(c, b, 1.0, m, x2, y2);
    double tx = x2 - x1, ty = y2 - y1;
    const double mag = sqrt(tx * tx + ty * ty);
    tx /= mag;
    ty /= mag;
    n[0] = -ty;
    n[1] = tx;
}

ODIS_HD inline LL intersect(LL a, LL b, LL c, LL d)
{
    double pa[3], pb[3], pc[3], pd[3], n1[3], n2[3], mp[3];
    latlon_xyz(a, pa); latlon_xyz(b, pb); latlon_xyz(c, pc); latlon_xyz(d, pd);
    n1[0] = pa[1] * pb[2] - pa[2] * pb[1];
    n1[1] = -(pa[0] * pb[2] - pa[2] * pb[0]);
    n1[2] = pa[0] * pb[1] - pa[1] * pb[0];
    n2[0] = pc[1] * pd[2] - pc[2] * pd[1];
    n2[1] = -(pc[0] * pd[2] - pc[2] * pd[0]);
    n2[2] = pc[0] * pd[1] - pc[1] * pd[0];
    double m1 = sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]);
    const double m2 = sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
    for (int k = 0; k < 3; k++) { n1[k] /= m1; n2[k] /= m2; }
    mp[0] = n1[1] * n2[2] - n2[1] * n1[2];
    mp[1] = n2[0] * n1[2] - n1[0] * n2[2];
    mp[2] = n1[0] * n2[1] - n2[0] * n1[1];
    m1 = sqrt(mp[0] * mp[0] + mp[1] * mp[1] + mp[2] * mp[2]);
    for (int k = 0; k < 3; k++) mp[k] /= m1;
    LL o{asin(mp[2] / 1.0), atan2(mp[1], mp[0])};
    if (o.lon < 0.0) o.lon += 2 * kGeoPi;
    return o;
}

// signed angle (rad) from q2 to q1 about c in c's stereographic plane
ODIS_HD inline double angle_about(LL q1, LL q2, LL c)
{
    double m, x1, y1, x2, y2;
    stereo(c, q1, 1.0, m, x1, y1);
    stereo(c, q2, 1.0, m, x2, y2);
    double a = atan2(y1 - 0.0, x1 - 0.0) - atan2(y2 - 0.0, x2 - 0.0);
    if (a > kGeoPi) a -= 2 * kGeoPi;
    else if (a < -kGeoPi) a += 2 * kGeoPi;
    return a;
}

ODIS_HD inline double sph_tri_area(LL p1, LL p2, LL p3, double r)
{
    const double c = fabs(acos(sin(p1.lat) * sin(p2.lat) + cos(p1.lat) * cos(p2.lat) * cos(fabs(p2.lon - p1.lon))));
    const double a = fabs(acos(sin(p2.lat) * sin(p3.lat) + cos(p2.lat) * cos(p3.lat) * cos(fabs(p3.lon - p2.lon))));
    const double b = fabs(acos(sin(p3.lat) * sin(p1.lat) + cos(p3.lat) * cos(p1.lat) * cos(fabs(p1.lon - p3.lon))));
    const double A = fabs(acos((cos(a) - cos(b) * cos(c)) / (sin(b) * sin(c))));
    const double B = fabs(acos((cos(b) - cos(a) * cos(c)) / (sin(a) * sin(c))));
    const double C = fabs(acos((cos(c) - cos(b) * cos(a)) / (sin(b) * sin(a))));
    return pow2(r) * fabs((A + B + C) - kGeoPi);
}

// an id (and its slot at the node) ranked by its angle (degrees) about a node
struct Ranked { int id; int slot; double deg; };

// the absolute angle of q in c's stereographic plane, as angle_about forms it
ODIS_HD inline double angle_in_plane(LL q, LL c)
{
    double m, x, y;
    stereo(c, q, 1.0, m, x, y);
    return atan2(y - 0.0, x - 0.0);
}

// angle_about(q1, q2, c) from the two absolute angles angle_in_plane(q1, c) and angle_in_plane(q2, c)
ODIS_HD inline double angle_between(double t1, double t2)
{
    double a = t1 - t2;
    if (a > kGeoPi) a -= 2 * kGeoPi;
    else if (a < -kGeoPi) a += 2 * kGeoPi;
    return a;
}

// descending insertion sort of k <= 6 entries (stable)
ODIS_HD inline void sort_desc(Ranked* r, int k)
{
    for (int a = 1; a < k; a++) {
        const Ranked x = r[a];
        int b = a - 1;
        while (b >= 0 && r[b].deg < x.deg) { r[b + 1] = r[b]; b--; }
        r[b + 1] = x;
    }
}

}  // namespace geo
}  // namespace odis
