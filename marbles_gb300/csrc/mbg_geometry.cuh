// mbg_geometry.cuh -- implicit functions of the embedded-boundary geometries
// (eb2.geom_type) and the cell classification behind the is_fluid flags,
// shared by the host driver (grid tagging) and the GPU flags kernel
// (mbg_geometry.cu).
//
// The reference builds these through AMReX EB2 (Source/EB.cpp:5-38: the
// built-in sphere, box, cylinder and plane; Source/Geometry.cpp:5-200: the
// project's own extruded triangles, rotated cylinder and rotated box).  AMReX
// is not part of the reference checkout, so its implicit functions are
// restated here from their definitions, with one convention throughout:
// phi >= 0 in the body (solid), phi < 0 in the fluid.
//   sphere    s (r^2 - |x - c|^2)
//   box       s min_d min(x_d - lo_d, hi_d - x_d)
//   cylinder  s min(r^2 - rho^2, (h/2)^2 - (x_a - c_a)^2), rho the distance
//             to the axis a through c; h <= 0 leaves the axis unbounded
//   plane     (x - p) . n                      (body on the normal's side)
// with s = -1 where the geometry has fluid inside.  Rotations turn the point
// back by the angle about the axis (through the rotation centre for the
// box, through the origin for the cylinder, as Geometry.cpp composes them).
// Extruded triangles: the body of a triangle is where all three edge planes
// (left normals of the anticlockwise edges) are >= 0, the union of the
// triangles is the maximum, extruded along z.
//
// A cell is covered (is_fluid = 0) when phi >= 0 at all 8 of its corners,
// otherwise fluid -- regular or cut cells count as fluid as in
// initialize_is_fluid (Source/LBM.cpp:1213-1262).
#pragma once

#include <cmath>

#include "../../include/marbles_gb300.h"

namespace mbg {

enum {
    GEOM_ALL_REGULAR = 0, GEOM_SPHERE = 1, GEOM_BOX = 2, GEOM_CYLINDER = 3, GEOM_PLANE = 4,
    GEOM_ROTATED_BOX = 5, GEOM_ROTATED_CYLINDER = 6, GEOM_EXTRUDED_TRIANGLES = 7
};

constexpr int GEOM_MAX_TRI = 5;

struct GeomDesc {
    int type = GEOM_ALL_REGULAR;
    int fluid_inside = 0;
    double center[3] = {0, 0, 0};
    double radius = 0.0;
    double height = -1.0;
    int direction = 0;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    double point[3] = {0, 0, 0}, normal[3] = {1, 0, 0};
    double rot_cos = 1.0, rot_sin = 0.0;   // of the rotation angle, taken on the host
    int rot_axis = 0;
    double rot_center[3] = {0, 0, 0};
    int ntri = 0;
    double tri[GEOM_MAX_TRI][3][2] = {};
};

// the point turned by -angle about `axis` through c (cs, sn: cos and sin
// of the angle, evaluated once on the host so that host and device agree)
__host__ __device__ inline void geom_unrotate(double cs, double sn, int axis, const double c[3], const double x[3],
                                              double out[3])
{
    double r[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
    const int i = (axis + 1) % 3, j = (axis + 2) % 3;
    const double u = r[i], v = r[j];
    r[i] = cs * u + sn * v;
    r[j] = -sn * u + cs * v;
    out[0] = r[0] + c[0];
    out[1] = r[1] + c[1];
    out[2] = r[2] + c[2];
}

__host__ __device__ inline double geom_box_phi(const GeomDesc& g, const double x[3])
{
    double m = x[0] - g.lo[0];
    for (int d = 0; d < 3; ++d) {
        const double a = x[d] - g.lo[d], b = g.hi[d] - x[d];
        m = a < m ? a : m;
        m = b < m ? b : m;
    }
    return g.fluid_inside ? -m : m;
}

__host__ __device__ inline double geom_cylinder_phi(const GeomDesc& g, const double x[3])
{
    const int a = g.direction;
    double rho2 = 0.0;
    for (int d = 0; d < 3; ++d)
        if (d != a) rho2 += (x[d] - g.center[d]) * (x[d] - g.center[d]);
    double m = g.radius * g.radius - rho2;
    if (g.height > 0.0) {
        const double t = x[a] - g.center[a];
        const double b = 0.25 * g.height * g.height - t * t;
        m = b < m ? b : m;
    }
    return g.fluid_inside ? -m : m;
}

__host__ __device__ inline double geom_phi(const GeomDesc& g, const double x[3])
{
    switch (g.type) {
    case GEOM_SPHERE: {
        const double ax = x[0] - g.center[0], ay = x[1] - g.center[1], az = x[2] - g.center[2];
        const double m = g.radius * g.radius - (ax * ax + ay * ay + az * az);
        return g.fluid_inside ? -m : m;
    }
    case GEOM_BOX:
        return geom_box_phi(g, x);
    case GEOM_CYLINDER:
        return geom_cylinder_phi(g, x);
    case GEOM_PLANE:
        return (x[0] - g.point[0]) * g.normal[0] + (x[1] - g.point[1]) * g.normal[1] +
               (x[2] - g.point[2]) * g.normal[2];
    case GEOM_ROTATED_BOX: {
        double y[3];
        geom_unrotate(g.rot_cos, g.rot_sin, g.rot_axis, g.rot_center, x, y);
        return geom_box_phi(g, y);
    }
    case GEOM_ROTATED_CYLINDER: {
        const double o[3] = {0.0, 0.0, 0.0};
        double y[3];
        geom_unrotate(g.rot_cos, g.rot_sin, g.rot_axis, o, x, y);
        return geom_cylinder_phi(g, y);
    }
    case GEOM_EXTRUDED_TRIANGLES: {
        double best = -1.0e300;
        for (int t = 0; t < g.ntri; ++t) {
            double m = 1.0e300;
            for (int e = 0; e < 3; ++e) {
                const double* p0 = g.tri[t][e];
                const double* p1 = g.tri[t][(e + 1) % 3];
                double nx = -(p1[1] - p0[1]), ny = p1[0] - p0[0];
                const double nrm = sqrt(nx * nx + ny * ny);
                nx = nx / nrm;
                ny = ny / nrm;
                const double v = (x[0] - p0[0]) * nx + (x[1] - p0[1]) * ny;
                m = v < m ? v : m;
            }
            best = m > best ? m : best;
        }
        return best;
    }
    default:
        return -1.0;
    }
}

// covered (all 8 corners in the body) for cell (i, j, k) of a level with
// lower corner plo and cell size dx
__host__ __device__ inline bool geom_covered(const GeomDesc& g, const double plo[3], const double dx[3], int i,
                                             int j, int k)
{
    if (g.type == GEOM_ALL_REGULAR) return false;
    for (int c = 0; c < 8; ++c) {
        const double x[3] = {plo[0] + (i + (c & 1)) * dx[0], plo[1] + (j + ((c >> 1) & 1)) * dx[1],
                             plo[2] + (k + ((c >> 2) & 1)) * dx[2]};
        if (!(geom_phi(g, x) >= 0.0)) return false;
    }
    return true;
}

// the implicit-function description of a C-ABI geometry (rotation angle in
// degrees turned into its cosine and sine on the host)
GeomDesc geom_from(const mbg_geometry& in);

}  // namespace mbg
