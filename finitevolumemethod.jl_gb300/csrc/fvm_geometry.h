// Per-triangle geometry and the Hilbert key, shared by the host mesh build (fvm_mesh.cpp,
// -ffp-contract=off) and the device ingest (fvm_mesh_dev.cu, -fmad=false): with no contraction
// and IEEE division and square root on both sides, the two round identically.
#pragma once
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define FVM_GEOM_HD __host__ __device__ __forceinline__
#else
#define FVM_GEOM_HD inline
#endif

namespace fvm {

// Geometry of triangle (i, j, k), in the operation order of src/geometry.jl:107-161:
// props[0..8] shape coefficients s, [9..14] dual-edge midpoints, [15..20] their unit normals,
// [21..23] their lengths; S[0..2] the triangle's share of each vertex's control volume.
FVM_GEOM_HD void triangle_geometry(const double* P, int32_t i, int32_t j, int32_t k, double* props, double S[3]) {
    const double px = P[2 * i], py = P[2 * i + 1];
    const double qx = P[2 * j], qy = P[2 * j + 1];
    const double rx = P[2 * k], ry = P[2 * k + 1];
    // DelaunayTriangulation statistics: centroid and edge midpoints
    const double cx = (px + qx + rx) / 3, cy = (py + qy + ry) / 3;
    const double m1x = (px + qx) / 2, m1y = (py + qy) / 2;
    const double m2x = (qx + rx) / 2, m2y = (qy + ry) / 2;
    const double m3x = (rx + px) / 2, m3y = (ry + py) / 2;
    const double pcx = cx - px, pcy = cy - py;
    const double qcx = cx - qx, qcy = cy - qy;
    const double rcx = cx - rx, rcy = cy - ry;
    const double m13x = m1x - m3x, m13y = m1y - m3y;
    const double m21x = m2x - m1x, m21y = m2y - m1y;
    const double m32x = m3x - m2x, m32y = m3y - m2y;
    S[0] = 0.5 * fabs(pcx * m13y - pcy * m13x);
    S[1] = 0.5 * fabs(qcx * m21y - qcy * m21x);
    S[2] = 0.5 * fabs(rcx * m32y - rcy * m32x);
    const double D = qx * ry - qy * rx - px * ry + rx * py + px * qy - qx * py;
    props[0] = (qy - ry) / D;
    props[1] = (ry - py) / D;
    props[2] = (py - qy) / D;
    props[3] = (rx - qx) / D;
    props[4] = (px - rx) / D;
    props[5] = (qx - px) / D;
    props[6] = (qx * ry - rx * qy) / D;
    props[7] = (rx * py - px * ry) / D;
    props[8] = (px * qy - qx * py) / D;
    const double mx[3] = {m1x, m2x, m3x}, my[3] = {m1y, m2y, m3y};
    for (int e = 0; e < 3; ++e) {
        props[9 + 2 * e] = (mx[e] + cx) / 2;
        props[10 + 2 * e] = (my[e] + cy) / 2;
        const double ex = cx - mx[e], ey = cy - my[e];
        const double l = sqrt(ex * ex + ey * ey);  // LinearAlgebra.norm of a 2-tuple, no rescaling needed
        props[15 + 2 * e] = ey / l;
        props[16 + 2 * e] = -ex / l;
        props[21 + e] = l;
    }
}

// Orientation determinant of (p, q, r), the D of the shape coefficients: positive for a
// counter-clockwise triangle.
FVM_GEOM_HD double triangle_det(const double* P, int32_t i, int32_t j, int32_t k) {
    const double px = P[2 * i], py = P[2 * i + 1], qx = P[2 * j], qy = P[2 * j + 1], rx = P[2 * k], ry = P[2 * k + 1];
    return qx * ry - qy * rx - px * ry + rx * py + px * qy - qx * py;
}

// Hilbert index of (x, y) on a 2^16 x 2^16 grid (the standard rotate-and-reflect walk).
FVM_GEOM_HD uint64_t hilbert_index(uint32_t x, uint32_t y) {
    const uint32_t n = 1u << 16;
    uint64_t d = 0;
    for (uint32_t s = n / 2; s > 0; s /= 2) {
        const uint32_t rx = (x & s) ? 1u : 0u;
        const uint32_t ry = (y & s) ? 1u : 0u;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = s - 1 - (x & (s - 1));
                y = s - 1 - (y & (s - 1));
            } else {
                x &= (s - 1);
                y &= (s - 1);
            }
            const uint32_t t = x;
            x = y;
            y = t;
        } else {
            x &= (s - 1);
            y &= (s - 1);
        }
    }
    return d;
}

// Hilbert key of a point: coordinates scaled to the 2^16 grid over the bounding square.
FVM_GEOM_HD uint64_t point_hilbert_key(double x, double y, double xmin, double ymin, double span) {
    const double gx = floor((x - xmin) / span * 65535.0), gy = floor((y - ymin) / span * 65535.0);
    const uint32_t hx = (uint32_t)(gx < 65535.0 ? gx : 65535.0);
    const uint32_t hy = (uint32_t)(gy < 65535.0 ? gy : 65535.0);
    return hilbert_index(hx, hy);
}

}  // namespace fvm
