// Post-processing on the device: point location over a uniform grid of triangles and the
// piecewise-linear interpolant of a solution (pl_interpolate, src/utils.jl:23-27) for many
// points per launch.  Compiled with -fmad=false: alpha, beta, gamma and alpha x + beta y +
// gamma round as the reference's (and the host mirror's) separate multiplies and adds.
#include "fvm_internal.h"
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <algorithm>
#include <cmath>

namespace fvm {
namespace {

constexpr int kThreads = 256;
inline unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

struct Grid {
    double xmin, ymin, inv_h;
    int64_t gx, gy;
    __device__ int64_t cx(double x) const {
        const double c = floor((x - xmin) * inv_h);
        return c < 0 ? 0 : (c >= (double)gx ? gx - 1 : (int64_t)c);
    }
    __device__ int64_t cy(double y) const {
        const double c = floor((y - ymin) * inv_h);
        return c < 0 ? 0 : (c >= (double)gy ? gy - 1 : (int64_t)c);
    }
};

__device__ void tri_box(const double* P, const int32_t* T, int64_t t, const Grid& g, int64_t& x0, int64_t& x1,
                        int64_t& y0, int64_t& y1) {
    const int32_t a = T[3 * t], b = T[3 * t + 1], c = T[3 * t + 2];
    const double xa = P[2 * a], xb = P[2 * b], xc = P[2 * c], ya = P[2 * a + 1], yb = P[2 * b + 1], yc = P[2 * c + 1];
    x0 = g.cx(fmin(xa, fmin(xb, xc)));
    x1 = g.cx(fmax(xa, fmax(xb, xc)));
    y0 = g.cy(fmin(ya, fmin(yb, yc)));
    y1 = g.cy(fmax(ya, fmax(yb, yc)));
}

__global__ void cells_per_tri_kernel(const double* P, const int32_t* T, int64_t nt, Grid g, int64_t* cnt) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t > nt) return;
    if (t == nt) {  // the scan's last entry
        cnt[t] = 0;
        return;
    }
    int64_t x0, x1, y0, y1;
    tri_box(P, T, t, g, x0, x1, y0, y1);
    cnt[t] = (x1 - x0 + 1) * (y1 - y0 + 1);
}

__global__ void fill_pairs_kernel(const double* P, const int32_t* T, int64_t nt, Grid g, const int64_t* off,
                                  uint32_t* cell, int32_t* tri) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int64_t x0, x1, y0, y1;
    tri_box(P, T, t, g, x0, x1, y0, y1);
    int64_t q = off[t];
    for (int64_t y = y0; y <= y1; ++y)
        for (int64_t x = x0; x <= x1; ++x) {
            cell[q] = (uint32_t)(y * g.gx + x);
            tri[q] = (int32_t)t;
            ++q;
        }
}

__global__ void cell_count_kernel(const uint32_t* cell, int64_t n, int64_t* cnt) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[cell[q]]), 1ull);
}

__global__ void shape_kernel(const double* props, int64_t nt, double* shape) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < 9 * nt) shape[q] = props[24 * (q / 9) + q % 9];
}

// orientation of (a, b, p): twice the signed area, positive when p is left of a -> b
__device__ double orient(double ax, double ay, double bx, double by, double px, double py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

// the first (lowest) listed triangle whose three orientations are >= 0; failing that, one
// within rounding of its edges (relative 1e-12 of the triangle's doubled area)
__global__ void locate_kernel(const double* P, const int32_t* T, Grid g, const int64_t* start, const int32_t* list,
                              const double* xy, int64_t nq, int64_t* out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const double px = xy[2 * q], py = xy[2 * q + 1];
    int64_t found = -1, near = -1;
    double best = -INFINITY;
    if (px >= g.xmin && py >= g.ymin && px <= g.xmin + g.gx / g.inv_h && py <= g.ymin + g.gy / g.inv_h) {
        const int64_t c = g.cy(py) * g.gx + g.cx(px);
        for (int64_t k = start[c]; k < start[c + 1]; ++k) {
            const int32_t t = list[k];
            const int32_t a = T[3 * t], b = T[3 * t + 1], cc = T[3 * t + 2];
            const double ax = P[2 * a], ay = P[2 * a + 1], bx = P[2 * b], by = P[2 * b + 1], cx = P[2 * cc],
                         cy = P[2 * cc + 1];
            const double o1 = orient(ax, ay, bx, by, px, py), o2 = orient(bx, by, cx, cy, px, py),
                         o3 = orient(cx, cy, ax, ay, px, py);
            if (o1 >= 0 && o2 >= 0 && o3 >= 0) {
                found = t;
                break;
            }
            const double area = fabs(orient(ax, ay, bx, by, cx, cy));
            const double m = fmin(o1, fmin(o2, o3)) / area;
            if (m > best) {
                best = m;
                near = t;
            }
        }
        if (found < 0 && best >= -1e-12) found = near;
    }
    out[q] = found;
}

template <bool INTERNAL>
__global__ void interp_kernel(const int32_t* T, const double* shape, const int32_t* iperm, const double* u, int ncomp,
                              const int64_t* tri, const double* xy, int64_t nq, int64_t nt, double* out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int64_t t = tri[q];
    if (t < 0 || t >= nt) {
        for (int c = 0; c < ncomp; ++c) out[q * ncomp + c] = NAN;
        return;
    }
    int64_t v[3];
    for (int k = 0; k < 3; ++k) {
        const int32_t w = T[3 * t + k];
        v[k] = INTERNAL ? iperm[w] : w;
    }
    const double* s = shape + 9 * t;
    const double x = xy[2 * q], y = xy[2 * q + 1];
    for (int c = 0; c < ncomp; ++c) {
        const double ua = u[v[0] * ncomp + c], ub = u[v[1] * ncomp + c], uc = u[v[2] * ncomp + c];
        const double al = s[0] * ua + s[1] * ub + s[2] * uc;
        const double be = s[3] * ua + s[4] * ub + s[5] * uc;
        const double ga = s[6] * ua + s[7] * ub + s[8] * uc;
        out[q * ncomp + c] = al * x + be * y + ga;
    }
}

template <class F>
void cub_call(DBuf& tmp, F&& f) {
    size_t bytes = 0;
    FVM_CUDA(f(nullptr, bytes));
    if (bytes > tmp.bytes || !tmp.p) tmp.alloc(std::max<size_t>(bytes, 256));  // a null pointer would only size
    FVM_CUDA(f(tmp.p, bytes));
}

Grid grid_of(const Locator& L) { return Grid{L.xmin, L.ymin, 1.0 / L.h, L.gx, L.gy}; }

void build_locator(fvm_mesh* m, cudaStream_t s) {
    Locator& L = m->loc;
    if (L.ready) return;
    const int64_t nt = m->nt, np = m->np;
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
    for (int64_t t = 0; t < 3 * nt; ++t) {  // the box of the triangles' vertices
        const int32_t v = m->tri[t];
        xmin = std::min(xmin, m->pts[2 * v]);
        xmax = std::max(xmax, m->pts[2 * v]);
        ymin = std::min(ymin, m->pts[2 * v + 1]);
        ymax = std::max(ymax, m->pts[2 * v + 1]);
    }
    const double w = std::max(xmax - xmin, 1e-300), hgt = std::max(ymax - ymin, 1e-300);
    // about two triangles per cell, at most 2^22 cells
    const double cells = std::min<double>(std::max<double>(1.0, nt / 2.0), 4194304.0);
    double h = std::sqrt(w * hgt / cells);
    if (!(h > 0)) h = std::max(w, hgt);
    L.gx = std::max<int64_t>(1, (int64_t)std::ceil(w / h));
    L.gy = std::max<int64_t>(1, (int64_t)std::ceil(hgt / h));
    while (L.gx * L.gy > 4194304) {
        h *= 1.25;
        L.gx = std::max<int64_t>(1, (int64_t)std::ceil(w / h));
        L.gy = std::max<int64_t>(1, (int64_t)std::ceil(hgt / h));
    }
    L.xmin = xmin;
    L.ymin = ymin;
    L.h = h;
    L.d_pts.upload(m->pts);
    L.d_tri.upload(m->tri);
    {
        DBuf d_props;
        d_props.upload(m->props);
        L.d_shape.alloc(sizeof(double) * 9 * nt);
        shape_kernel<<<blocks_for(9 * nt), kThreads, 0, s>>>(d_props.as<double>(), nt, L.d_shape.as<double>());
        FVM_CUDA(cudaStreamSynchronize(s));
    }
    const Grid g = grid_of(L);
    DBuf cnt, off, tmp;
    cnt.alloc(sizeof(int64_t) * (nt + 1));
    off.alloc(sizeof(int64_t) * (nt + 1));
    cells_per_tri_kernel<<<blocks_for(nt + 1), kThreads, 0, s>>>(L.d_pts.as<double>(), L.d_tri.as<int32_t>(), nt, g,
                                                                 cnt.as<int64_t>());
    cub_call(tmp, [&](void* p, size_t& b) {
        return cub::DeviceScan::ExclusiveSum(p, b, cnt.as<int64_t>(), off.as<int64_t>(), (int)(nt + 1), s);
    });
    int64_t npairs = 0;
    FVM_CUDA(cudaMemcpyAsync(&npairs, off.as<int64_t>() + nt, sizeof npairs, cudaMemcpyDeviceToHost, s));
    FVM_CUDA(cudaStreamSynchronize(s));
    if (npairs >= (int64_t)INT32_MAX) fail(FVM_ERR_UNSUPPORTED, "point location grid too large");
    DBuf cell, cell_sorted, tri, tri_sorted;
    cell.alloc(sizeof(uint32_t) * std::max<int64_t>(npairs, 1));
    cell_sorted.alloc(sizeof(uint32_t) * std::max<int64_t>(npairs, 1));
    tri.alloc(sizeof(int32_t) * std::max<int64_t>(npairs, 1));
    L.d_cell_tri.alloc(sizeof(int32_t) * std::max<int64_t>(npairs, 1));
    fill_pairs_kernel<<<blocks_for(nt), kThreads, 0, s>>>(L.d_pts.as<double>(), L.d_tri.as<int32_t>(), nt, g,
                                                          off.as<int64_t>(), cell.as<uint32_t>(), tri.as<int32_t>());
    // stable by cell: each cell's triangles stay in ascending order
    int cbits = 1;
    while (cbits < 32 && ((uint64_t)(L.gx * L.gy) >> cbits) != 0) ++cbits;
    cub_call(tmp, [&](void* p, size_t& b) {
        return cub::DeviceRadixSort::SortPairs(p, b, cell.as<uint32_t>(), cell_sorted.as<uint32_t>(), tri.as<int32_t>(),
                                               L.d_cell_tri.as<int32_t>(), (int)npairs, 0, cbits, s);
    });
    const int64_t ncell = L.gx * L.gy;
    DBuf ccnt;
    ccnt.alloc(sizeof(int64_t) * (ncell + 1));
    FVM_CUDA(cudaMemsetAsync(ccnt.p, 0, sizeof(int64_t) * (ncell + 1), s));
    cell_count_kernel<<<blocks_for(npairs), kThreads, 0, s>>>(cell_sorted.as<uint32_t>(), npairs, ccnt.as<int64_t>());
    L.d_cell_start.alloc(sizeof(int64_t) * (ncell + 1));
    cub_call(tmp, [&](void* p, size_t& b) {
        return cub::DeviceScan::ExclusiveSum(p, b, ccnt.as<int64_t>(), L.d_cell_start.as<int64_t>(), (int)(ncell + 1),
                                             s);
    });
    FVM_CUDA(cudaStreamSynchronize(s));
    (void)np;
    L.ready = true;
}

// device copy of a host array (or the device pointer itself)
template <class T>
const T* to_device(const T* p, size_t n, bool host, DBuf& keep, cudaStream_t s) {
    if (!host) return p;
    keep.alloc(sizeof(T) * std::max<size_t>(n, 1));
    if (n) FVM_CUDA(cudaMemcpyAsync(keep.p, p, sizeof(T) * n, cudaMemcpyHostToDevice, s));
    return keep.as<T>();
}

}  // namespace
}  // namespace fvm

using namespace fvm;

extern "C" int fvm_mesh_locate(fvm_mesh* m, int64_t nq, const double* xy, int64_t* tri_out, int32_t flags,
                               void* stream) {
    return guard_call([&] {
        if (!m || (nq > 0 && (!xy || !tri_out))) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (nq < 0) fail(FVM_ERR_INVALID_ARGUMENT, "nq must be >= 0");
        const int32_t loc = flags & 3;
        if (loc != FVM_PTR_HOST && loc != FVM_PTR_DEVICE) fail(FVM_ERR_INVALID_ARGUMENT, "flags: FVM_PTR_HOST or FVM_PTR_DEVICE");
        cudaStream_t s = (cudaStream_t)stream;
        build_locator(m, s);
        if (nq == 0) return FVM_OK;
        const bool host = loc == FVM_PTR_HOST;
        DBuf kxy, kout;
        const double* dxy = to_device(xy, 2 * (size_t)nq, host, kxy, s);
        int64_t* dout = tri_out;
        if (host) {
            kout.alloc(sizeof(int64_t) * nq);
            dout = kout.as<int64_t>();
        }
        const Locator& L = m->loc;
        locate_kernel<<<blocks_for(nq), kThreads, 0, s>>>(L.d_pts.as<double>(), L.d_tri.as<int32_t>(), grid_of(L),
                                                          L.d_cell_start.as<int64_t>(), L.d_cell_tri.as<int32_t>(), dxy,
                                                          nq, dout);
        FVM_CUDA(cudaGetLastError());
        if (host) {
            FVM_CUDA(cudaMemcpyAsync(tri_out, dout, sizeof(int64_t) * nq, cudaMemcpyDeviceToHost, s));
            FVM_CUDA(cudaStreamSynchronize(s));
        }
        return FVM_OK;
    });
}

extern "C" int fvm_pl_interpolate(fvm_mesh* m, const double* u, int32_t ncomp, int64_t nq, const int64_t* tri,
                                  const double* xy, double* out, int32_t flags, void* stream) {
    return guard_call([&] {
        if (!m || !u || (nq > 0 && (!tri || !xy || !out))) fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        if (ncomp < 1 || nq < 0) fail(FVM_ERR_INVALID_ARGUMENT, "ncomp must be >= 1 and nq >= 0");
        const int32_t loc = flags & 3;
        if (loc > FVM_PTR_DEVICE_INTERNAL) fail(FVM_ERR_INVALID_ARGUMENT, "bad pointer-location flag");
        cudaStream_t s = (cudaStream_t)stream;
        build_locator(m, s);
        if (nq == 0) return FVM_OK;
        const bool host = loc == FVM_PTR_HOST;
        DBuf ku, kt, kxy, kout;
        const double* du = to_device(u, (size_t)m->np * ncomp, host, ku, s);
        const int64_t* dt = to_device(tri, (size_t)nq, host, kt, s);
        const double* dxy = to_device(xy, 2 * (size_t)nq, host, kxy, s);
        double* dout = out;
        if (host) {
            kout.alloc(sizeof(double) * nq * ncomp);
            dout = kout.as<double>();
        }
        const Locator& L = m->loc;
        if (loc == FVM_PTR_DEVICE_INTERNAL)
            interp_kernel<true><<<blocks_for(nq), kThreads, 0, s>>>(L.d_tri.as<int32_t>(), L.d_shape.as<double>(),
                                                                    m->d_iperm.as<int32_t>(), du, ncomp, dt, dxy, nq,
                                                                    m->nt, dout);
        else
            interp_kernel<false><<<blocks_for(nq), kThreads, 0, s>>>(L.d_tri.as<int32_t>(), L.d_shape.as<double>(),
                                                                     nullptr, du, ncomp, dt, dxy, nq, m->nt, dout);
        FVM_CUDA(cudaGetLastError());
        if (host) {
            FVM_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * nq * ncomp, cudaMemcpyDeviceToHost, s));
            FVM_CUDA(cudaStreamSynchronize(s));
        }
        return FVM_OK;
    });
}
