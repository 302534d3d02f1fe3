// Device mesh ingest: the FVMGeometry precompute (src/geometry.jl:99-169), the boundary-edge
// triangles (src/utils.jl:1-11), the Hilbert renumbering and the vertex-neighbour pattern as
// kernels and radix sorts, producing exactly what the host build in fvm_mesh.cpp produces.
//   * Triangle geometry: one thread per triangle, the shared triangle_geometry() with no FMA
//     contraction (this file compiles with -fmad=false), so every property rounds as on the host.
//   * Control volumes: the corners are sorted by vertex (a stable radix sort of the corner
//     index by vertex keeps each vertex's corners in triangle order) and each vertex sums its
//     shares in that order, the order of the host's serial scatter: bit-identical sums.
//   * Hilbert order: keys from point_hilbert_key(), stable radix sort of (key, vertex) pairs,
//     ties in vertex order as std::sort of the pairs gives.
//   * Pattern: (row, column) keys of every pair within a triangle plus the diagonal, radix
//     sorted and made unique: the rows' sorted, duplicate-free column lists.
// Sorts, scans and unique selection call CUB (the CUDA toolkit's device primitives).
#include "fvm_internal.h"
#include "fvm_geometry.h"
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>
#include <algorithm>
#include <climits>

namespace fvm {
namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

int bits_for(uint64_t n) {  // bits needed to hold the values 0 .. n
    int b = 1;
    while (b < 64 && (n >> b) != 0) ++b;
    return b;
}

// error words: [0] first clockwise / degenerate triangle, [1] first boundary edge with no
// triangle on its left, [2] first boundary edge whose boundary_adjacent entry disagrees
__global__ void geometry_kernel(const double* __restrict__ P, const int32_t* __restrict__ tri, int64_t nt,
                                double* __restrict__ props, double* __restrict__ S, int* __restrict__ err) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int32_t i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
    if (!(triangle_det(P, i, j, k) > 0)) atomicMin(&err[0], (int)t);
    double s[3];
    triangle_geometry(P, i, j, k, props + 24 * t, s);
    S[3 * t] = s[0];
    S[3 * t + 1] = s[1];
    S[3 * t + 2] = s[2];
}

__global__ void iota_kernel(int32_t* __restrict__ a, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (int32_t)i;
}

__global__ void count_kernel(const int32_t* __restrict__ corner_vertex, int64_t n, int32_t* __restrict__ cnt) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) atomicAdd(&cnt[corner_vertex[c]], 1);
}

// vol[v] = sum of the shares of v's corners in triangle order; has_vertex[v] = 1 if any
__global__ void volume_kernel(const int64_t* __restrict__ start, const int32_t* __restrict__ corners,
                              const double* __restrict__ S, int64_t np, double* __restrict__ vol,
                              uint8_t* __restrict__ has_vertex) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= np) return;
    double acc = 0.0;
    for (int64_t q = start[v]; q < start[v + 1]; ++q) acc += S[corners[q]];
    vol[v] = acc;
    has_vertex[v] = start[v + 1] > start[v] ? 1 : 0;
}

// the triangle holding boundary edge (i, j) with i followed by j, and its third vertex
__global__ void boundary_kernel(const int32_t* __restrict__ be, int64_t nbe, const int32_t* __restrict__ tri,
                                const int64_t* __restrict__ start, const int32_t* __restrict__ corners,
                                const int32_t* __restrict__ given_adj, int32_t* __restrict__ btri,
                                int32_t* __restrict__ badj, int* __restrict__ err) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbe) return;
    const int32_t i = be[2 * e], j = be[2 * e + 1];
    int32_t t_found = -1, k = -1;
    for (int64_t q = start[i]; q < start[i + 1]; ++q) {  // every match; the last one is kept
        const int32_t c = corners[q];
        const int32_t t = c / 3, at = c % 3;
        if (tri[3 * t + (at + 1) % 3] == j) {
            t_found = t;
            k = tri[3 * t + (at + 2) % 3];
        }
    }
    btri[e] = t_found;
    badj[e] = k;
    if (t_found < 0) atomicMin(&err[1], (int)e);
    else if (given_adj && given_adj[e] != k) atomicMin(&err[2], (int)e);
}

__global__ void hilbert_key_kernel(const double* __restrict__ P, const uint8_t* __restrict__ has_vertex, int64_t np,
                                   double xmin, double ymin, double span, uint64_t* __restrict__ key) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= np) return;
    // every Hilbert index is below 2^32: points that are not vertices go last
    key[v] = has_vertex[v] ? point_hilbert_key(P[2 * v], P[2 * v + 1], xmin, ymin, span) : (uint64_t(1) << 32);
}

__global__ void inverse_perm_kernel(const int32_t* __restrict__ perm, int64_t np, int32_t* __restrict__ iperm) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < np) iperm[perm[v]] = (int32_t)v;
}

// keys row << 32 | col (internal numbering): six per triangle, then the np diagonals
__global__ void pair_key_kernel(const int32_t* __restrict__ tri, int64_t nt, const int32_t* __restrict__ iperm,
                                int64_t np, uint64_t* __restrict__ key) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nt) {
        const uint64_t w0 = (uint32_t)iperm[tri[3 * q]], w1 = (uint32_t)iperm[tri[3 * q + 1]],
                       w2 = (uint32_t)iperm[tri[3 * q + 2]];
        uint64_t* k = key + 6 * q;
        k[0] = w0 << 32 | w1;
        k[1] = w0 << 32 | w2;
        k[2] = w1 << 32 | w0;
        k[3] = w1 << 32 | w2;
        k[4] = w2 << 32 | w0;
        k[5] = w2 << 32 | w1;
    } else if (q < nt + np) {
        const uint64_t v = (uint64_t)(q - nt);
        key[6 * nt + (q - nt)] = v << 32 | v;
    }
}

__global__ void csr_kernel(const uint64_t* __restrict__ key, int64_t nnz, int32_t* __restrict__ col,
                           int64_t* __restrict__ rowptr) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nnz) return;
    const uint64_t r = key[q] >> 32;
    col[q] = (int32_t)(key[q] & 0xffffffffu);
    if (q == 0 || (key[q - 1] >> 32) != r) rowptr[r] = q;  // every row holds its diagonal
}

__global__ void inv_volume_kernel(const double* __restrict__ vol, const int32_t* __restrict__ perm, int64_t np,
                                  double* __restrict__ invV) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= np) return;
    const double V = vol[perm[v]];
    invV[v] = V > 0 ? 1.0 / V : 0.0;
}

// CUB's two-phase calls: the first sizes the scratch, the second runs
template <class F>
void cub_call(DBuf& tmp, F&& f) {
    size_t bytes = 0;
    FVM_CUDA(f(nullptr, bytes));
    if (bytes > tmp.bytes || !tmp.p) tmp.alloc(std::max<size_t>(bytes, 256));  // a null pointer would only size
    FVM_CUDA(f(tmp.p, bytes));
}

template <class T>
void download(std::vector<T>& dst, const DBuf& src, size_t n, cudaStream_t s) {
    dst.resize(n);
    if (n) FVM_CUDA(cudaMemcpyAsync(dst.data(), src.p, sizeof(T) * n, cudaMemcpyDeviceToHost, s));
}

}  // namespace

void mesh_ingest_device(fvm_mesh* m, const int32_t* boundary_adjacent, bool renumber) {
    const int64_t np = m->np, nt = m->nt, nbe = m->nbe;
    if (3 * nt >= (int64_t)INT_MAX || 6 * nt + np >= (int64_t)INT_MAX)
        fail(FVM_ERR_INVALID_ARGUMENT, "mesh too large for the device ingest (use FVM_MESH_HOST_INGEST)");
    cudaStream_t s = nullptr;  // legacy default stream: ordered with the library's later uploads
    SetupTrace tr("mesh device");
    DBuf d_P, d_tri, d_be, d_adj, d_err, d_props, d_S, tmp;
    d_P.upload(m->pts);
    d_tri.upload(m->tri);
    if (nbe) d_be.upload(m->be);
    if (nbe && boundary_adjacent) {
        std::vector<int32_t> adj(boundary_adjacent, boundary_adjacent + nbe);
        d_adj.upload(adj);
    }
    const std::vector<int> err_init = {INT_MAX, INT_MAX, INT_MAX};
    d_err.upload(err_init);
    int* err = d_err.as<int>();
    d_props.alloc(sizeof(double) * 24 * nt);
    d_S.alloc(sizeof(double) * 3 * nt);
    geometry_kernel<<<blocks_for(nt), kThreads, 0, s>>>(d_P.as<double>(), d_tri.as<int32_t>(), nt,
                                                       d_props.as<double>(), d_S.as<double>(), err);
    FVM_CUDA(cudaGetLastError());

    // corners sorted by vertex, each vertex's corners in triangle order
    const int64_t nc = 3 * nt;
    DBuf d_cidx, d_ckey_out, d_corners, d_cnt, d_start;
    d_cidx.alloc(sizeof(int32_t) * nc);
    d_ckey_out.alloc(sizeof(int32_t) * nc);
    d_corners.alloc(sizeof(int32_t) * nc);
    iota_kernel<<<blocks_for(nc), kThreads, 0, s>>>(d_cidx.as<int32_t>(), nc);
    const int vbits = bits_for((uint64_t)np);
    cub_call(tmp, [&](void* p, size_t& b) {
        return cub::DeviceRadixSort::SortPairs(p, b, reinterpret_cast<const uint32_t*>(d_tri.p),
                                               d_ckey_out.as<uint32_t>(), d_cidx.as<int32_t>(),
                                               d_corners.as<int32_t>(), (int)nc, 0, vbits, s);
    });
    d_cnt.alloc(sizeof(int32_t) * (np + 1));
    FVM_CUDA(cudaMemsetAsync(d_cnt.p, 0, sizeof(int32_t) * (np + 1), s));
    count_kernel<<<blocks_for(nc), kThreads, 0, s>>>(d_tri.as<int32_t>(), nc, d_cnt.as<int32_t>());
    d_start.alloc(sizeof(int64_t) * (np + 1));
    cub_call(tmp, [&](void* p, size_t& b) {
        return cub::DeviceScan::ExclusiveSum(p, b, d_cnt.as<int32_t>(), d_start.as<int64_t>(), (int)(np + 1), s);
    });
    DBuf d_vol, d_has;
    d_vol.alloc(sizeof(double) * np);
    d_has.alloc(np);
    volume_kernel<<<blocks_for(np), kThreads, 0, s>>>(d_start.as<int64_t>(), d_corners.as<int32_t>(),
                                                      d_S.as<double>(), np, d_vol.as<double>(),
                                                      d_has.as<uint8_t>());
    DBuf d_btri, d_badj;
    if (nbe) {
        d_btri.alloc(sizeof(int32_t) * nbe);
        d_badj.alloc(sizeof(int32_t) * nbe);
        boundary_kernel<<<blocks_for(nbe), kThreads, 0, s>>>(
            d_be.as<int32_t>(), nbe, d_tri.as<int32_t>(), d_start.as<int64_t>(), d_corners.as<int32_t>(),
            boundary_adjacent ? d_adj.as<int32_t>() : nullptr, d_btri.as<int32_t>(), d_badj.as<int32_t>(), err);
    }
    FVM_CUDA(cudaGetLastError());
    int herr[3];
    FVM_CUDA(cudaMemcpyAsync(herr, err, sizeof herr, cudaMemcpyDeviceToHost, s));
    download(m->has_vertex, d_has, (size_t)np, s);
    FVM_CUDA(cudaStreamSynchronize(s));
    if (herr[0] != INT_MAX) {
        const int32_t* w = &m->tri[3 * (size_t)herr[0]];
        fail(FVM_ERR_BAD_MESH, "triangle " + std::to_string(herr[0]) + " is clockwise or degenerate (determinant " +
                                   std::to_string(triangle_det(m->pts.data(), w[0], w[1], w[2])) + ")");
    }
    if (herr[1] != INT_MAX) {
        const int e = herr[1];
        fail(FVM_ERR_BAD_MESH, "boundary edge " + std::to_string(e) + " (" + std::to_string(m->be[2 * e]) + ", " +
                                   std::to_string(m->be[2 * e + 1]) + ") has no solid triangle on its left");
    }
    if (herr[2] != INT_MAX)
        fail(FVM_ERR_BAD_MESH, "boundary_adjacent[" + std::to_string(herr[2]) + "] does not match the triangle on the edge");
    m->nv = 0;
    for (int64_t v = 0; v < np; ++v) m->nv += m->has_vertex[v];
    tr.mark("geometry+volumes+boundary");

    // Hilbert renumbering (the bounding square over every point, as on the host)
    DBuf d_key, d_key_out, d_vidx, d_perm, d_iperm;
    d_perm.alloc(sizeof(int32_t) * np);
    d_iperm.alloc(sizeof(int32_t) * np);
    if (renumber) {
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        const double* P = m->pts.data();
        for (int64_t v = 0; v < np; ++v) {
            xmin = std::min(xmin, P[2 * v]);
            xmax = std::max(xmax, P[2 * v]);
            ymin = std::min(ymin, P[2 * v + 1]);
            ymax = std::max(ymax, P[2 * v + 1]);
        }
        double span = std::max(xmax - xmin, ymax - ymin);
        if (!(span > 0)) span = 1.0;
        d_key.alloc(sizeof(uint64_t) * np);
        d_key_out.alloc(sizeof(uint64_t) * np);
        d_vidx.alloc(sizeof(int32_t) * np);
        hilbert_key_kernel<<<blocks_for(np), kThreads, 0, s>>>(d_P.as<double>(), d_has.as<uint8_t>(), np, xmin, ymin,
                                                               span, d_key.as<uint64_t>());
        iota_kernel<<<blocks_for(np), kThreads, 0, s>>>(d_vidx.as<int32_t>(), np);
        cub_call(tmp, [&](void* p, size_t& b) {
            return cub::DeviceRadixSort::SortPairs(p, b, d_key.as<uint64_t>(), d_key_out.as<uint64_t>(),
                                                   d_vidx.as<int32_t>(), d_perm.as<int32_t>(), (int)np, 0, 33, s);
        });
    } else {
        iota_kernel<<<blocks_for(np), kThreads, 0, s>>>(d_perm.as<int32_t>(), np);
    }
    inverse_perm_kernel<<<blocks_for(np), kThreads, 0, s>>>(d_perm.as<int32_t>(), np, d_iperm.as<int32_t>());
    FVM_CUDA(cudaGetLastError());
    tr.mark("hilbert");

    // vertex-neighbour pattern: sorted, unique (row, col) keys
    {
        const int64_t nk = 6 * nt + np;
        DBuf d_pk, d_pk_sorted, d_nsel;
        d_pk.alloc(sizeof(uint64_t) * nk);
        d_pk_sorted.alloc(sizeof(uint64_t) * nk);
        d_nsel.alloc(sizeof(int64_t));
        pair_key_kernel<<<blocks_for(nt + np), kThreads, 0, s>>>(d_tri.as<int32_t>(), nt, d_iperm.as<int32_t>(), np,
                                                                 d_pk.as<uint64_t>());
        cub_call(tmp, [&](void* p, size_t& b) {
            return cub::DeviceRadixSort::SortKeys(p, b, d_pk.as<uint64_t>(), d_pk_sorted.as<uint64_t>(), (int)nk, 0,
                                                  32 + vbits, s);
        });
        cub_call(tmp, [&](void* p, size_t& b) {
            return cub::DeviceSelect::Unique(p, b, d_pk_sorted.as<uint64_t>(), d_pk.as<uint64_t>(),
                                             d_nsel.as<int64_t>(), (int)nk, s);
        });
        int64_t nnz = 0;
        FVM_CUDA(cudaMemcpyAsync(&nnz, d_nsel.p, sizeof nnz, cudaMemcpyDeviceToHost, s));
        FVM_CUDA(cudaStreamSynchronize(s));
        DBuf d_col, d_rowptr;
        d_col.alloc(sizeof(int32_t) * std::max<int64_t>(nnz, 1));
        d_rowptr.alloc(sizeof(int64_t) * (np + 1));
        csr_kernel<<<blocks_for(nnz), kThreads, 0, s>>>(d_pk.as<uint64_t>(), nnz, d_col.as<int32_t>(),
                                                        d_rowptr.as<int64_t>());
        FVM_CUDA(cudaMemcpyAsync(d_rowptr.as<int64_t>() + np, &nnz, sizeof nnz, cudaMemcpyHostToDevice, s));
        FVM_CUDA(cudaGetLastError());
        SellPattern& pat = m->pat;
        pat.nrows = np;
        download(pat.rowptr, d_rowptr, (size_t)(np + 1), s);
        download(pat.csr_col, d_col, (size_t)nnz, s);
        FVM_CUDA(cudaStreamSynchronize(s));
        tr.mark("pattern (device)");
        finalize_sell(pat, np);
        SellPattern& off = m->pat_off;
        off.nrows = np;
        off.rowptr.assign(np + 1, 0);
        off.csr_col.reserve(pat.nnz);
        for (int64_t v = 0; v < np; ++v) {
            for (int64_t q = pat.rowptr[v]; q < pat.rowptr[v + 1]; ++q)
                if (pat.csr_col[q] != v) off.csr_col.push_back(pat.csr_col[q]);
            off.rowptr[v + 1] = (int64_t)off.csr_col.size();
        }
        finalize_sell(off, np);
        tr.mark("pattern (sliced ELL)");
    }

    // device-side vertex data, and the host copies the set-up code reads
    m->d_invV.alloc(sizeof(double) * np);
    inv_volume_kernel<<<blocks_for(np), kThreads, 0, s>>>(d_vol.as<double>(), d_perm.as<int32_t>(), np,
                                                          m->d_invV.as<double>());
    FVM_CUDA(cudaGetLastError());
    download(m->vol, d_vol, (size_t)np, s);
    download(m->props, d_props, (size_t)24 * nt, s);
    download(m->perm, d_perm, (size_t)np, s);
    download(m->iperm, d_iperm, (size_t)np, s);
    if (nbe) {
        download(m->btri, d_btri, (size_t)nbe, s);
        download(m->badj, d_badj, (size_t)nbe, s);
    }
    FVM_CUDA(cudaStreamSynchronize(s));
    m->d_perm = std::move(d_perm);
    m->d_iperm = std::move(d_iperm);
    tr.mark("download");
}

}  // namespace fvm
