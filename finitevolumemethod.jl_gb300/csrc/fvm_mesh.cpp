// Host side of the mesh: geometry (FVMGeometry), Hilbert renumbering, the vertex-neighbour
// operator pattern (sliced ELL) and the vertex tiles of the per-triangle flux kernel.
// Compiled with -ffp-contract=off so the geometry arithmetic rounds like the reference.
#include "fvm_internal.h"
#include "fvm_geometry.h"
#include <algorithm>
#include <cmath>
#include <numeric>
#include <unordered_map>

namespace fvm {

int64_t SellPattern::find_csr(int32_t row, int32_t c) const {
    int64_t lo = rowptr[row], hi = rowptr[row + 1];
    const int32_t* b = csr_col.data();
    if (hi - lo <= 16) {  // the usual vertex degree: a short sorted scan
        for (int64_t q = lo; q < hi && b[q] <= c; ++q)
            if (b[q] == c) return q;
        return -1;
    }
    const int32_t* it = std::lower_bound(b + lo, b + hi, c);
    if (it == b + hi || *it != c) return -1;
    return it - b;
}

int64_t SellPattern::find(int32_t row, int32_t c) const {
    int64_t q = find_csr(row, c);
    return q < 0 ? -1 : csr_slot[q];
}

}  // namespace fvm

using namespace fvm;

static inline uint64_t edge_key(int64_t a, int64_t b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }

// Sliced ELL from the CSR view (rowptr, csr_col): slices of 32 rows, width = longest row in the
// slice, slots column-major; padding slots point at the row itself with value 0.
void fvm::finalize_sell(SellPattern& pat, int64_t nrows) {
    pat.nnz = (int64_t)pat.csr_col.size();
    pat.nslices = (nrows + kSlice - 1) / kSlice;
    pat.slice_ptr.assign(pat.nslices + 1, 0);
    pat.width.assign(pat.nslices, 0);
    for (int64_t s = 0; s < pat.nslices; ++s) {
        int32_t w = 0;
        for (int64_t r = s * kSlice; r < std::min<int64_t>(nrows, (s + 1) * kSlice); ++r)
            w = std::max<int32_t>(w, (int32_t)(pat.rowptr[r + 1] - pat.rowptr[r]));
        pat.width[s] = w;
        pat.maxw = std::max(pat.maxw, (int)w);
        pat.slice_ptr[s + 1] = pat.slice_ptr[s] + (int64_t)w * kSlice;
    }
    pat.nslots = pat.slice_ptr[pat.nslices];
    pat.col.assign(pat.nslots, 0);
    pat.csr_slot.assign(pat.nnz, 0);
    for (int64_t s = 0; s < pat.nslices; ++s)
        for (int lane = 0; lane < kSlice; ++lane) {
            int64_t r = s * kSlice + lane;
            int64_t len = r < nrows ? pat.rowptr[r + 1] - pat.rowptr[r] : 0;
            int32_t pad = r < nrows ? (int32_t)r : (int32_t)(nrows - 1);
            for (int32_t q = 0; q < pat.width[s]; ++q) {
                int64_t slot = pat.slice_ptr[s] + (int64_t)q * kSlice + lane;
                if (q < len) {
                    pat.col[slot] = pat.csr_col[pat.rowptr[r] + q];
                    pat.csr_slot[pat.rowptr[r] + q] = slot;
                } else {
                    pat.col[slot] = pad;
                }
            }
        }
    {  // two padding entries: the streamed kernel copies its window of offsets in 16-byte units
        std::vector<int64_t> padded(pat.slice_ptr);
        padded.push_back(pat.nslots);
        padded.push_back(pat.nslots);
        pat.d_slice_ptr.upload(padded);
    }
    pat.d_width.upload(pat.width);
    pat.d_col.upload(pat.col);
}

extern "C" int fvm_mesh_create_impl(const double* points, int64_t npoints, const int32_t* triangles, int64_t ntri,
                                     const int32_t* boundary_edges, const int32_t* boundary_adjacent,
                                     int64_t nbedge, int32_t tile_vertices, int32_t flags, fvm_mesh** out) {
    if (!out) fail(FVM_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (npoints <= 0 || ntri <= 0 || nbedge < 0) fail(FVM_ERR_INVALID_ARGUMENT, "mesh sizes must be positive");
    if (!points || !triangles || (nbedge > 0 && !boundary_edges)) fail(FVM_ERR_INVALID_ARGUMENT, "NULL mesh array");
    if (npoints >= (int64_t)INT32_MAX || ntri >= (int64_t)INT32_MAX) fail(FVM_ERR_INVALID_ARGUMENT, "mesh too large for 32-bit indices");
    SetupTrace tr("mesh");
    std::unique_ptr<fvm_mesh> m(new fvm_mesh());
    FVM_CUDA(cudaGetDevice(&m->device));
    m->np = npoints;
    m->nt = ntri;
    m->nbe = nbedge;
    m->tile_vertices_req = tile_vertices;
    m->pts.assign(points, points + 2 * npoints);
    m->tri.assign(triangles, triangles + 3 * ntri);
    m->be.assign(boundary_edges, boundary_edges + 2 * nbedge);
    for (int64_t t = 0; t < 3 * ntri; ++t)
        if (m->tri[t] < 0 || m->tri[t] >= npoints)
            fail(FVM_ERR_BAD_MESH, "triangle " + std::to_string(t / 3) + " has a vertex index out of range");
    for (int64_t e = 0; e < 2 * nbedge; ++e)
        if (m->be[e] < 0 || m->be[e] >= npoints)
            fail(FVM_ERR_BAD_MESH, "boundary edge " + std::to_string(e / 2) + " has a vertex index out of range");
    tr.mark("copy");
    if (!(flags & FVM_MESH_HOST_INGEST)) {
        mesh_ingest_device(m.get(), boundary_adjacent, !(flags & FVM_MESH_NO_RENUMBER));
        *out = m.release();
        return FVM_OK;
    }

    // geometry (src/geometry.jl:99-169), triangles in the caller's order
    m->vol.assign(npoints, 0.0);
    m->props.resize((size_t)24 * ntri);
    m->has_vertex.assign(npoints, 0);
    const double* P = m->pts.data();
    for (int64_t t = 0; t < ntri; ++t) {
        int32_t i = m->tri[3 * t], j = m->tri[3 * t + 1], k = m->tri[3 * t + 2];
        double px = P[2 * i], py = P[2 * i + 1], qx = P[2 * j], qy = P[2 * j + 1], rx = P[2 * k], ry = P[2 * k + 1];
        double D = qx * ry - qy * rx - px * ry + rx * py + px * qy - qx * py;
        if (!(D > 0))
            fail(FVM_ERR_BAD_MESH, "triangle " + std::to_string(t) + " is clockwise or degenerate (determinant " +
                                       std::to_string(D) + ")");
        double S[3];
        triangle_geometry(P, i, j, k, &m->props[24 * t], S);
        m->vol[i] += S[0];
        m->vol[j] += S[1];
        m->vol[k] += S[2];
        m->has_vertex[i] = m->has_vertex[j] = m->has_vertex[k] = 1;
    }
    m->nv = 0;
    for (int64_t v = 0; v < npoints; ++v) m->nv += m->has_vertex[v];
    tr.mark("geometry");

    // boundary edge -> triangle (get_adjacent + _safe_get_triangle_props, src/utils.jl:1-11)
    {
        std::unordered_map<uint64_t, int32_t> dir;
        dir.reserve((size_t)ntri * 3 * 2);
        for (int64_t t = 0; t < ntri; ++t)
            for (int e = 0; e < 3; ++e) {
                int32_t a = m->tri[3 * t + e], b = m->tri[3 * t + (e + 1) % 3];
                dir[edge_key(a, b)] = (int32_t)t;
            }
        m->btri.resize(nbedge);
        m->badj.resize(nbedge);
        for (int64_t e = 0; e < nbedge; ++e) {
            int32_t i = m->be[2 * e], j = m->be[2 * e + 1];
            auto it = dir.find(edge_key(i, j));
            if (it == dir.end())
                fail(FVM_ERR_BAD_MESH, "boundary edge " + std::to_string(e) + " (" + std::to_string(i) + ", " +
                                           std::to_string(j) + ") has no solid triangle on its left");
            int32_t t = it->second;
            int32_t k = -1;
            for (int c = 0; c < 3; ++c) {
                int32_t v = m->tri[3 * t + c];
                if (v != i && v != j) k = v;
            }
            if (boundary_adjacent && boundary_adjacent[e] != k)
                fail(FVM_ERR_BAD_MESH, "boundary_adjacent[" + std::to_string(e) + "] does not match the triangle on the edge");
            m->btri[e] = t;
            m->badj[e] = k;
        }
    }

    tr.mark("boundary triangles");
    // Hilbert renumbering of vertices; points that are not vertices go last
    m->perm.resize(npoints);
    m->iperm.resize(npoints);
    if (flags & FVM_MESH_NO_RENUMBER) {
        std::iota(m->perm.begin(), m->perm.end(), 0);
    } else {
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
        for (int64_t v = 0; v < npoints; ++v) {
            xmin = std::min(xmin, P[2 * v]);
            xmax = std::max(xmax, P[2 * v]);
            ymin = std::min(ymin, P[2 * v + 1]);
            ymax = std::max(ymax, P[2 * v + 1]);
        }
        double span = std::max(xmax - xmin, ymax - ymin);
        if (!(span > 0)) span = 1.0;
        std::vector<std::pair<uint64_t, int32_t>> key(npoints);
        for (int64_t v = 0; v < npoints; ++v) {
            uint64_t h = point_hilbert_key(P[2 * v], P[2 * v + 1], xmin, ymin, span);
            if (!m->has_vertex[v]) h = ~0ull;
            key[v] = {h, (int32_t)v};
        }
        std::sort(key.begin(), key.end());
        for (int64_t v = 0; v < npoints; ++v) m->perm[v] = key[v].second;
    }
    for (int64_t v = 0; v < npoints; ++v) m->iperm[m->perm[v]] = (int32_t)v;

    tr.mark("hilbert");
    // vertex-neighbour pattern (internal numbering): diagonal + every pair within a triangle
    {
        SellPattern& pat = m->pat;
        pat.nrows = npoints;
        std::vector<int64_t> cnt(npoints + 1, 0);
        for (int64_t v = 0; v < npoints; ++v) cnt[v] = 1;
        for (int64_t t = 0; t < ntri; ++t)
            for (int a = 0; a < 3; ++a) cnt[m->iperm[m->tri[3 * t + a]]] += 2;
        std::vector<int64_t> start(npoints + 1, 0);
        for (int64_t v = 0; v < npoints; ++v) start[v + 1] = start[v] + cnt[v];
        std::vector<int32_t> tmp(start[npoints]);
        std::vector<int64_t> fillp(start.begin(), start.end() - 1);
        for (int64_t v = 0; v < npoints; ++v) tmp[fillp[v]++] = (int32_t)v;
        for (int64_t t = 0; t < ntri; ++t) {
            int32_t w[3] = {m->iperm[m->tri[3 * t]], m->iperm[m->tri[3 * t + 1]], m->iperm[m->tri[3 * t + 2]]};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    if (a != b) tmp[fillp[w[a]]++] = w[b];
        }
        pat.rowptr.assign(npoints + 1, 0);
        pat.csr_col.clear();
        pat.csr_col.reserve(start[npoints] / 2 + npoints);
        for (int64_t v = 0; v < npoints; ++v) {
            std::sort(tmp.begin() + start[v], tmp.begin() + start[v + 1]);
            int32_t last = -1;
            for (int64_t q = start[v]; q < start[v + 1]; ++q)
                if (tmp[q] != last) {
                    pat.csr_col.push_back(tmp[q]);
                    last = tmp[q];
                }
            pat.rowptr[v + 1] = (int64_t)pat.csr_col.size();
        }
        finalize_sell(pat, npoints);
        // the same neighbourhoods without the diagonal
        SellPattern& off = m->pat_off;
        off.nrows = npoints;
        off.rowptr.assign(npoints + 1, 0);
        off.csr_col.reserve(pat.nnz);
        for (int64_t v = 0; v < npoints; ++v) {
            for (int64_t q = pat.rowptr[v]; q < pat.rowptr[v + 1]; ++q)
                if (pat.csr_col[q] != v) off.csr_col.push_back(pat.csr_col[q]);
            off.rowptr[v + 1] = (int64_t)off.csr_col.size();
        }
        finalize_sell(off, npoints);
    }

    tr.mark("pattern");
    // device-side vertex data
    m->d_perm.upload(m->perm);
    m->d_iperm.upload(m->iperm);
    {
        std::vector<double> invV(npoints, 0.0);
        for (int64_t v = 0; v < npoints; ++v) {
            double V = m->vol[m->perm[v]];
            invV[v] = V > 0 ? 1.0 / V : 0.0;
        }
        m->d_invV.upload(invV);
    }
    tr.mark("upload");
    *out = m.release();
    return FVM_OK;
}

// Tiles of the per-triangle flux kernel: vertex range [t*TV, (t+1)*TV) of the internal
// numbering; a tile lists every triangle (and boundary edge) that scatters into it.
void fvm_mesh::build_tiles() {
    if (tiles.built) return;
    Tiles& T = tiles;
    int TV = tile_vertices_req > 0 ? tile_vertices_req : 1024;
    if (TV % 32 || TV > 4096) fail(FVM_ERR_INVALID_ARGUMENT, "tile_vertices must be a multiple of 32 and <= 4096");
    T.tile_vertices = TV;
    T.ntiles = (np + TV - 1) / TV;
    // triangles ordered by their smallest internal vertex
    std::vector<int32_t> order(nt);
    std::iota(order.begin(), order.end(), 0);
    std::vector<int32_t> minv(nt);
    for (int64_t t = 0; t < nt; ++t)
        minv[t] = std::min({iperm[tri[3 * t]], iperm[tri[3 * t + 1]], iperm[tri[3 * t + 2]]});
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return minv[a] < minv[b]; });
    std::vector<int64_t> cnt(T.ntiles + 1, 0);
    auto tiles_of = [&](const int32_t* w, int n, int64_t* out) {
        int c = 0;
        for (int a = 0; a < n; ++a) {
            int64_t tt = w[a] / TV;
            bool dup = false;
            for (int b = 0; b < c; ++b) dup |= out[b] == tt;
            if (!dup) out[c++] = tt;
        }
        return c;
    };
    for (int64_t t = 0; t < nt; ++t) {
        int32_t w[3] = {iperm[tri[3 * t]], iperm[tri[3 * t + 1]], iperm[tri[3 * t + 2]]};
        int64_t ts[3];
        int c = tiles_of(w, 3, ts);
        for (int a = 0; a < c; ++a) cnt[ts[a]]++;
    }
    T.off.assign(T.ntiles + 1, 0);
    for (int64_t t = 0; t < T.ntiles; ++t) T.off[t + 1] = T.off[t] + cnt[t];
    T.nelem = T.off[T.ntiles];
    T.etri.assign(T.nelem, 0);
    T.ev.assign(3 * T.nelem, 0);
    std::vector<int64_t> fill(T.off.begin(), T.off.end() - 1);
    for (int64_t q = 0; q < nt; ++q) {
        int32_t t = order[q];
        int32_t w[3] = {iperm[tri[3 * t]], iperm[tri[3 * t + 1]], iperm[tri[3 * t + 2]]};
        int64_t ts[3];
        int c = tiles_of(w, 3, ts);
        for (int a = 0; a < c; ++a) {
            int64_t e = fill[ts[a]]++;
            T.etri[e] = t;
            T.ev[e] = w[0];
            T.ev[T.nelem + e] = w[1];
            T.ev[2 * T.nelem + e] = w[2];
        }
    }
    // geometric flux coefficients g[e][v] = -l_e (s_v n_ex + s_{3+v} n_ey), v = 0, 1 in the
    // difference basis (u_v - u_2): Q_e = D_e (g[e][0] (u0 - u2) + g[e][1] (u1 - u2))
    std::vector<double> g(6 * T.nelem);
    for (int64_t e = 0; e < T.nelem; ++e) {
        const double* pr = &props[24 * (size_t)T.etri[e]];
        for (int d = 0; d < 3; ++d) {
            double nx = pr[15 + 2 * d], ny = pr[16 + 2 * d], l = pr[21 + d];
            for (int v = 0; v < 2; ++v) g[(2 * d + v) * T.nelem + e] = -l * (pr[v] * nx + pr[3 + v] * ny);
        }
    }
    // boundary edges
    std::vector<int64_t> bcnt(T.ntiles + 1, 0);
    for (int64_t e = 0; e < nbe; ++e) {
        int32_t w[2] = {iperm[be[2 * e]], iperm[be[2 * e + 1]]};
        int64_t ts[2];
        int c = tiles_of(w, 2, ts);
        for (int a = 0; a < c; ++a) bcnt[ts[a]]++;
    }
    T.boff.assign(T.ntiles + 1, 0);
    for (int64_t t = 0; t < T.ntiles; ++t) T.boff[t + 1] = T.boff[t] + bcnt[t];
    T.nbelem = T.boff[T.ntiles];
    T.ebedge.assign(T.nbelem, 0);
    T.bv.assign(3 * T.nbelem, 0);
    std::vector<double> bg(3 * std::max<int64_t>(T.nbelem, 1));
    std::vector<int64_t> bfill(T.boff.begin(), T.boff.end() - 1);
    for (int64_t e = 0; e < nbe; ++e) {
        int32_t i = be[2 * e], j = be[2 * e + 1], k = badj[e];
        int32_t w[2] = {iperm[i], iperm[j]};
        int64_t ts[2];
        int c = tiles_of(w, 2, ts);
        // G = -l_h (alpha nx + beta ny) in the basis (u_i - u_k), (u_j - u_k)
        double px = pts[2 * i], py = pts[2 * i + 1], qx = pts[2 * j], qy = pts[2 * j + 1];
        double lij = std::sqrt((qx - px) * (qx - px) + (qy - py) * (qy - py));
        double nx = (qy - py) / lij, ny = -(qx - px) / lij;
        double mijx = (px + qx) / 2, mijy = (py + qy) / 2;
        double lh = std::sqrt((mijx - px) * (mijx - px) + (mijy - py) * (mijy - py));
        const double* pr = &props[24 * (size_t)btri[e]];
        int32_t tv[3] = {tri[3 * btri[e]], tri[3 * btri[e] + 1], tri[3 * btri[e] + 2]};
        double gi = 0, gj = 0;
        for (int v = 0; v < 3; ++v) {
            double c0 = -lh * (pr[v] * nx + pr[3 + v] * ny);
            if (tv[v] == i) gi = c0;
            if (tv[v] == j) gj = c0;
        }
        for (int a = 0; a < c; ++a) {
            int64_t q = bfill[ts[a]]++;
            T.ebedge[q] = (int32_t)e;
            T.bv[q] = iperm[i];
            T.bv[T.nbelem + q] = iperm[j];
            T.bv[2 * T.nbelem + q] = iperm[k];
            bg[q] = gi;
            bg[T.nbelem + q] = gj;
            bg[2 * T.nbelem + q] = lh;
        }
    }
    T.d_off.upload(T.off);
    T.d_boff.upload(T.boff);
    T.d_ev.upload(T.ev);
    T.d_bv.upload(T.bv);
    T.d_g.upload(g);
    bg.resize(3 * T.nbelem);
    T.d_bg.upload(bg);
    T.built = true;
}
