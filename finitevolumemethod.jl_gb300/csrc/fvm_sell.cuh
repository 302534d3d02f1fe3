// Sliced-ELL row product shared by the RHS, template and Krylov kernels.
//
// One warp per 32-row slice, one lane per row; slots are column-major within the slice so
// each slot step of a warp reads 32 consecutive columns and values (coalesced).  For a
// compile-time maximum width MAXW the slot loop is fully unrolled: every column and value
// load of the row is issued first, then every gather of x, then the FMA chain, so a warp
// waits for one DRAM round trip and one L2 round trip instead of one per slot.  MAXW = 0
// keeps a rolled loop for very wide rows.
#pragma once
#include <cstdint>

namespace fvm {

// sum_k val[k] * x[col[k]]                 (DIFF = false)
// sum_k val[k] * (x[col[k]] - xr)          (DIFF = true)
template <class V, class T, class X, bool DIFF, int MAXW>
__device__ __forceinline__ T sell_row_product(const int64_t* __restrict__ slice_ptr, const int32_t* __restrict__ width,
                                              const int32_t* __restrict__ col, const V* __restrict__ val,
                                              const X* __restrict__ x, T xr, int64_t s, int lane) {
    const int64_t base = __ldg(&slice_ptr[s]) + lane;
    const int w = __ldg(&width[s]);
    T acc = 0;
    if constexpr (MAXW > 0) {
        int32_t c[MAXW];
        V v[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) {
                c[k] = __ldg(&col[base + (int64_t)k * 32]);
                v[k] = __ldg(&val[base + (int64_t)k * 32]);
            }
        T xs[MAXW];
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) xs[k] = (T)__ldg(&x[c[k]]);
#pragma unroll
        for (int k = 0; k < MAXW; ++k)
            if (k < w) {
                if constexpr (DIFF)
                    acc += (T)v[k] * (xs[k] - xr);
                else
                    acc += (T)v[k] * xs[k];
            }
    } else {
        for (int k = 0; k < w; ++k) {
            int64_t i = base + (int64_t)k * 32;
            T xv = (T)__ldg(&x[__ldg(&col[i])]);
            if constexpr (DIFF)
                acc += (T)__ldg(&val[i]) * (xv - xr);
            else
                acc += (T)__ldg(&val[i]) * xv;
        }
    }
    return acc;
}

// compile-time width bucket for a pattern whose widest slice has `maxw` slots
inline int sell_bucket(int maxw) { return maxw <= 4 ? 4 : maxw <= 8 ? 8 : maxw <= 12 ? 12 : maxw <= 16 ? 16 : 0; }

}  // namespace fvm

// Expands CALL(MAXW) for the bucket of `maxw`.
#define FVM_SELL_DISPATCH(maxw, CALL)          \
    switch (::fvm::sell_bucket(maxw)) {        \
        case 4: CALL(4); break;                \
        case 8: CALL(8); break;                \
        case 12: CALL(12); break;              \
        case 16: CALL(16); break;              \
        default: CALL(0); break;               \
    }
