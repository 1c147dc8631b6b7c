// gfe_sell.cuh -- the row of a sliced-ELL matrix (32-row slices, column-major inside a
// slice): the SpMV building block of the CG solvers (gfe_solve.cu) and of the p-multigrid
// smoother (gfe_pmg.cu). Included inside namespace gfe.
#pragma once

// y = A x on the sliced-ELL copy; thread per row, FMA chain in the accumulation type of TV.
// `load(c)` gives x at column c (a plain load, or a value formed on the fly).
template <typename TV, class Load>
__device__ __forceinline__ TV sell_row_f(int64_t r, const int64_t* __restrict__ sptr,
                                         const int32_t* __restrict__ scol,
                                         const TV* __restrict__ sval, const Load& load) {
  const int64_t s = r >> 5;
  const int l = (int)(r & 31);
  const int64_t base = __ldg(sptr + s) + l;
  const int32_t w = (int32_t)((__ldg(sptr + s + 1) - __ldg(sptr + s)) >> 5);
  TV acc = (TV)0;
  int32_t k = 0;
  for (; k + 4 <= w; k += 4) {
    const int64_t i = base + (int64_t)k * 32;
    const int32_t c0 = __ldcs(scol + i), c1 = __ldcs(scol + i + 32), c2 = __ldcs(scol + i + 64),
                  c3 = __ldcs(scol + i + 96);
    const TV v0 = __ldcs(sval + i), v1 = __ldcs(sval + i + 32), v2 = __ldcs(sval + i + 64),
             v3 = __ldcs(sval + i + 96);
    acc = fma(v0, (TV)load(c0), acc);
    acc = fma(v1, (TV)load(c1), acc);
    acc = fma(v2, (TV)load(c2), acc);
    acc = fma(v3, (TV)load(c3), acc);
  }
  for (; k < w; ++k) {
    const int64_t i = base + (int64_t)k * 32;
    acc = fma(__ldcs(sval + i), (TV)load(__ldcs(scol + i)), acc);
  }
  return acc;
}

template <typename TV, typename TX>
__device__ __forceinline__ TV sell_row(int64_t r, const int64_t* __restrict__ sptr,
                                       const int32_t* __restrict__ scol,
                                       const TV* __restrict__ sval, const TX* __restrict__ x) {
  return sell_row_f(r, sptr, scol, sval, [x](int32_t c) { return __ldg(x + c); });
}
