// Element plumbing shared by the RPA kernels: grouped-index mapping of the
// particle-hole vertex (rpa.cpp:40,54-55) and the same operations on an FP64
// (double2) or double-float (cdf) complex element.
#pragma once

#include "common.cuh"

namespace tprf {

template <int NB>
__device__ __forceinline__ int colmap(int c) {  // grouped column (d, c') -> offset c' * nb + d
  return (c % NB) * NB + c / NB;
}

// element-type plumbing: double2 (FP64) or cdf (double-float)
__device__ __forceinline__ double2 el_from(double2 z, double2 *) { return z; }
__device__ __forceinline__ cdf el_from(double2 z, cdf *) { return to_cdf(z); }
__device__ __forceinline__ double2 el_to(double2 z) { return z; }
// the solves' outputs: one FP64 addition per part (the FP64 pipe is otherwise
// nearly idle in the RPA kernels, and the bit-operation conversion took a tenth
// of the pair kernel's time)
__device__ __forceinline__ double2 el_to(cdf z) { return make_double2(to_double_add(z.x), to_double_add(z.y)); }
__device__ __forceinline__ double2 el_one(double2 *) { return make_double2(1.0, 0.0); }
__device__ __forceinline__ cdf el_one(cdf *) { return cdf{dfl{1.f, 0.f}, dfl{0.f, 0.f}}; }
__device__ __forceinline__ double2 el_zero(double2 *) { return make_double2(0.0, 0.0); }
__device__ __forceinline__ cdf el_zero(cdf *) { return cdf{dfl{0.f, 0.f}, dfl{0.f, 0.f}}; }
__device__ __forceinline__ double el_abs2(double2 z) { return cabs2(z); }
__device__ __forceinline__ double el_abs2(cdf z) { return (double)(z.x.hi * z.x.hi + z.y.hi * z.y.hi); }
__device__ __forceinline__ float el_absf(double2 z) { return (float)sqrt(cabs2(z)); }
__device__ __forceinline__ float el_absf(cdf z) { return sqrtf(z.x.hi * z.x.hi + z.y.hi * z.y.hi); }
template <class E> struct IsDf { static constexpr bool value = false; };
template <> struct IsDf<cdf> { static constexpr bool value = true; };
__device__ __forceinline__ double2 el_fms(double2 a, double2 b, double2 acc) { return cfms(a, b, acc); }
__device__ __forceinline__ cdf el_fms(cdf a, cdf b, cdf acc) { return cfms_df(a, b, acc); }
// the elimination's updates: unnormalised double-float (cfms_df_lazy), with
// el_norm before a value is read by a product, a magnitude or a conversion
__device__ __forceinline__ double2 el_fms_lazy(double2 a, double2 b, double2 acc) { return cfms(a, b, acc); }
__device__ __forceinline__ cdf el_fms_lazy(cdf a, cdf b, cdf acc) { return cfms_df_lazy(a, b, acc); }
__device__ __forceinline__ double2 el_norm(double2 a) { return a; }
__device__ __forceinline__ cdf el_norm(cdf a) { return cnorm(a); }
__device__ __forceinline__ double2 el_recip(double2 a) { return crecip(a); }
__device__ __forceinline__ cdf el_recip(cdf a) {
  // 1/(x + iy) = (x - iy) / (x^2 + y^2); the real reciprocal by one Newton step from the float one
  const dfl d = ddot_add(a.x, a.x, a.y, a.y);
  const float r0 = __frcp_rn(d.hi);
  const dfl e = dsub(dfl{1.f, 0.f}, dmul(d, dfl{r0, 0.f}));
  const dfl r = dadd(dfl{r0, 0.f}, dmul(dfl{r0, 0.f}, e));
  return cdf{dmul(a.x, r), dneg(dmul(a.y, r))};
}


// Squared conditioning estimate above which a double-float solution is
// recomputed in FP64: (max|A| / min pivot)^2 > 1e4, i.e. the estimate > 100.
// Double-float carries ~2^-48 per operation, so below it the solve stays well
// inside 1e-10 relative; near an RPA instability (1 - chi0 U nearly singular)
// the point is solved in FP64.
constexpr double kDf64CondLimit2 = 1e4;

}  // namespace tprf
