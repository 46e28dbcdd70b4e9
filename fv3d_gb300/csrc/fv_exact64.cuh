// fv_exact64.cuh -- FP64 building blocks that round exactly like the plain
// IEEE operations they replace, with fewer FP64-pipe instructions.
//
// On GB300 the FP64 pipe executes about 1/73 of the FP32 rate, so the plain
// FP64 path is bound by its count of FP64 instructions.  Every helper here
// returns bit-for-bit the value of the reference expression it stands for
// (for finite operands away from the subnormal range), so the FP64 stage
// kernel stays bit-identical to the reference's CPU arithmetic.
//
// Division by a value whose correctly rounded reciprocal is known uses
// Markstein's correction (P. Markstein, "Computation of elementary functions
// on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; see
// also Muller et al., Handbook of Floating-Point Arithmetic, the theorem on
// correcting a quotient with a fused multiply-add): with y = RN(1/b) and
// q0 = RN(a*y), which lies within one ulp of a/b, the residual
// r = a - b*q0 is exactly representable (one fma) and RN(q0 + r*y) = RN(a/b).
#pragma once

#include <cuda_runtime.h>

namespace fv {

// RN(a / b) given y = RN(1 / b): one multiply and two fused operations
// instead of a full IEEE division.
__device__ __forceinline__ double div_by_rcp(double a, double b, double y) {
  const double q0 = __dmul_rn(a, y);
  const double r = fma(-b, q0, a);
  return fma(r, y, q0);
}

// (x) / d for a cell size d: an exact multiplication by 1/d when d is a power
// of two (then 1/d is exact and scaling by it rounds nowhere), else the
// corrected quotient above (exact for any d).  P2 is a compile-time choice:
// the kernels branch once, uniformly, on "every cell size is a power of two",
// because a per-call select would issue both forms.
template <bool P2>
__device__ __forceinline__ double div_cell(double x, double d, double inv_d) {
  return P2 ? __dmul_rn(x, inv_d) : div_by_rcp(x, d, inv_d);
}

// The reference formula of minmod, out of line: the rare operands that reach
// it (NaN, infinities, a product that may underflow) take a real branch, so
// its FP64 instructions are not issued on the common path.
static __device__ __noinline__ double minmod_rare(double dL, double dR) {
  if (dL * dR < 0.0) return 0.0;
  return fabs(dL) < fabs(dR) ? dL : dR;
}

// minmod of Update.h:73-80 -- 0 if dL*dR < 0, else the argument of smaller
// magnitude, ties to dR -- decided on the bit patterns without FP64
// instructions.  The sign test equals `dL*dR < 0` whenever the product cannot
// underflow to zero (exponent sum check) and neither operand is NaN; the
// magnitude test equals `fabs(dL) < fabs(dR)` because IEEE magnitudes order
// like their bit patterns.  The remaining cases take the reference formula.
__device__ __forceinline__ double minmod_exact(double dL, double dR) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(dL);
  const unsigned long long b = (unsigned long long)__double_as_longlong(dR);
  const unsigned long long ma = a & 0x7fffffffffffffffull, mb = b & 0x7fffffffffffffffull;
  const unsigned long long kInf = 0x7ff0000000000000ull;
  if (ma <= kInf && mb <= kInf) {
    if (ma == 0ull || mb == 0ull || ((a ^ b) >> 63) == 0ull) return ma < mb ? dL : dR;
    const unsigned ea = (unsigned)(ma >> 52), eb = (unsigned)(mb >> 52);
    if (ea != 0u && eb != 0u && ea + eb >= 972u) return 0.0;  // |dL*dR| >= 2^-1074
  }
  return minmod_rare(dL, dR);
}

// Comparisons and C99 fmin / fmax on bit patterns (integer pipe; the FP64
// pipe's DSETP / DMNMX issue at the FP64 rate).  For non-NaN operands each
// returns what the FP64 instruction returns -- min / max give one operand
// exactly; where the two operands are +0 and -0 the sign of the zero chosen
// may differ, which none of the callers can observe (their results do not
// depend on the sign of a zero speed or of a zero compared with zero).  A
// NaN operand is handled as fmin / fmax and the IEEE comparisons do.
__device__ __forceinline__ bool is_nan_bits(long long b) { return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }

// Signed-integer key that orders like the double (negative values reversed).
__device__ __forceinline__ long long order_key(long long b) { return b ^ ((b >> 63) & 0x7fffffffffffffffLL); }

__device__ __forceinline__ double fmin_bits(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  if (is_nan_bits(x)) return b;
  if (is_nan_bits(y)) return a;
  return order_key(y) < order_key(x) ? b : a;
}

__device__ __forceinline__ double fmax_bits(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  if (is_nan_bits(x)) return b;
  if (is_nan_bits(y)) return a;
  return order_key(y) > order_key(x) ? b : a;
}

// x >= 0.0, x > 0.0 and x <= 0.0 as IEEE comparisons (false for NaN).
__device__ __forceinline__ bool ge0_bits(double v) {
  const long long b = __double_as_longlong(v);
  return (b >= 0 && b <= 0x7ff0000000000000LL) || b == (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool gt0_bits(double v) {
  const long long b = __double_as_longlong(v);
  return b > 0 && b <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool le0_bits(double v) {
  const long long b = __double_as_longlong(v);
  return b == 0 || (b < 0 && !is_nan_bits(b));
}

// !(v <= limit) for a limit > 0 and a v that is >= 0 or NaN (a CFL sum).
__device__ __forceinline__ bool above_bits(double v, double limit) {
  const long long b = __double_as_longlong(v);
  return !(b >= 0 && b <= __double_as_longlong(limit));
}

// RN(0.5 * x) with integer instructions only.  For |x| >= 2^-1021 the
// product is exact: x with its exponent decremented (only the high word
// changes).  Below that the halved value is subnormal: the magnitude in units
// of 2^-1074 is halved with round-to-nearest-even.  Infinities and NaN are
// returned unchanged.
__device__ __forceinline__ double half64(double x) {
  const int hi = __double2hiint(x);
  const unsigned e = ((unsigned)hi >> 20) & 0x7ffu;
  if (e - 2u < 0x7fdu) return __hiloint2double(hi - 0x100000, __double2loint(x));
  if (e == 0x7ffu) return x;
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long m = b & 0x7fffffffffffffffull;
  const unsigned long long r = (m >> 1) + (m & (m >> 1) & 1ull);
  return __longlong_as_double((long long)((b & 0x8000000000000000ull) | r));
}

// 0.5 * x for either precision (FP32 keeps its multiply: that pipe is fast).
__device__ __forceinline__ double half_of(double x) { return half64(x); }
__device__ __forceinline__ float half_of(float x) { return 0.5f * x; }

// Face-state reconstruction q + (slope*sign)*0.5 (Update.h:21): the product
// with +-0.5 is exact, so a single fused operation rounds identically.
__device__ __forceinline__ double recon_plus(double q, double slope) { return fma(slope, 0.5, q); }
__device__ __forceinline__ double recon_minus(double q, double slope) { return fma(slope, -0.5, q); }

// Constants every FP64 kernel needs, computed on the host with IEEE double
// arithmetic exactly as the reference evaluates them.
struct Consts64 {
  double gamma;     // gamma0
  double gm1;       // gamma0 - 1 (exact for 1 < gamma0 < 3)
  double inv_gm1;   // RN(1 / (gamma0 - 1)), also HLLC's `entho`
};

}  // namespace fv
