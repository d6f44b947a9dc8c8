// Device physics for the RK4 residual path.
//
// Every function is templated on the arithmetic type R of the flux, gradient
// and limiter work: R = double is the plain form and keeps, expression by
// expression, the operand order of the reference functors so that (built with
// --fmad=false) results are bit-identical to the reference's serial run;
// R = float is the mixed form's fast path.
//
//   primitives           kokkos/GasModel.h:69-90
//   roe_flux             kokkos/Roe_Flux.h:50-265
//   viscous_flux         kokkos/Viscous_Flux.h:66-98, GasModel.h:92-106
//   venkat / vanalbada   kokkos/VenkatLimiter.h:45-73, VanAlbadaLimiter.h:45-65
//   reflect_state        kokkos/Tangent_BC.h:86-102, NoSlip_BC.h:93-109
#pragma once
#include <cuda_runtime.h>
#include <cfloat>
#include <cstdint>
#include <type_traits>

namespace miniaero {
namespace dev {

template <class R> __device__ __forceinline__ R dsqrt(R x);
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <class R> __device__ __forceinline__ R dabs(R x);
// |x| as the sign bit cleared on the integer pipe (fabs, for every input).
template <> __device__ __forceinline__ double dabs<double>(double x) {
  return __hiloint2double(__double2hiint(x) & 0x7FFFFFFF, __double2loint(x));
}
template <> __device__ __forceinline__ float dabs<float>(float x) { return fabsf(x); }

// a / b rounded to nearest, given y = RN(1/b) computed once per divisor.
// Method: q0 = RN(a*y) is within 1.5 ulp of a/b; one residual correction
// q1 = RN(q0 + RN(a - b*q0)*y) is faithful (error <= 1/2 ulp + O(2^-104));
// by Markstein's theorem (y correctly rounded, q1 faithful, binary64, no
// underflow or overflow) RN(q1 + (a - b*q1)*y) is the correctly rounded
// quotient. 1 multiply + 4 FMAs instead of a full division. The residuals
// a - b*q are exact only while their lowest bit, about ulp(b)*ulp(q), is not
// below the subnormal spacing, and the argument wants a normal RN(1/b): when
// the exponents of q and b add up to less than -960 (quotients near or in the
// subnormal range), q is not finite, or b is subnormal or >= 2^1022, the IEEE
// division is taken instead (rare; integer tests decide). A zero numerator
// returns a*y, which already is the IEEE zero quotient with its sign.
__device__ __forceinline__ double div_by_recip(double a, double b, double y) {
  double q = a * y;
  const uint32_t eq = (static_cast<uint32_t>(__double2hiint(q)) >> 20) & 0x7FFu;
  const uint32_t eb = (static_cast<uint32_t>(__double2hiint(b)) >> 20) & 0x7FFu;
  if (eq + eb < 1086u || eq == 0x7FFu || eb - 1u > 2043u) {
    const uint32_t ah = static_cast<uint32_t>(__double2hiint(a)) & 0x7FFFFFFFu;
    if ((ah | static_cast<uint32_t>(__double2loint(a))) == 0u) return q;
    return a / b;
  }
  double r = fma(-q, b, a);
  q = fma(r, y, q);
  r = fma(-q, b, a);
  return fma(r, y, q);
}
__device__ __forceinline__ float div_by_recip(float a, float /*b*/, float y) { return a * y; }

// Exact FP64 identities taken off the FP64 pipe, which bounds the plain form
// on GB300 (2 FP64 lanes per SM per clock): the integer ALU gives the same
// bits in a few instructions.
//
// halve(x) = 0.5 * x: for a normal x above the smallest binade the exponent
// field steps down by one (the product is exact). Below it (zeros, subnormals,
// the smallest binade) the pattern is the value in units of 2^-1074, so the
// result is that integer halved, ties to even; infinities and NaNs return
// themselves. No FP64 instruction on any path (a multiply in a rarely taken
// branch would still issue once the compiler predicates the branch).
__device__ __forceinline__ double halve(double x) {
  const uint32_t hi = static_cast<uint32_t>(__double2hiint(x));
  const uint32_t e = (hi >> 20) & 0x7FFu;
  if (e - 2u < 2045u) return __hiloint2double(static_cast<int>(hi - 0x100000u), __double2loint(x));
  if (e == 0x7FFu) return x;
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long sign = b & 0x8000000000000000ull, m = b ^ sign;
  return __longlong_as_double(static_cast<long long>(sign | ((m >> 1) + (m & (m >> 1) & 1ull))));
}
__device__ __forceinline__ float halve(float x) { return 0.5f * x; }
// twice(x) = 2 * x: the exponent field steps up by one while the result
// stays finite (biased exponent 1..2045); from the top binade it overflows to
// infinity; a zero or subnormal pattern doubles as an integer (exact, and it
// carries into the exponent field as the value turns normal); infinities and
// NaNs return themselves. Integer instructions only.
__device__ __forceinline__ double twice(double x) {
  const uint32_t hi = static_cast<uint32_t>(__double2hiint(x));
  const uint32_t e = (hi >> 20) & 0x7FFu;
  if (e - 1u < 2045u) return __hiloint2double(static_cast<int>(hi + 0x100000u), __double2loint(x));
  if (e == 0x7FFu) return x;
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const unsigned long long sign = b & 0x8000000000000000ull, m = b ^ sign;
  return __longlong_as_double(static_cast<long long>(sign | (e == 0u ? (m << 1) : 0x7FF0000000000000ull)));
}
__device__ __forceinline__ float twice(float x) { return 2.0f * x; }
// zero_plus(x) = 0 + x in round to nearest: x itself, except that -0 becomes
// +0 (a sum that starts at +0 and adds x). A NaN stays a NaN.
__device__ __forceinline__ double zero_plus(double x) {
  const uint32_t hi = static_cast<uint32_t>(__double2hiint(x));
  const bool negzero = (hi == 0x80000000u) & (__double2loint(x) == 0);
  return __hiloint2double(negzero ? 0 : static_cast<int>(hi), __double2loint(x));
}
__device__ __forceinline__ float zero_plus(float x) { return 0.0f + x; }
// a < b for an a with a clear sign bit (an absolute value): as signed 64-bit
// integers the patterns of non-negative doubles keep their order, and a
// negative b (sign bit set) is below every such a. Same result as the double
// compare for every b but a NaN.
__device__ __forceinline__ bool less_nonneg(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b);
}
__device__ __forceinline__ bool less_nonneg(float a, float b) { return a < b; }

// Low-order part of the reciprocal: for y = RN(1/b) the residual 1 - b*y is
// exact (one FMA), and y + ylo with ylo = RN((1 - b*y) * y) is 1/b to about
// 2^-105 relative. For callers that divide many values by one b.
__device__ __forceinline__ double recip_lo(double b, double y) { return fma(-b, y, 1.0) * y; }
__device__ __forceinline__ float recip_lo(float /*b*/, float /*y*/) { return 0.0f; }

// a / b for hot loops that divide many values by one b, with the IEEE
// fallback left to the caller. With the two-part reciprocal y + ylo,
// q1 = RN(a*y + RN(a*ylo)) is within 2^-104 relative of a/b before its
// rounding, hence faithful, so Markstein's correction RN(q1 + (a - b*q1)*y)
// alone gives the correctly rounded quotient: one multiply and three FMAs
// (div_by_recip takes one and four). `inexact` is set under div_by_recip's
// range conditions, where the result may differ from a/b; zero numerators
// are excluded: their quotient is a zero of either sign, and the callers only
// add it to sums that start at +0, where the sign of a zero never shows.
__device__ __forceinline__ double div_by_recip2_flag(double a, double b, double y, double ylo, bool& inexact) {
  const double q = fma(a, y, a * ylo);
  const uint32_t eq = (static_cast<uint32_t>(__double2hiint(q)) >> 20) & 0x7FFu;
  const uint32_t eb = (static_cast<uint32_t>(__double2hiint(b)) >> 20) & 0x7FFu;
  const uint32_t ah = static_cast<uint32_t>(__double2hiint(a)) & 0x7FFFFFFFu;
  const bool range = (eq + eb < 1086u) | (eq == 0x7FFu) | (eb - 1u > 2043u);
  inexact |= range & ((ah | static_cast<uint32_t>(__double2loint(a))) != 0u);
  return fma(fma(-q, b, a), y, q);
}
__device__ __forceinline__ float div_by_recip2_flag(float a, float /*b*/, float y, float /*ylo*/, bool& /*inexact*/) {
  return a * y;
}

// float -> double by bit manipulation on the integer pipe (the FP64 pipe is
// the residual kernel's bottleneck): exact for normal floats, zeros, inf and
// NaN; FP32 subnormals (|x| < 1.2e-38) become signed zeros.
__device__ __forceinline__ double widen_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t sign = u & 0x80000000u;
  const uint32_t mant = u & 0x7FFFFFu;
  const uint32_t lo = mant << 29;
  const uint32_t hi_norm = sign | ((e + 896u) << 20) | (mant >> 3);
  const uint32_t hi_inf = sign | 0x7FF00000u | (mant >> 3);
  const uint32_t hi = (e == 0u) ? sign : (e == 0xFFu ? hi_inf : hi_norm);
  return __hiloint2double(static_cast<int>(hi), e == 0u ? 0 : static_cast<int>(lo));
}

// double -> float rounded to nearest even on the integer pipe (the hardware
// conversion issues on the FP64 pipe): bit-identical to the conversion for
// results in the normal float range and for zeros; the other inputs (float
// subnormals, overflow, inf, NaN) take the hardware conversion.
__device__ __forceinline__ float narrow_rn(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  const uint32_t hi = static_cast<uint32_t>(b >> 32), lo = static_cast<uint32_t>(b);
  const uint32_t E = (hi >> 20) & 0x7FFu;
  const uint32_t sign = hi & 0x80000000u;
  if (E >= 897u && E <= 1150u) {
    uint32_t r = sign | ((E - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1FFFFFFFu;
    if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) ++r;  // a carry into the exponent is right
    return __uint_as_float(r);
  }
  if ((hi & 0x7FFFFFFFu) == 0u && lo == 0u) return __uint_as_float(sign);
  return __double2float_rn(x);
}

// Sum of six FP32 values (bit patterns) as the exact sum rounded once to
// FP64: never less accurate than adding them in FP64 one after another, and
// done on the integer pipe. Each value's 24-bit significand is placed in a
// 64-bit fixed-point word 36 bits above the binade of the largest value
// (six such words stay below 2^63), the words are summed exactly, and the
// integer is converted once (round to nearest even) and scaled by a power of
// two, also on the integer pipe. Zeros and FP32 subnormals add nothing (the
// mixed form's widening also takes subnormals as zero). `exact` becomes false
// when a nonzero value lies more than 36 binades below the largest, or a value
// is infinite or NaN; the caller then adds in FP64.
__device__ __forceinline__ double exact_sum_f32(const uint32_t (&u)[6], bool& exact) {
  uint32_t emax = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i) emax = max(emax, (u[i] >> 23) & 0xFFu);
  bool ok = emax < 255u;
  long long acc = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const uint32_t e = (u[i] >> 23) & 0xFFu;
    const uint32_t d = emax - e;
    const bool live = e != 0u;
    const bool fits = d <= 36u;
    ok &= !live | fits;
    const long long m = static_cast<long long>((u[i] & 0x7FFFFFu) | 0x800000u);
    const long long a = (live & fits) ? (m << (36u - d)) : 0LL;
    acc += (u[i] >> 31) ? -a : a;
  }
  exact = ok;
  if (acc == 0) return 0.0;
  // Integer-pipe conversion: normalise |acc| to bit 63, round to 53 bits
  // (nearest even), assemble sign, exponent and fraction.
  const unsigned long long neg = acc < 0 ? 1ull : 0ull;
  const unsigned long long mag = neg ? static_cast<unsigned long long>(-acc) : static_cast<unsigned long long>(acc);
  const int lz = __clzll(static_cast<long long>(mag));
  const unsigned long long nrm = mag << lz;
  unsigned long long frac = nrm >> 11;                 // 53 bits with the leading one
  const unsigned long long rem = nrm & 0x7FFull;
  frac += (rem > 0x400ull || (rem == 0x400ull && (frac & 1ull))) ? 1ull : 0ull;
  // value = frac * 2^(63 - lz - 52) * 2^(emax - 186); frac may have carried to
  // 2^53, which the exponent addition below absorbs.
  const long long e = (1023LL + 63 - lz) + (static_cast<long long>(emax) - 186LL);
  const unsigned long long bits = (neg << 63) + (static_cast<unsigned long long>(e) << 52) + (frac - (1ull << 52));
  return __longlong_as_double(static_cast<long long>(bits));
}

// -x when neg, by flipping the sign bit on the integer pipe (IEEE negation).
__device__ __forceinline__ double negate_if(double x, bool neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ (static_cast<long long>(neg) << 63));
}

// Conserved -> primitive (rho, u, v, w, T); always FP64 (the state is FP64).
// T = e (gamma - 1) / Rgas is divided through the correctly rounded
// reciprocal of Rgas (div_by_recip: the IEEE quotient for finite values).
__device__ __forceinline__ void primitives(const double U[5], double V[5]) {
  const double gamma = 1.4;
  const double Rgas = 287.05;
  constexpr double kRgasInv = 1.0 / 287.05;
  const double r = U[0];
  const double ri = 1.0 / r;
  const double u = U[1] * ri;
  const double v = U[2] * ri;
  const double w = U[3] * ri;
  const double k = halve(u * u + v * v + w * w);
  const double e = U[4] * ri - k;
  const double T = div_by_recip(e * (gamma - 1.0), Rgas, kRgasInv);
  V[0] = r; V[1] = u; V[2] = v; V[3] = w; V[4] = T;
}

// Face frame precomputed once per mesh from the reference's own expressions:
// |n| = sqrt(n.n) and the three unit vectors n/|n|, t/|t|, b/|b|.
template <class R>
struct FaceFrame {
  R n[3];    // area vector
  R nu[3];   // unit normal
  R tu[3];   // unit tangent
  R bu[3];   // unit binormal
  R nn;      // |n|
};

// Roe approximate Riemann flux on primitive states.
template <class R>
__device__ __forceinline__ void roe_flux(const R pl[5], const R pr[5], const FaceFrame<R>& f, R flux[5]) {
  const R efix_u = R(0.1), efix_c = R(0.1), gm1 = R(0.4);
  const R* n = f.n;
  const R rl = pl[0], ul = pl[1], vl = pl[2], wl = pl[3];
  const R p_l = rl * R(287.05) * pl[4];
  const R h_l = R(1004.0) * pl[4];
  const R H_l = h_l + halve(ul * ul + vl * vl + wl * wl);
  const R mf_l = rl * (n[0] * ul + n[1] * vl + n[2] * wl);
  const R rr = pr[0], ur = pr[1], vr = pr[2], wr = pr[3];
  const R p_r = rr * R(287.05) * pr[4];
  const R h_r = R(1004.0) * pr[4];
  const R H_r = h_r + halve(ur * ur + vr * vr + wr * wr);
  const R mf_r = rr * (n[0] * ur + n[1] * vr + n[2] * wr);
  const R psum = p_l + p_r;

  flux[0] = halve(mf_l + mf_r);
  flux[1] = halve(mf_l * ul + mf_r * ur + n[0] * psum);
  flux[2] = halve(mf_l * vl + mf_r * vr + n[1] * psum);
  flux[3] = halve(mf_l * wl + mf_r * wr + n[2] * psum);
  flux[4] = halve(mf_l * H_l + mf_r * H_r);

  const R* nu = f.nu;
  const R* tu = f.tu;
  const R* bu = f.bu;
  const R srl = dsqrt<R>(rl);
  const R denom = R(1.0) / (srl + dsqrt<R>(rr));
  const R alpha = srl * denom;
  const R beta = R(1.0) - alpha;
  const R uroe = alpha * ul + beta * ur;
  const R vroe = alpha * vl + beta * vr;
  const R wroe = alpha * wl + beta * wr;
  const R hroe = alpha * h_l + beta * h_r +
                 halve(alpha) * beta *
                     ((ur - ul) * (ur - ul) + (vr - vl) * (vr - vl) + (wr - wl) * (wr - wl));
  const R c = dsqrt<R>(gm1 * hroe);

  const R nv = uroe * nu[0] + vroe * nu[1] + wroe * nu[2];
  const R tv = uroe * tu[0] + vroe * tu[1] + wroe * tu[2];
  const R bv = uroe * bu[0] + vroe * bu[1] + wroe * bu[2];
  const R ke = halve(uroe * uroe + vroe * vroe + wroe * wroe);
  const R cssi = R(1.0) / (c * c);
  const R hcssi = halve(cssi);

  R dq[5];
  dq[0] = rr - rl;
  dq[1] = rr * ur - rl * ul;
  dq[2] = rr * vr - rl * vl;
  dq[3] = rr * wr - rl * wl;
  dq[4] = (rr * H_r - p_r) - (rl * H_l - p_l);

  const R cbar = c * f.nn;
  const R ubar = uroe * n[0] + vroe * n[1] + wroe * n[2];
  const R cfl = dabs<R>(ubar) + cbar;
  const R eig1 = ubar + cbar, eig2 = ubar - cbar, eig3 = ubar;
  R a1 = dabs<R>(eig1), a2 = dabs<R>(eig2), a3 = dabs<R>(eig3);
  const R epuc = efix_u * cfl, epcc = efix_c * cfl;
  if (less_nonneg(a1, epcc)) a1 = halve(eig1 * eig1 + epcc * epcc) / epcc;
  if (less_nonneg(a2, epcc)) a2 = halve(eig2 * eig2 + epcc * epcc) / epcc;
  if (less_nonneg(a3, epuc)) a3 = halve(eig3 * eig3 + epuc * epuc) / epuc;
  // |lambda| per characteristic: eigp - eigm of the reference.
  const R ep1 = halve(eig1 + a1), em1 = halve(eig1 - a1);
  const R ep2 = halve(eig2 + a2), em2 = halve(eig2 - a2);
  const R ep3 = halve(eig3 + a3), em3 = halve(eig3 - a3);
  const R lam[5] = {ep1 - em1, ep2 - em2, ep3 - em3, ep3 - em3, ep3 - em3};

  // Left eigenvector rows times the conserved jump (MatVec5 with beta = 0).
  const R gk = gm1 * (ke - hroe);
  R L[5][5] = {
      {gk + c * (c - nv), c * nu[0] - gm1 * uroe, c * nu[1] - gm1 * vroe, c * nu[2] - gm1 * wroe, gm1},
      {gk + c * (c + nv), -c * nu[0] - gm1 * uroe, -c * nu[1] - gm1 * vroe, -c * nu[2] - gm1 * wroe, gm1},
      {ke - hroe, -uroe, -vroe, -wroe, R(1.0)},
      {-tv, tu[0], tu[1], tu[2], R(0.0)},
      {-bv, bu[0], bu[1], bu[2], R(0.0)}};
  R ldq[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    R acc = zero_plus(L[i][0] * dq[0]);  // a sum from +0
#pragma unroll
    for (int j = 1; j < 5; ++j) acc += L[i][j] * dq[j];
    ldq[i] = lam[i] * acc;
  }
  const R hk = hroe + ke;
  R M[5][5] = {
      {hcssi, hcssi, -gm1 * cssi, R(0.0), R(0.0)},
      {(uroe + nu[0] * c) * hcssi, (uroe - nu[0] * c) * hcssi, -gm1 * uroe * cssi, tu[0], bu[0]},
      {(vroe + nu[1] * c) * hcssi, (vroe - nu[1] * c) * hcssi, -gm1 * vroe * cssi, tu[1], bu[1]},
      {(wroe + nu[2] * c) * hcssi, (wroe - nu[2] * c) * hcssi, -gm1 * wroe * cssi, tu[2], bu[2]},
      {(hk + c * nv) * hcssi, (hk - c * nv) * hcssi, (c * c - gm1 * hk) * cssi, tv, bv}};
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    R acc = zero_plus(M[i][0] * ldq[0]);  // a sum from +0
#pragma unroll
    for (int j = 1; j < 5; ++j) acc += M[i][j] * ldq[j];
    flux[i] -= halve(acc);
  }
}

// Roe flux on an axis-aligned face: the area vector and unit normal are
// nonzero only along axis D, the unit tangent only along T = (D+2)%3 and the
// unit binormal only along B = (D+1)%3 (the frame the mesh builds for such a
// face; the host checks the zero pattern). Every product with one of the
// exactly-zero components is a signed zero; the terms left are evaluated in
// the reference's order, so every nonzero intermediate equals roe_flux's. A
// zero intermediate may differ in sign only; none reaches a division, a
// square root or a comparison that could tell.
// The mixed form's Roe flux on an axis-aligned face (FP32; the mixed form
// keeps no reference bits). Same central flux, Roe averages and entropy fix
// as roe_flux_axis, with a*b+c written as fused multiply-adds (explicit
// fmaf: the same bits in every kernel that inlines it, so batch and single
// runs agree), and the dissipation |A| dU evaluated as its acoustic, entropy
// and shear waves instead of the two eigenvector products. The wave
// strengths come from the conserved jumps dq with the reference's gm1 = 0.4,
// as its left eigenvectors take them (its gas has cp 1004 and R 287.05, so a
// strength built on the jump of p = rho R T would be a different scheme):
// with P = gm1 (dq4 - v~.dqm + ke dq0) and mn = n.dqm - u~n dq0 the rows give
// L0.dq = P + c mn, L1.dq = P - c mn, L2.dq = P/gm1 - hroe dq0, L3.dq =
// tu (dqm_T - v~_T dq0) and L4.dq = bu (dqm_B - v~_B dq0), and the right
// eigenvectors (with c^2 = gm1 hroe) turn them into the waves below.
template <int D>
__device__ __forceinline__ void roe_flux_axis_f32(const float pl[5], const float pr[5], float nD, float nuD,
                                                  float nn, float flux[5]) {
  constexpr int T = (D + 2) % 3, B = (D + 1) % 3;
  const float gm1 = 0.4f, efix = 0.1f;
  const float rl = pl[0], rr = pr[0];
  const float vl[3] = {pl[1], pl[2], pl[3]};
  const float vr[3] = {pr[1], pr[2], pr[3]};
  const float p_l = rl * 287.05f * pl[4], p_r = rr * 287.05f * pr[4];
  const float h_l = 1004.0f * pl[4], h_r = 1004.0f * pr[4];
  const float H_l = fmaf(0.5f, fmaf(vl[0], vl[0], fmaf(vl[1], vl[1], vl[2] * vl[2])), h_l);
  const float H_r = fmaf(0.5f, fmaf(vr[0], vr[0], fmaf(vr[1], vr[1], vr[2] * vr[2])), h_r);
  const float mf_l = rl * (nD * vl[D]), mf_r = rr * (nD * vr[D]);

  flux[0] = 0.5f * (mf_l + mf_r);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    float m = fmaf(mf_l, vl[j], mf_r * vr[j]);
    if (j == D) m = fmaf(nD, p_l + p_r, m);
    flux[1 + j] = 0.5f * m;
  }
  flux[4] = 0.5f * fmaf(mf_l, H_l, mf_r * H_r);

  const float srl = sqrtf(rl), srr = sqrtf(rr);
  const float alpha = srl / (srl + srr);
  const float beta = 1.0f - alpha;
  float vroe[3], dv[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    vroe[j] = fmaf(alpha, vl[j], beta * vr[j]);
    dv[j] = vr[j] - vl[j];
  }
  const float dv2 = fmaf(dv[0], dv[0], fmaf(dv[1], dv[1], dv[2] * dv[2]));
  const float hroe = fmaf(alpha, h_l, fmaf(beta, h_r, 0.5f * alpha * beta * dv2));
  const float c = sqrtf(gm1 * hroe);
  const float ke = 0.5f * fmaf(vroe[0], vroe[0], fmaf(vroe[1], vroe[1], vroe[2] * vroe[2]));
  const float cssi = 1.0f / (c * c);

  // Eigenvalues (with the face area) and the entropy fix of the reference.
  const float cbar = c * nn;
  const float ubar = vroe[D] * nD;
  const float cfl = fabsf(ubar) + cbar;
  const float eig1 = ubar + cbar, eig2 = ubar - cbar, eig3 = ubar;
  float a1 = fabsf(eig1), a2 = fabsf(eig2), a3 = fabsf(eig3);
  const float ep = efix * cfl;
  if (a1 < ep) a1 = 0.5f * fmaf(eig1, eig1, ep * ep) / ep;
  if (a2 < ep) a2 = 0.5f * fmaf(eig2, eig2, ep * ep) / ep;
  if (a3 < ep) a3 = 0.5f * fmaf(eig3, eig3, ep * ep) / ep;

  // Conserved jumps and wave strengths (a1: the u+c wave, a2: u-c, a3: u).
  const float dq0 = rr - rl;
  float dqm[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) dqm[j] = fmaf(rr, vr[j], -(rl * vl[j]));
  const float dq4 = fmaf(rr, H_r, -p_r) - fmaf(rl, H_l, -p_l);
  const float vdq = fmaf(vroe[0], dqm[0], fmaf(vroe[1], dqm[1], vroe[2] * dqm[2]));
  const float P = gm1 * fmaf(ke, dq0, dq4 - vdq);
  const float cmn = c * (fmaf(-vroe[D], dq0, dqm[D]) * nuD);
  const float h2 = 0.5f * cssi;
  const float w5 = a1 * ((P + cmn) * h2);
  const float w1 = a2 * ((P - cmn) * h2);
  const float w2 = a3 * fmaf(-P, cssi, dq0);
  const float sT = a3 * fmaf(-vroe[T], dq0, dqm[T]);
  const float sB = a3 * fmaf(-vroe[B], dq0, dqm[B]);
  const float wsum = w1 + w2 + w5;
  const float cun = c * (vroe[D] * nuD);
  const float hk = hroe + ke;
  float dis[5];
  dis[0] = wsum;
  dis[1 + D] = fmaf(wsum, vroe[D], (c * nuD) * (w5 - w1));
  dis[1 + T] = fmaf(wsum, vroe[T], sT);
  dis[1 + B] = fmaf(wsum, vroe[B], sB);
  dis[4] = fmaf(w1, hk - cun, fmaf(w5, hk + cun, fmaf(w2, ke, fmaf(vroe[T], sT, vroe[B] * sB))));
#pragma unroll
  for (int k = 0; k < 5; ++k) flux[k] = fmaf(-0.5f, dis[k], flux[k]);
}

template <class R, int D>
__device__ __forceinline__ void roe_flux_axis(const R pl[5], const R pr[5], R nD, R nuD, R tuT, R buB, R nn,
                                              R flux[5]) {
  if constexpr (std::is_same<R, float>::value) {
    roe_flux_axis_f32<D>(pl, pr, nD, nuD, nn, flux);
    return;
  }
  constexpr int T = (D + 2) % 3, B = (D + 1) % 3;
  const R efix_u = R(0.1), efix_c = R(0.1), gm1 = R(0.4);
  const R rl = pl[0];
  const R vel_l[3] = {pl[1], pl[2], pl[3]};
  const R p_l = rl * R(287.05) * pl[4];
  const R h_l = R(1004.0) * pl[4];
  const R H_l = h_l + halve(vel_l[0] * vel_l[0] + vel_l[1] * vel_l[1] + vel_l[2] * vel_l[2]);
  const R mf_l = rl * (nD * vel_l[D]);
  const R rr = pr[0];
  const R vel_r[3] = {pr[1], pr[2], pr[3]};
  const R p_r = rr * R(287.05) * pr[4];
  const R h_r = R(1004.0) * pr[4];
  const R H_r = h_r + halve(vel_r[0] * vel_r[0] + vel_r[1] * vel_r[1] + vel_r[2] * vel_r[2]);
  const R mf_r = rr * (nD * vel_r[D]);
  const R psum = p_l + p_r;

  flux[0] = halve(mf_l + mf_r);
#pragma unroll
  for (int j = 0; j < 3; ++j)
    flux[1 + j] = (j == D) ? halve(mf_l * vel_l[j] + mf_r * vel_r[j] + nD * psum)
                           : halve(mf_l * vel_l[j] + mf_r * vel_r[j]);
  flux[4] = halve(mf_l * H_l + mf_r * H_r);

  const R srl = dsqrt<R>(rl);
  const R denom = R(1.0) / (srl + dsqrt<R>(rr));
  const R alpha = srl * denom;
  const R beta = R(1.0) - alpha;
  R vroe[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) vroe[j] = alpha * vel_l[j] + beta * vel_r[j];
  const R hroe = alpha * h_l + beta * h_r +
                 halve(alpha) * beta *
                     ((vel_r[0] - vel_l[0]) * (vel_r[0] - vel_l[0]) + (vel_r[1] - vel_l[1]) * (vel_r[1] - vel_l[1]) +
                      (vel_r[2] - vel_l[2]) * (vel_r[2] - vel_l[2]));
  const R c = dsqrt<R>(gm1 * hroe);

  const R nv = vroe[D] * nuD;
  const R tv = vroe[T] * tuT;
  const R bv = vroe[B] * buB;
  const R ke = halve(vroe[0] * vroe[0] + vroe[1] * vroe[1] + vroe[2] * vroe[2]);
  const R cssi = R(1.0) / (c * c);
  const R hcssi = halve(cssi);

  R dq[5];
  dq[0] = rr - rl;
#pragma unroll
  for (int j = 0; j < 3; ++j) dq[1 + j] = rr * vel_r[j] - rl * vel_l[j];
  dq[4] = (rr * H_r - p_r) - (rl * H_l - p_l);

  const R cbar = c * nn;
  const R ubar = vroe[D] * nD;
  const R cfl = dabs<R>(ubar) + cbar;
  const R eig1 = ubar + cbar, eig2 = ubar - cbar, eig3 = ubar;
  R a1 = dabs<R>(eig1), a2 = dabs<R>(eig2), a3 = dabs<R>(eig3);
  const R epuc = efix_u * cfl, epcc = efix_c * cfl;
  if (less_nonneg(a1, epcc)) a1 = halve(eig1 * eig1 + epcc * epcc) / epcc;
  if (less_nonneg(a2, epcc)) a2 = halve(eig2 * eig2 + epcc * epcc) / epcc;
  if (less_nonneg(a3, epuc)) a3 = halve(eig3 * eig3 + epuc * epuc) / epuc;
  const R ep1 = halve(eig1 + a1), em1 = halve(eig1 - a1);
  const R ep2 = halve(eig2 + a2), em2 = halve(eig2 - a2);
  const R ep3 = halve(eig3 + a3), em3 = halve(eig3 - a3);
  const R lam[5] = {ep1 - em1, ep2 - em2, ep3 - em3, ep3 - em3, ep3 - em3};


  // Left eigenvectors: rows 0/1 hold c*nu_j - gm1*u_j (c*nu_j = +-0 off D),
  // rows 3/4 have a single nonzero tangent/binormal entry.
  const R gk = gm1 * (ke - hroe);
  R row0[5], row1[5];
  row0[0] = gk + c * (c - nv);
  row1[0] = gk + c * (c + nv);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    row0[1 + j] = (j == D) ? c * nuD - gm1 * vroe[j] : -(gm1 * vroe[j]);
    // (-c) nu_D is -(c nu_D) exactly (round to nearest is symmetric): one product for both rows.
    row1[1 + j] = (j == D) ? -(c * nuD) - gm1 * vroe[j] : -(gm1 * vroe[j]);
  }
  row0[4] = gm1;
  row1[4] = gm1;
  R ldq[5];
  {
    // Sums that start at +0: the first term is zero_plus (0 + x).
    R a0 = zero_plus(row0[0] * dq[0]), b0 = zero_plus(row1[0] * dq[0]);
#pragma unroll
    for (int j = 1; j < 5; ++j) {
      a0 += row0[j] * dq[j];
      b0 += row1[j] * dq[j];
    }
    R c0 = zero_plus((ke - hroe) * dq[0]);
    c0 += -vroe[0] * dq[1];
    c0 += -vroe[1] * dq[2];
    c0 += -vroe[2] * dq[3];
    c0 += R(1.0) * dq[4];
    R d0 = zero_plus(-tv * dq[0]);
    d0 += tuT * dq[1 + T];
    R e0 = zero_plus(-bv * dq[0]);
    e0 += buB * dq[1 + B];
    ldq[0] = lam[0] * a0;
    ldq[1] = lam[1] * b0;
    ldq[2] = lam[2] * c0;
    ldq[3] = lam[3] * d0;
    ldq[4] = lam[4] * e0;
  }
  // Right eigenvectors.
  const R hk = hroe + ke;
  {
    R acc = zero_plus(hcssi * ldq[0]);
    acc += hcssi * ldq[1];
    acc += -gm1 * cssi * ldq[2];
    flux[0] -= halve(acc);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    R acc;
    if (j == D) {
      acc = zero_plus((vroe[j] + nuD * c) * hcssi * ldq[0]);
      acc += (vroe[j] - nuD * c) * hcssi * ldq[1];
    } else {
      acc = zero_plus(vroe[j] * hcssi * ldq[0]);
      acc += vroe[j] * hcssi * ldq[1];
    }
    acc += -(gm1 * vroe[j]) * cssi * ldq[2];  // (-gm1) u_j, as the rows' product negated
    if (j == T) acc += tuT * ldq[3];
    if (j == B) acc += buB * ldq[4];
    flux[1 + j] -= halve(acc);
  }
  {
    R acc = zero_plus((hk + c * nv) * hcssi * ldq[0]);
    acc += (hk - c * nv) * hcssi * ldq[1];
    acc += (c * c - gm1 * hk) * cssi * ldq[2];
    acc += tv * ldq[3];
    acc += bv * ldq[4];
    flux[4] -= halve(acc);
  }
}

// Gas transport: Sutherland law (reference) or constant mu with given Prandtl.
struct Transport {
  int model;       // 0 Sutherland, 1 constant
  double mu;
  double prandtl;
  double k;        // constant model: mu * 1006 / prandtl, rounded as on the device
  float mu_f, k_f; // mu and k rounded to float on the host (no per-face conversion)
};

inline Transport make_transport(int model, double mu, double prandtl) {
  Transport t{model, mu, prandtl, 0.0, 0.0f, 0.0f};
  if (model == 1) t.k = mu * 1006.0 / prandtl;
  t.mu_f = static_cast<float>(t.mu);
  t.k_f = static_cast<float>(t.k);
  return t;
}

template <class R>
__device__ __forceinline__ void transport(const Transport& tr, R T, R& mu, R& k) {
  if (tr.model == 1) {
    if constexpr (std::is_same<R, float>::value) {
      mu = tr.mu_f;
      k = tr.k_f;
    } else {
      mu = tr.mu;
      k = tr.k;
    }
  } else {
    mu = R(1.458e-6) * T * dsqrt<R>(T) / (T + R(110.4));
    k = mu * R(1006.0) / R(0.71);
  }
}

// Newtonian stress and Fourier heat flux through area vector a.
template <class R>
__device__ __forceinline__ void viscous_flux(const R g[5][3], const R prim[5], const R a[3], const Transport& tr,
                                             R vflux[5]) {
  R mu, kc;
  transport<R>(tr, prim[4], mu, kc);
  R div = R(0);
#pragma unroll
  for (int i = 0; i < 5; ++i) vflux[i] = R(0.0);
#pragma unroll
  for (int i = 0; i < 3; ++i) div += g[i + 1][i];
  // t_ij = S_ij - div*delta_ij/3. Off the diagonal the subtracted term is a
  // signed zero, so t_ij = S_ij up to the sign of a zero, which cannot change
  // the +0-started sums below; on the diagonal div/3 is rounded exactly.
  const R div3 = div_by_recip(div * R(1), R(3.), R(1.0 / 3.0));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R S = R(0.5) * (g[i + 1][j] + g[j + 1][i]);
      const R tij = (i == j) ? S - div3 : S;
      vflux[1 + i] += (R(2) * mu * tij) * a[j];
      vflux[4] += (R(2) * mu * tij) * prim[i + 1] * a[j];
    }
    vflux[4] += kc * g[4][i] * a[i];
  }
}

// viscous_flux for an area vector that is nonzero only along axis D: the
// terms with a zero area component are signed zeros in +0-started sums.
template <class R, int D>
__device__ __forceinline__ void viscous_flux_axis(const R g[5][3], const R prim[5], R aD, const Transport& tr,
                                                  R vflux[5]) {
  R mu, kc;
  transport<R>(tr, prim[4], mu, kc);
  R div = R(0);
#pragma unroll
  for (int i = 0; i < 3; ++i) div += g[i + 1][i];
  const R div3 = div_by_recip(div * R(1), R(3.), R(1.0 / 3.0));
  vflux[0] = R(0.0);
  R v4 = R(0.0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const R S = halve(g[i + 1][D] + g[D + 1][i]);
    const R tiD = (i == D) ? S - div3 : S;
    vflux[1 + i] = zero_plus((twice(mu) * tiD) * aD);  // 0 + term
    const R t4 = (twice(mu) * tiD) * prim[i + 1] * aD;
    v4 = i == 0 ? zero_plus(t4) : v4 + t4;
    if (i == D) v4 += kc * g[4][D] * aD;
  }
  vflux[4] = v4;
}

// The reference's two branches (du > 1e-40 with dumax, du < -1e-40 with
// dumin) are one expression with the stencil difference selected first, so a
// warp whose cells see both signs evaluates it once.
template <class R>
__device__ __forceinline__ R venkat(R dumax, R dumin, R du, R deltax3) {
  const R eps2 = deltax3;  // deltax3 * beta^3 with beta = 1
  const bool pos = du > R(1e-40), neg = du < R(-1e-40);
  if (!(pos || neg)) return R(1);
  const R dm = pos ? dumax : dumin;
  const R num = (dm * dm + eps2) * du + R(2) * du * du * dm;
  const R den = du * (dm * dm + R(2) * du * du + dm * du + eps2);
  return num / den;
}

// Numerator and denominator of the Venkatakrishnan function, rounded exactly
// as venkat() rounds them, normalised to n >= 0, d > 0 (both are negated
// when du < 0, which is exact). Returns false where venkat() returns 1.
// Order keys: double comparisons on the integer pipe (on GB300 a double
// compare occupies the FP64 pipe like an add, and that pipe bounds the sweep).
// ikey(x) is a signed 64-bit key, monotone and injective over all non-NaN
// doubles, with ikey(-0) = -1 just below ikey(+0) = 0; from_ikey inverts it.
// ckey moves the negative keys up by one, so -0 and +0 meet: comparing ckeys
// gives the IEEE result of <, ==, > for every pair of non-NaN doubles.
__device__ __forceinline__ long long ikey(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double from_ikey(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL));
}
__device__ __forceinline__ long long ckey(long long k) { return k - (k >> 63); }
__device__ __forceinline__ long long okey(double x) { return ckey(ikey(x)); }

__device__ __forceinline__ bool venkat_ratio(double dumax, double dumin, double du, double eps2, double& n,
                                             double& d) {
  // du > 1e-40 and du < -1e-40 as key comparisons (same result for non-NaN
  // du); one evaluation with the selected difference, as in venkat().
  const long long kd = okey(du);
  const bool pos = kd > okey(1e-40), neg = kd < okey(-1e-40);
  if (!(pos | neg)) return false;
  const double dm = pos ? dumax : dumin;
  n = negate_if((dm * dm + eps2) * du + twice(du) * du * dm, neg);
  d = negate_if(du * (dm * dm + twice(du) * du + dm * du + eps2), neg);
  return true;
}

// Exact test n1/d1 < n2/d2 for d1, d2 > 0: compares n1*d2 with n2*d1 as
// unevaluated sums p + e (p = RN(x*y), e = fma(x, y, -p) exact).
// The comparisons use order keys (exact for non-NaN values).
__device__ __forceinline__ bool ratio_less(double n1, double d1, double n2, double d2) {
  const double p1 = n1 * d2, p2 = n2 * d1;
  const long long k1 = okey(p1), k2 = okey(p2);
  if (k1 != k2) return k1 < k2;
  return okey(fma(n1, d2, -p1)) < okey(fma(n2, d1, -p2));
}

template <class R>
__device__ __forceinline__ R vanalbada(R dumax, R dumin, R du) {
  // The reference's threshold is DBL_EPSILON in both precisions. Its two
  // quotients (dumax / du for du > eps, dumin / du for du < -eps) are one
  // division of the selected difference.
  const bool pos = du > R(DBL_EPSILON), neg = du < R(-DBL_EPSILON);
  R y = R(2);
  if (pos || neg) y = (pos ? dumax : dumin) / du;
  R phi = R(1);
  if (y < R(2)) {
    phi = (R(4) * y - y * y) / (y * y - R(4) * y + R(8));
    phi = (phi < R(0.0)) ? R(0.0) : phi;   // std::max(phi, 0.0)
    phi = (R(1.0) < phi) ? R(1.0) : phi;   // std::min(phi, 1.0)
  }
  return phi;
}

// Ghost state with the normal velocity reflected; nn is |n| computed as
// sqrt(((0 + n0^2) + n1^2) + n2^2), which equals the Roe |n|.
template <class R>
__device__ __forceinline__ void reflect_state(const R n[3], R nn, const R pl[5], R pr[5]) {
  R ub = zero_plus(pl[1] * n[0] / nn);  // a sum from +0
  ub += pl[2] * n[1] / nn;
  ub += pl[3] * n[2] / nn;
  const R ub2 = twice(ub);
  pr[0] = pl[0];
  pr[1] = pl[1] - ub2 * n[0] / nn;
  pr[2] = pl[2] - ub2 * n[1] / nn;
  pr[3] = pl[3] - ub2 * n[2] / nn;
  pr[4] = pl[4];
}

}  // namespace dev
}  // namespace miniaero
