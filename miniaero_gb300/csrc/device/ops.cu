// Operator-level kernels (unit parity of the device physics against the
// oracle) and the state check. FP64, compiled with --fmad=false.
#include <cstdint>

#include "kernels.cuh"

namespace miniaero {
namespace dev {

namespace {

__global__ void k_check_state(int C, const double* __restrict__ Un, unsigned long long* first_bad) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 5; ++k) bad |= !isfinite(Un[k * C + c]);
  bad |= !(Un[c] > 0.0) || !(Un[4 * C + c] > 0.0);
  if (bad) atomicMin(first_bad, static_cast<unsigned long long>(c));
}

// ---- operator-level kernels ----
__global__ void k_op_roe(int n, const double* pl, const double* pr, const double* nrm, const double* tan_,
                         const double* bin, double* flux) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  FaceFrame<double> fr;
  const double* a = nrm + 3 * i;
  const double* tt = tan_ + 3 * i;
  const double* b = bin + 3 * i;
  const double nn = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double tn = sqrt(tt[0] * tt[0] + tt[1] * tt[1] + tt[2] * tt[2]);
  const double bn = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  for (int d = 0; d < 3; ++d) {
    fr.n[d] = a[d];
    fr.nu[d] = a[d] / nn;
    fr.tu[d] = tt[d] / tn;
    fr.bu[d] = b[d] / bn;
  }
  fr.nn = nn;
  roe_flux<double>(pl + 5 * i, pr + 5 * i, fr, flux + 5 * i);
}

__global__ void k_op_viscous(int n, const double* grad, const double* prim, const double* area, Transport tr,
                             double* vflux) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double g[5][3];
  for (int k = 0; k < 5; ++k)
    for (int d = 0; d < 3; ++d) g[k][d] = grad[15 * i + 3 * k + d];
  viscous_flux<double>(g, prim + 5 * i, area + 3 * i, tr, vflux + 5 * i);
}

__global__ void k_op_limiter(int n, int kind, const double* dumax, const double* dumin, const double* du,
                             const double* d2, double* phi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  phi[i] = kind == 1 ? vanalbada<double>(dumax[i], dumin[i], du[i]) : venkat<double>(dumax[i], dumin[i], du[i], d2[i]);
}

__global__ void k_op_primitives(int n, const double* U, double* V) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  primitives(U + 5 * i, V + 5 * i);
}

// Each cell's boundary-face contributions summed in its residual list order
// (boundary sets grouped Extrapolate, Tangent, NoSlip, Inflow), from +0 as
// zero_cell_flux leaves the accumulator: out [5][C].
__global__ void k_bc_gather(TopoView t, const double* __restrict__ fflux, double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= t.C) return;
  const int C = t.C;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int s = 0; s < kMaxCellFaces; ++s) {
    const int code = t.csr_flux[s * C + c];
    if (code < 0) continue;
    const int f = code >> 1;
    if (f < t.Fi) continue;
#pragma unroll
    for (int k = 0; k < 5; ++k) acc[k] += fflux[static_cast<size_t>(f) * 5 + k];
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) out[k * C + c] = acc[k];
}

// W = ComputePrimitives(U) per cell on [5][C] arrays (U as given, no stage update).
__global__ void k_field_primitives(int C, const double* __restrict__ U, double* __restrict__ W) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  double u[5], v[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) u[k] = U[k * C + c];
  primitives(u, v);
#pragma unroll
  for (int k = 0; k < 5; ++k) W[k * C + c] = v[k];
}

// apply_cell_flux (Flux.h:188-229) on host-layout arrays: res = 0 + (dt/V) flux.
__global__ void k_op_apply_cell_flux(int n, double dt, const double* __restrict__ vol, const double* __restrict__ flux,
                                     double* __restrict__ res) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double dtv = dt / vol[c];
#pragma unroll
  for (int k = 0; k < 5; ++k) res[5 * c + k] = 0.0 + dtv * flux[5 * c + k];
}

// update (TimeSolverExplicitRK4.h:106-128): dst = src + alpha * res.
__global__ void k_op_rk_update(long long n, double alpha, const double* __restrict__ res,
                               const double* __restrict__ src, double* __restrict__ dst) {
  const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  if (i < n) dst[i] = src[i] + alpha * res[i];
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Double with random significand bits and a biased exponent in [e0, e0 + span).
__device__ __forceinline__ double make_double(uint64_t r, int e0, int span, bool negative_ok) {
  const uint64_t mant = r & 0x000FFFFFFFFFFFFFull;
  const uint64_t e = static_cast<uint64_t>(e0 + static_cast<int>((r >> 52) % static_cast<uint64_t>(span)));
  const uint64_t sign = (negative_ok && ((r >> 63) & 1)) ? (1ull << 63) : 0ull;
  return __longlong_as_double(static_cast<long long>(sign | (e << 52) | mant));
}

// div_by_recip against the IEEE quotient on generated operand pairs.
// mode 0: random a and b; 1: b with an all-ones significand (possibly a few
// bits cleared); 2: quotients close to a rounding midpoint; 5: tiny,
// subnormal and zero numerators (3 and 4 check the float conversions, 6 the
// FP64 identities done with integer instructions).
__global__ void k_check_division(int mode, unsigned long long n, unsigned long long seed,
                                 unsigned long long* mismatches, double* example) {
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    uint64_t st = seed ^ (i * 0xD1B54A32D192ED03ull);
    const uint64_t r1 = splitmix64(st), r2 = splitmix64(st), r3 = splitmix64(st);
    double a = make_double(r1, 1023 - 300, 600, true);
    double b = make_double(r2, 1023 - 60, 120, false);
    if (mode == 1) {
      const uint64_t clear = (r3 & 7) ? (r3 >> 8) & ((1ull << (r3 & 7)) - 1) : 0ull;
      b = __longlong_as_double(static_cast<long long>((__double_as_longlong(b) | 0x000FFFFFFFFFFFFFull) & ~clear));
    } else if (mode == 2) {
      const double m = make_double(r3, 1023 - 40, 80, true);
      const double h = __longlong_as_double(static_cast<long long>(
          (static_cast<uint64_t>(__double_as_longlong(m)) & 0x7FF0000000000000ull) - (53ull << 52)));
      a = fma(b, m, b * h);  // a / b close to the midpoint between m and its successor
    }
    if (mode == 4) {  // narrow_rn against the hardware conversion
      // Random bit patterns (any exponent), values in and next to the float
      // normal range, exact midpoints between floats and their neighbours.
      uint64_t bits = r1;
      const uint32_t kind = static_cast<uint32_t>(r3 & 3u);
      if (kind >= 1u) {
        const uint64_t E = 895u + (r2 % 258u);  // 895..1152: both edges of the float range
        bits = (r1 & 0x800FFFFFFFFFFFFFull) | (E << 52);
      }
      if (kind >= 2u) {
        bits = (bits & ~0x1FFFFFFFull) | 0x10000000ull;  // exact midpoint
        if (kind == 3u) bits += ((r3 >> 8) & 1u) ? 1u : static_cast<uint64_t>(-1);
      }
      const double x = __longlong_as_double(static_cast<long long>(bits));
      const float got = narrow_rn(x), ref = __double2float_rn(x);
      const bool same = (ref != ref) ? (got != got) : (__float_as_uint(got) == __float_as_uint(ref));
      if (!same && atomicAdd(mismatches, 1ull) == 0ull) {
        example[0] = x;
        example[1] = static_cast<double>(got);
      }
      continue;
    }
    if (mode == 3) {  // widen_exact against the hardware conversion
      const float f = __uint_as_float(static_cast<uint32_t>(r1));
      const double w = widen_exact(f);
      const bool sub = ((static_cast<uint32_t>(r1) >> 23) & 0xFFu) == 0u;
      const double ref = sub ? __longlong_as_double(static_cast<long long>(static_cast<uint64_t>(r1 & 0x80000000u) << 32))
                             : static_cast<double>(f);
      const bool same = (f != f) ? (w != w) : (__double_as_longlong(w) == __double_as_longlong(ref));
      if (!same && atomicAdd(mismatches, 1ull) == 0ull) {
        example[0] = static_cast<double>(f);
        example[1] = w;
      }
      continue;
    }
    if (mode == 6) {
      // The FP64 identities taken on the integer pipe against the FP64
      // instructions they replace: halve = 0.5 * x, twice = 2 * x,
      // zero_plus = 0 + x, dabs = fabs and less_nonneg(|x|, y) = |x| < y (y not
      // a NaN), over every exponent class (zeros, subnormals, the smallest and
      // largest binades, infinities and NaNs, and random normal values).
      uint64_t bits = r1;
      const uint32_t kind = static_cast<uint32_t>(r3 & 7u);
      const uint64_t E = kind == 0u ? 0u : kind == 1u ? 1u : kind == 2u ? 2u : kind == 3u ? 2045u
                       : kind == 4u ? 2046u : kind == 5u ? 2047u : ((r2 >> 52) & 0x7FFu);
      bits = (bits & 0x800FFFFFFFFFFFFFull) | (E << 52);
      if (((r3 >> 3) & 15u) == 0u) bits &= 0x8000000000000000ull | (E << 52);  // zero significand
      const double x = __longlong_as_double(static_cast<long long>(bits));
      const double y = __longlong_as_double(static_cast<long long>(r2));
      auto same = [](double p, double q) {
        return (q != q) ? (p != p) : (__double_as_longlong(p) == __double_as_longlong(q));
      };
      const double ax = fabs(x);
      bool ok = same(halve(x), __dmul_rn(0.5, x)) && same(twice(x), __dmul_rn(2.0, x)) &&
                same(zero_plus(x), __dadd_rn(0.0, x)) && same(dabs<double>(x), ax);
      if (y == y && x == x) ok = ok && (less_nonneg(ax, y) == (ax < y)) && (less_nonneg(ax, x) == (ax < x));
      if (!ok && atomicAdd(mismatches, 1ull) == 0ull) {
        example[0] = x;
        example[1] = y;
      }
      continue;
    }
    if (mode == 5) {
      // Numerators from the subnormal range up to 2^-880 (quotients near and
      // below the underflow threshold), and signed zeros.
      const uint64_t e = r2 % 144u;  // biased exponents 0..143
      a = __longlong_as_double(static_cast<long long>((r1 & 0x800FFFFFFFFFFFFFull) | (e << 52)));
      if ((r3 & 63u) == 0u) a = ((r3 >> 6) & 1u) ? -0.0 : 0.0;
    }
    const double y = 1.0 / b;
    const double q = div_by_recip(a, b, y);
    const double ref = a / b;
    // The sweep's form with the two-part reciprocal, where it does not flag
    // the quotient for the IEEE division (zero quotients of either sign).
    bool inexact = false;
    const double q2 = div_by_recip2_flag(a, b, y, recip_lo(b, y), inexact);
    const bool ok2 = inexact || (a == 0.0 ? q2 == 0.0 : __double_as_longlong(q2) == __double_as_longlong(ref));
    if (__double_as_longlong(q) != __double_as_longlong(ref) || !ok2) {  // zeros included, with their sign
      if (atomicAdd(mismatches, 1ull) == 0ull) {
        example[0] = a;
        example[1] = b;
      }
    }
  }
}

// FP64 issue rate: 4 independent chains of one operation per thread
// (op 0 x + y, 1 x * y, 2 fma(x, y, y)); y comes in as a parameter so the
// chains cannot be folded, and each thread stores its sum.
template <int OP>
__global__ void __launch_bounds__(256) k_fp64_rate(int iters, double y, double* __restrict__ out) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double x[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) x[j] = 1.0 + 1e-3 * (tid + j);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) x[j] = OP == 0 ? x[j] + y : OP == 1 ? x[j] * y : fma(x[j], y, y);
  }
  out[tid] = (x[0] + x[1]) + (x[2] + x[3]);
}

// dt = cfl * min_c V_c / sum_f (|u.n| + c |n|) on the current U_n.
__global__ void k_cfl(TopoView t, GeomView<double> g, const double* __restrict__ Un,
                      unsigned long long* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= t.C) return;
  const int C = t.C, F = t.F;
  double U[5], V[5];
  for (int k = 0; k < 5; ++k) U[k] = Un[k * C + c];
  primitives(U, V);
  const double a = sqrt(1.4 * 287.05 * V[4]);
  double sum = 0.0;
  for (int s = 0; s < kMaxCellFaces; ++s) {
    const int code = t.csr_grad[s * C + c];
    if (code < 0) continue;
    const int f = code >> 1;
    const double un = V[1] * g.fn[f] + V[2] * g.fn[F + f] + V[3] * g.fn[2 * F + f];
    sum += fabs(un) + a * g.fnn[f];
  }
  const double r = t.vol[c] / sum;
  if (r > 0.0) atomicMin(out, static_cast<unsigned long long>(__double_as_longlong(r)));
}

inline unsigned blocks_for(int n, int bs) { return static_cast<unsigned>((n + bs - 1) / bs); }

}  // namespace

int launches_per_stage(const PathConfig& cfg, const TopoView& t) {
  int n = 1;  // residual
  if (cfg.second_order || cfg.viscous) ++n;
  if (t.Fi > 0) ++n;
  if (t.Fb > 0) ++n;
  return n;
}

cudaError_t launch_op_roe(int n, const double* pl, const double* pr, const double* normal, const double* tangent,
                          const double* binormal, double* flux, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_roe<<<blocks_for(n, 128), 128, 0, stream>>>(n, pl, pr, normal, tangent, binormal, flux);
  return cudaGetLastError();
}

cudaError_t launch_op_viscous(int n, const double* grad, const double* prim, const double* area, Transport tr,
                              double* vflux, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_viscous<<<blocks_for(n, 128), 128, 0, stream>>>(n, grad, prim, area, tr, vflux);
  return cudaGetLastError();
}

cudaError_t launch_op_limiter(int n, int kind, const double* dumax, const double* dumin, const double* du,
                              const double* d2, double* phi, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_limiter<<<blocks_for(n, 256), 256, 0, stream>>>(n, kind, dumax, dumin, du, d2, phi);
  return cudaGetLastError();
}

cudaError_t launch_op_primitives(int n, const double* U, double* V, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_primitives<<<blocks_for(n, 256), 256, 0, stream>>>(n, U, V);
  return cudaGetLastError();
}

cudaError_t launch_check_division(int mode, unsigned long long n, unsigned long long seed,
                                  unsigned long long* mismatches, double* example, cudaStream_t stream) {
  k_check_division<<<152 * 8, 256, 0, stream>>>(mode, n, seed, mismatches, example);
  return cudaGetLastError();
}

cudaError_t launch_bc_gather(const TopoView& t, const double* fflux, double* out, cudaStream_t stream) {
  if (t.C <= 0) return cudaSuccess;
  k_bc_gather<<<blocks_for(t.C, 256), 256, 0, stream>>>(t, fflux, out);
  return cudaGetLastError();
}

cudaError_t launch_field_primitives(int C, const double* U, double* W, cudaStream_t stream) {
  if (C <= 0) return cudaSuccess;
  k_field_primitives<<<blocks_for(C, 256), 256, 0, stream>>>(C, U, W);
  return cudaGetLastError();
}

cudaError_t launch_op_apply_cell_flux(int n, double dt, const double* vol, const double* flux, double* res,
                                      cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_op_apply_cell_flux<<<blocks_for(n, 256), 256, 0, stream>>>(n, dt, vol, flux, res);
  return cudaGetLastError();
}

cudaError_t launch_op_rk_update(long long n, double alpha, const double* res, const double* src, double* dst,
                                cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = (n + 255) / 256;
  k_op_rk_update<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(n, alpha, res, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_fp64_rate(int op, int blocks, int iters, double* out, cudaStream_t stream) {
  const double y = op == 1 ? 1.0000001 : 1e-9;
  if (op == 0) k_fp64_rate<0><<<blocks, 256, 0, stream>>>(iters, y, out);
  else if (op == 1) k_fp64_rate<1><<<blocks, 256, 0, stream>>>(iters, y, out);
  else k_fp64_rate<2><<<blocks, 256, 0, stream>>>(iters, y, out);
  return cudaGetLastError();
}

cudaError_t launch_cfl(const TopoView& t, const GeomView<double>& g, const double* Un, unsigned long long* out,
                       cudaStream_t stream) {
  if (t.C <= 0) return cudaSuccess;
  k_cfl<<<blocks_for(t.C, 256), 256, 0, stream>>>(t, g, Un, out);
  return cudaGetLastError();
}

cudaError_t launch_check_state(int C, const double* Un, unsigned long long* first_bad, cudaStream_t stream) {
  if (C <= 0) return cudaSuccess;
  k_check_state<<<blocks_for(C, 256), 256, 0, stream>>>(C, Un, first_bad);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace miniaero
