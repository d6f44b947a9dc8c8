// Kernel templates of the RK4 residual path, included by the translation
// unit of each precision (kernels_fp64.cu with --fmad=false for the plain,
// bit-exact form; kernels_mixed.cu for the mixed form). Per RK stage:
//   k_sweep1        cell-centric: Green-Gauss gradient, stencil min/max and
//                   limiter of one cell from its ordered face list
//                   (GreenGauss.h:51-270, StencilLimiter.h:56-500)
//   k_internal_flux face-centric: extrapolation, Roe and viscous flux of one
//                   internal face (Flux.h:89-180)
//   k_bc_flux       face-centric: boundary ghost state and flux
//                   (Extrapolate_BC.h, Tangent_BC.h, NoSlip_BC.h, Inflow_BC.h)
//   k_residual      cell-centric: ordered face-flux gather, dt/V scaling, RK4
//                   accumulation and the next stage's primitives
//                   (Flux.h:188-229, TimeSolverExplicitRK4.h:106-128,352-489)
// Each accumulator is summed in the reference's serial order (the per-cell
// lists are built on the host), so the FP64 instantiation reproduces the
// reference's Serial results bit for bit.
#pragma once
#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "kernels.cuh"

namespace miniaero {
namespace dev {

namespace {

constexpr int kCellBlock = 256;
constexpr int kFaceBlock = 128;
constexpr int kSmallMeshCells = 152 * kCellBlock * 2;
// Resident sweep blocks per SM: the FP32 sweep waits on dependent gathers; at
// 4 blocks (64 registers, no spill) it runs 12 % faster than at 5 (48
// registers, 44 bytes spilled) with the approximate FP32 division. The FP64
// sweep is FP64-pipe bound at 2.
template <class R>
constexpr int kSweepMinBlocks = std::is_same<R, float>::value ? 4 : 2;
// The FP32 face flux at 8 blocks of 128 (64 registers): 6 % faster than the
// 7 blocks its approximate division and square root would otherwise leave.
// The first-order inviscid FP64 flux at 5 (96 registers): on small meshes
// (94 k faces on 32 k cells) its 734 blocks then fit one wave, where 4 per SM
// left a fifth block running alone, latency-bound, on most SMs.
template <class R, bool SECOND, bool VISC>
constexpr int kFluxMinBlocks = std::is_same<R, float>::value ? 8 : (!SECOND && !VISC ? 5 : 0);

// Resident residual blocks per SM (0: no bound). The mixed residual holds a
// cell's 30 face-flux words for its integer sums.
template <class R>
constexpr int kResidualMinBlocks = std::is_same<R, float>::value ? 6 : 0;

// Primitives of an FP64 state written as R: FP64 arithmetic for the plain
// form (bit-exact), FP32 for the mixed form (its flux work is FP32 anyway).
template <class R>
__device__ __forceinline__ void store_primitives(const double ut[5], R* __restrict__ W, int C, int c) {
  if constexpr (std::is_same<R, double>::value) {
    double v[5];
    primitives(ut, v);
#pragma unroll
    for (int k = 0; k < 5; ++k) W[k * C + c] = v[k];
  } else {
    // narrow_rn: the float conversion, on the integer pipe.
    const float r = narrow_rn(ut[0]);
    const float ri = 1.0f / r;
    const float u = narrow_rn(ut[1]) * ri, v = narrow_rn(ut[2]) * ri, w = narrow_rn(ut[3]) * ri;
    const float e = narrow_rn(ut[4]) * ri - 0.5f * (u * u + v * v + w * w);
    W[c] = r;
    W[C + c] = u;
    W[2 * C + c] = v;
    W[3 * C + c] = w;
    W[4 * C + c] = e * (0.4f / 287.05f);
  }
}

template <class R> __device__ __forceinline__ double to_double(R x);
template <> __device__ __forceinline__ double to_double<double>(double x) { return x; }
template <> __device__ __forceinline__ double to_double<float>(float x) { return widen_exact(x); }

template <class R> __device__ __forceinline__ R big_value();
template <> __device__ __forceinline__ double big_value<double>() { return 1.0e300; }
template <> __device__ __forceinline__ float big_value<float>() { return FLT_MAX; }

template <class R>
__device__ __forceinline__ FaceFrame<R> load_frame(const GeomView<R>& g, int f, int F) {
  FaceFrame<R> fr;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    fr.n[d] = g.fn[d * F + f];
    fr.nu[d] = g.fnu[d * F + f];
    fr.tu[d] = g.ftu[d * F + f];
    fr.bu[d] = g.fbu[d * F + f];
  }
  fr.nn = g.fnn[f];
  return fr;
}

// Running stencil minimum and maximum with the selections the existing
// kernels make for min_max_face / gather_min_max (StencilLimiter.h:57,246):
// fmin = (pr < pl) ? pr : pl, fmax = (pr > pl) ? pr : pl, then
// mn = (fmin < mn) ? fmin : mn, mx = (mx < fmax) ? fmax : mx.
template <class R>
struct Extrema {
  R mn, mx;
  __device__ __forceinline__ Extrema() : mn(big_value<R>()), mx(-big_value<R>()) {}
  __device__ __forceinline__ void face(R pl, R pr) {
    const R fmin_ = (pr < pl) ? pr : pl;
    const R fmax_ = (pr > pl) ? pr : pl;
    mn = (fmin_ < mn) ? fmin_ : mn;
    mx = (mx < fmax_) ? fmax_ : mx;
  }
  __device__ __forceinline__ void one(R w) {
    mn = (w < mn) ? w : mn;
    mx = (mx < w) ? w : mx;
  }
  __device__ __forceinline__ R min() const { return mn; }
  __device__ __forceinline__ R max() const { return mx; }
};

// FP64: the same selections made on order keys (integer pipe); the running
// values are held as injective keys, so the selected double (sign of zero
// included) comes back exactly. Identical to the compares above for non-NaN
// values.
template <>
struct Extrema<double> {
  long long mn, mx;
  __device__ __forceinline__ Extrema() : mn(ikey(big_value<double>())), mx(ikey(-big_value<double>())) {}
  __device__ __forceinline__ void face(double pl, double pr) {
    const long long kl = ikey(pl), kr = ikey(pr);
    const long long cl = ckey(kl), cr = ckey(kr);
    const bool lt = cr < cl, gt = cr > cl;
    const long long kmin = lt ? kr : kl, cmin = lt ? cr : cl;
    const long long kmax = gt ? kr : kl, cmax = gt ? cr : cl;
    mn = (cmin < ckey(mn)) ? kmin : mn;
    mx = (ckey(mx) < cmax) ? kmax : mx;
  }
  __device__ __forceinline__ void one(double w) {
    const long long kw = ikey(w), cw = ckey(kw);
    mn = (cw < ckey(mn)) ? kw : mn;
    mx = (ckey(mx) < cw) ? kw : mx;
  }
  __device__ __forceinline__ double min() const { return from_ikey(mn); }
  __device__ __forceinline__ double max() const { return from_ikey(mx); }
};

// Venkatakrishnan limiter of one cell in FP64: min(1, phi_f over its faces)
// with phi_f = RN(n_f / d_f). Rounding is monotone, so the minimum equals
// RN(min_f n_f / d_f): the smallest ratio is found with exact
// cross-multiplied comparisons and divided once per component. AXIS: the
// cell's offsets are nonzero only along the axis of each face (slots 2p,
// 2p+1 normal to axis p), so the dot products 0 + dx*gx + dy*gy + dz*gz
// reduce to their p term (the others are signed zeros for finite gradients,
// which cannot change a +0-started sum; a zero du is not limited either way).
template <bool AXIS>
__device__ __forceinline__ void venkat_cell(const TopoView& t, const GeomView<double>& g, const double wc[5],
                                            const double mn[5], const double mx[5], const double gsum[5][3],
                                            double* __restrict__ phi, int c) {
  const int C = t.C, F = t.F;
  double nm[5], dm[5], dmax[5], dmin[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    nm[k] = 1.0;
    dm[k] = 1.0;
    dmax[k] = mx[k] - wc[k];  // the stencil differences, once per cell
    dmin[k] = mn[k] - wc[k];
  }
  if constexpr (AXIS) {
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll 1
      for (int q = 0; q < 2; ++q) {
        const int code = t.csr_grad[(2 * p + q) * C + c];
        const int f = code >> 1;
        const double* dv = (code & 1) ? g.dL : g.dR;
        const double dp = dv[p * F + f];
        const double dist = dp * dp;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const double du = dp * gsum[k][p];
          double n, dd;
          if (venkat_ratio(dmax[k], dmin[k], du, dist, n, dd) && ratio_less(n, dd, nm[k], dm[k])) {
            nm[k] = n;
            dm[k] = dd;
          }
        }
      }
    }
  } else {
#pragma unroll 1
    for (int s = 0; s < kMaxCellFaces; ++s) {
      const int code = t.csr_grad[s * C + c];
      if (code < 0) continue;
      const int f = code >> 1;
      const double* dv = (code & 1) ? g.dL : g.dR;
      const double disp[3] = {dv[f], dv[F + f], dv[2 * F + f]};
      double dist = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) dist += disp[d] * disp[d];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        double du = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) du += disp[d] * gsum[k][d];
        double n, dd;
        if (venkat_ratio(dmax[k], dmin[k], du, dist, n, dd) && ratio_less(n, dd, nm[k], dm[k])) {
          nm[k] = n;
          dm[k] = dd;
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) phi[k * C + c] = (nm[k] == 1.0 && dm[k] == 1.0) ? 1.0 : nm[k] / dm[k];
}

// Warp buffer of the FP64 Venkatakrishnan limiter: one slot per (lane, face)
// holding the face's selected stencil difference, du and |x_f - x_c|^2 (the
// first two are overwritten by n and d), and the list of active slots.
struct VenkatWarpBuf {
  double a[32 * kMaxCellFaces];
  double b[32 * kMaxCellFaces];
  double e[32 * kMaxCellFaces];
  uint8_t slot[32 * kMaxCellFaces];
};
constexpr int kVenkatBufBytes = static_cast<int>(sizeof(VenkatWarpBuf));

__device__ __forceinline__ VenkatWarpBuf& venkat_warp_buf() {
  extern __shared__ __align__(16) unsigned char venkat_smem[];
  return reinterpret_cast<VenkatWarpBuf*>(venkat_smem)[threadIdx.x >> 5];
}

// Venkatakrishnan limiter of the warp's 32 cells in FP64. Every lane of the
// warp calls it (a lane with !valid has no items and stores nothing).
// phi = min(1, phi_f over the faces) with phi_f = RN(n_f / d_f); rounding is
// monotone, so the minimum is RN(min_f n_f / d_f): the smallest ratio is
// found with exact cross-multiplied comparisons and divided once per
// component. Per component, each cell puts the faces whose du passes the
// limiter's threshold in its buffer slots; then the warp either skips the
// component (no such face), lets each lane evaluate its own slots (as many
// rounds as its busiest lane has faces), or, when fewer rounds result, lists
// the active slots end to end (prefix sum over the lanes) and has the 32
// lanes evaluate the list 32 at a time, so a warp whose cells are partly
// inside a wave does not run the formula on idle lanes. Each cell then
// compares its own results in its face order, as the serial loop does, so
// ties resolve identically and the bits are venkat_cell's. axis: the
// cell's offsets lie along the axis of each face (slots 2p, 2p+1 normal to
// axis p), so the dot products 0 + dx*gx + dy*gy + dz*gz reduce to their p
// term (the others are signed zeros for finite gradients, which cannot change
// a +0-started sum; a zero du is not limited either way).
__device__ __forceinline__ void venkat_warp(const TopoView& t, const GeomView<double>& g, const double wc[5],
                                            const double mn[5], const double mx[5], const double gsum[5][3],
                                            double* __restrict__ phi, int c, bool valid, bool axis,
                                            VenkatWarpBuf& buf) {
  const int C = t.C, F = t.F;
  const int lane = threadIdx.x & 31;
  const int own = lane * kMaxCellFaces;
  // |x_f - x_c|^2 per face, once per cell.
  unsigned faces = 0;  // slots with a face
#pragma unroll 1
  for (int s = 0; s < kMaxCellFaces; ++s) {
    const int code = t.csr_grad[s * C + c];
    if (!valid || code < 0) continue;
    faces |= 1u << s;
    const int f = code >> 1;
    const double* dv = (code & 1) ? g.dL : g.dR;
    double dist;
    if (axis) {
      const double dp = dv[(s >> 1) * F + f];
      dist = dp * dp;
    } else {
      dist = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) dist += dv[d * F + f] * dv[d * F + f];
    }
    buf.e[own + s] = dist;
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double dmax = mx[k] - wc[k], dmin = mn[k] - wc[k];  // the stencil differences
    double gk[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) gk[d] = gsum[k][d];
    unsigned act = 0;
#pragma unroll 1
    for (int s = 0; s < kMaxCellFaces; ++s) {
      if (!((faces >> s) & 1u)) continue;
      const int code = t.csr_grad[s * C + c];
      const int f = code >> 1;
      const double* dv = (code & 1) ? g.dL : g.dR;
      double du;
      if (axis) {
        const int p = s >> 1;
        du = dv[p * F + f] * (p == 0 ? gk[0] : p == 1 ? gk[1] : gk[2]);
      } else {
        du = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) du += dv[d * F + f] * gk[d];
      }
      // du > 1e-40 and du < -1e-40 as key comparisons (same result for non-NaN du).
      const long long kd = okey(du);
      const bool pos = kd > okey(1e-40), neg = kd < okey(-1e-40);
      if (pos | neg) {
        act |= 1u << s;
        buf.a[own + s] = pos ? dmax : dmin;
        buf.b[own + s] = du;
      }
    }
    // Per warp: no item, each lane evaluating its own items (as many rounds
    // as the busiest lane has items), or the compacted list (total / 32
    // rounds plus the listing), whichever is shorter.
    const unsigned cnt = __popc(act);
    const unsigned most = __reduce_max_sync(0xffffffffu, cnt);
    double nm = 1.0, dn = 1.0;
    if (most) {
      const unsigned total = __reduce_add_sync(0xffffffffu, cnt);
      const bool compact = (total + 31) / 32 + 1 < most;
      if (compact) {
        unsigned incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += v;
        }
        unsigned at = incl - cnt;
        for (unsigned m = act; m; m &= m - 1) buf.slot[at++] = static_cast<uint8_t>(own + __ffs(m) - 1);
      }
      __syncwarp();
      auto evaluate = [&](int q) {
        const double dm = buf.a[q], du = buf.b[q], eps2 = buf.e[q];
        const bool neg = okey(du) < 0;  // du is past the threshold: its sign decides
        buf.a[q] = negate_if((dm * dm + eps2) * du + twice(du) * du * dm, neg);
        buf.b[q] = negate_if(du * (dm * dm + twice(du) * du + dm * du + eps2), neg);
      };
      if (compact) {
        for (unsigned i = lane; i < total; i += 32) evaluate(buf.slot[i]);
      } else {
        for (unsigned m = act; m; m &= m - 1) evaluate(own + __ffs(m) - 1);
      }
      __syncwarp();
      for (unsigned m = act; m; m &= m - 1) {
        const int q = own + __ffs(m) - 1;
        const double n = buf.a[q], d = buf.b[q];
        if (ratio_less(n, d, nm, dn)) {
          nm = n;
          dn = d;
        }
      }
      __syncwarp();  // the next component reuses the slots
    }
    if (valid) phi[k * C + c] = (nm == 1.0 && dn == 1.0) ? 1.0 : nm / dn;
  }
}

// Limiter of one cell (MODE 1 Venkatakrishnan in FP32, MODE 2 Van Albada):
// minimum over its faces of the limiter function, in serial face order.
// AXIS: offsets along each face's axis only, slots grouped by axis as in
// venkat_warp; du and |d|^2 reduce to their one nonzero term.
template <class R, int MODE, bool AXIS>
__device__ __forceinline__ void limiter_cell(const TopoView& t, const GeomView<R>& g, const R wc[5], const R mn[5],
                                             const R mx[5], const R gsum[5][3], R* __restrict__ phi, int c) {
  const int C = t.C, F = t.F;
  R lim[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) lim[k] = R(1.0);
  auto apply = [&](int k, R du, R dist) {
    const R dumax = mx[k] - wc[k];
    const R dumin = mn[k] - wc[k];
    const R p = (MODE == 1) ? venkat<R>(dumax, dumin, du, dist) : vanalbada<R>(dumax, dumin, du);
    lim[k] = (p < lim[k]) ? p : lim[k];
  };
  if constexpr (AXIS) {
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int code = t.csr_grad[(2 * p + q) * C + c];
        const int f = code >> 1;
        const R dp = ((code & 1) ? g.dL : g.dR)[p * F + f];
        const R dist = dp * dp;
#pragma unroll
        for (int k = 0; k < 5; ++k) apply(k, dp * gsum[k][p], dist);
      }
    }
  } else {
#pragma unroll 1
    for (int s = 0; s < kMaxCellFaces; ++s) {
      const int code = t.csr_grad[s * C + c];
      if (code < 0) continue;
      const int f = code >> 1;
      const R* dv = (code & 1) ? g.dL : g.dR;
      const R disp[3] = {dv[f], dv[F + f], dv[2 * F + f]};
      R dist = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) dist += disp[d] * disp[d];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        R du = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) du += disp[d] * gsum[k][d];
        apply(k, du, dist);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) phi[k * C + c] = lim[k];
}

// Green-Gauss terms of one cell added into acc in the reference's serial
// face order (GreenGauss.h:79-220), div(a) giving each term a / V; with
// MINMAX the stencil min/max too. Axis-aligned cells (axis_cell bit 0): slots
// 2p, 2p+1 are the faces normal to axis p, in serial order, and only the
// gradient components along p get nonzero terms. A boundary face lists the
// cell as its own neighbour and takes the internal expressions, which give
// its terms exactly (GreenGauss.h:168-220, min_max_face<false>):
// 0.5 * (w + w) * n = w * n (w below half the largest finite value), and the
// min and max of (w, w) are w; so no branch holds back the gathers.
template <class R, bool MINMAX, class Div>
__device__ __forceinline__ void green_gauss_cell(const TopoView& t, const GeomView<R>& g, const R* __restrict__ W,
                                                 int c, const R wc[5], R acc[5][3], Extrema<R>* ex, Div div) {
  const int C = t.C, F = t.F;
  if (t.axis_cell[c]) {
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int s = 2 * p + q;
        const int code = t.csr_grad[s * C + c];
        const int f = code >> 1;
        const bool left = code & 1;
        const R np = g.fn[p * F + f];
        const int nb = t.csr_nbr[s * C + c];
        R wn[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) wn[k] = W[k * C + nb];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          const R pl = left ? wc[k] : wn[k];
          const R pr = left ? wn[k] : wc[k];
          const R gr = halve(pl + pr) * np;
          // acc starts at +0: its first term is 0 + x
          acc[k][p] = q == 0 ? zero_plus(div(left ? gr : -gr)) : acc[k][p] + div(left ? gr : -gr);
          if (MINMAX) ex[k].face(pl, pr);
        }
      }
    }
    return;
  }
#pragma unroll 1
  for (int s = 0; s < kMaxCellFaces; ++s) {
    const int code = t.csr_grad[s * C + c];
    if (code < 0) continue;
    const int f = code >> 1;
    const bool left = code & 1;
    const R n[3] = {g.fn[f], g.fn[F + f], g.fn[2 * F + f]};
    const int nb = t.csr_nbr[s * C + c];
    R wn[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) wn[k] = W[k * C + nb];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const R pl = left ? wc[k] : wn[k];
      const R pr = left ? wn[k] : wc[k];
      const R h = R(0.5) * (pl + pr);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const R gr = h * n[d];
        acc[k][d] += div(left ? gr : -gr);
      }
      if (MINMAX) ex[k].face(pl, pr);
    }
  }
}

// The gradient of one cell with every term divided by IEEE division, written
// as 0 + sum: the rare path for cells whose reciprocal-method terms may be
// inexact (quotients near the underflow threshold). Out of line, so its
// registers do not weigh on the sweep.
__device__ __noinline__ void gradient_exact(const TopoView& t, const GeomView<double>& g, const double* __restrict__ W,
                                            double* __restrict__ grad, int c) {
  const int C = t.C;
  double wc[5], acc[5][3];
  for (int k = 0; k < 5; ++k) {
    wc[k] = W[k * C + c];
    for (int d = 0; d < 3; ++d) acc[k][d] = 0.0;
  }
  const double V = g.vol[c];
  green_gauss_cell<double, false>(t, g, W, c, wc, acc, static_cast<Extrema<double>*>(nullptr),
                                  [&](double a) { return a / V; });
  for (int k = 0; k < 5; ++k)
    for (int d = 0; d < 3; ++d) grad[(3 * k + d) * C + c] = zero_plus(acc[k][d]);
}

// MODE: 0 gradient only (viscous first order), 1 + Venkatakrishnan, 2 + Van Albada.
// WARP: the FP64 Venkatakrishnan limiter is evaluated across the warp
// (venkat_warp; the batched sweep, whose small boxes leave many warps partly
// inside a wave): all 32 lanes call the sweep, and a lane past the last cell
// (valid false) recomputes a real cell and stores nothing. The single-mesh
// sweep keeps the per-cell limiter (venkat_cell), faster where warps are
// either wholly inside or wholly outside the waves. Both give the same bits.
template <class R, int MODE, bool WARP>
constexpr bool kWarpVenkat = WARP && MODE == 1 && std::is_same<R, double>::value;

template <class R, int MODE, bool WARP = false>
__device__ __forceinline__ void sweep1_cell(const TopoView& t, const GeomView<R>& g, const R* __restrict__ W,
                                            R* __restrict__ grad, R* __restrict__ phi, int c, bool valid = true) {
  const int C = t.C;
  R wc[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) wc[k] = W[k * C + c];
  const R V = g.vol[c];
  const R Vinv = g.vinv[c];  // RN(1/V), see div_by_recip
  const R Vlo = recip_lo(V, Vinv);  // 1/V = Vinv + Vlo for the 30 divisions below
  R acc[5][3];
  Extrema<R> ex[5];
#pragma unroll
  for (int k = 0; k < 5; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d) acc[k][d] = R(0.0);
  const int ac = t.axis_cell[c];
  bool inexact = false;  // some term's reciprocal quotient may differ from the IEEE one
  green_gauss_cell<R, (MODE > 0)>(t, g, W, c, wc, acc, ex,
                                  [&](R a) { return div_by_recip2_flag(a, V, Vinv, Vlo, inexact); });
  R gsum[5][3];
  bool exact_done = false;
  if constexpr (std::is_same<R, double>::value) {
    if (inexact) {  // rare: tiny quotients; redo the cell's sums with IEEE division
      // (a lane with !valid recomputes a real cell: it writes that cell's own bits)
      gradient_exact(t, g, W, grad, c);
#pragma unroll
      for (int k = 0; k < 5; ++k)
#pragma unroll
        for (int d = 0; d < 3; ++d) gsum[k][d] = grad[(3 * k + d) * C + c];
      exact_done = true;
    }
  }
  if (!exact_done) {
#pragma unroll
    for (int k = 0; k < 5; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        gsum[k][d] = zero_plus(acc[k][d]);  // green_gauss_gradient_sum: 0 + sum
        if (valid) grad[(3 * k + d) * C + c] = gsum[k][d];
      }
  }
  if constexpr (MODE > 0) {
    R mn[5], mx[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      mn[k] = ex[k].min();
      mx[k] = ex[k].max();
    }
    if constexpr (kWarpVenkat<R, MODE, WARP>) {
      venkat_warp(t, g, wc, mn, mx, gsum, phi, c, valid, (ac & 2) != 0, venkat_warp_buf());
    } else if constexpr (MODE == 1 && std::is_same<R, double>::value) {
      if (ac & 2) venkat_cell<true>(t, g, wc, mn, mx, gsum, phi, c);
      else venkat_cell<false>(t, g, wc, mn, mx, gsum, phi, c);
    } else {
      if (ac & 2) limiter_cell<R, MODE, true>(t, g, wc, mn, mx, gsum, phi, c);
      else limiter_cell<R, MODE, false>(t, g, wc, mn, mx, gsum, phi, c);
    }
  }
}

// Roe (+ viscous) flux of an internal face whose frame is aligned with axis D.
template <class R, bool VISC, int D>
__device__ __forceinline__ void face_flux_axis(const TopoView& t, const GeomView<R>& g, const R* __restrict__ grad,
                                               const R pl[5], const R pr[5], const Transport& tr, int f, int L,
                                               int Rc, R flux[5]) {
  constexpr int T = (D + 2) % 3, B = (D + 1) % 3;
  const int C = t.C, F = t.F;
  const R nD = g.fn[D * F + f];
  roe_flux_axis<R, D>(pl, pr, nD, g.fnu[D * F + f], g.ftu[T * F + f], g.fbu[B * F + f], g.fnn[f], flux);
  if (VISC) {
    R pf[5], gf[5][3], vf[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      pf[k] = halve(pl[k] + pr[k]);
#pragma unroll
      for (int d = 0; d < 3; ++d) gf[k][d] = halve(grad[(3 * k + d) * C + L] + grad[(3 * k + d) * C + Rc]);
    }
    viscous_flux_axis<R, D>(gf, pf, nD, tr, vf);
#pragma unroll
    for (int k = 0; k < 5; ++k) flux[k] -= vf[k];
  }
}

template <class R, bool SECOND, bool VISC>
__device__ __forceinline__ void internal_flux_face(const TopoView& t, const GeomView<R>& g, const R* __restrict__ W,
                                                   const R* __restrict__ grad, const R* __restrict__ phi,
                                                   const Transport& tr, R* __restrict__ fflux, int f) {
  const int C = t.C, F = t.F;
  const int L = t.fconn[f];
  const int Rc = t.fconn[F + f];
  R pl[5], pr[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    pl[k] = W[k * C + L];
    pr[k] = W[k * C + Rc];
  }
  const int cls = t.fclass[f];
  if (SECOND) {
    if (cls < 3) {
      // Offsets nonzero only along D = cls: the serial dot product
      // 0 + dx*gx + dy*gy + dz*gz adds signed-zero products that cannot
      // change an accumulator starting at +0 (finite gradients), so only the
      // D term is evaluated.
      const int D = cls;
      const R dl = g.dL[D * F + f], dr = g.dR[D * F + f];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        if constexpr (std::is_same<R, float>::value) {
          // Mixed form: one fused multiply-add per side (no reference bits to keep).
          pl[k] = fmaf(dl * grad[(3 * k + D) * C + L], phi[k * C + L], pl[k]);
          pr[k] = fmaf(dr * grad[(3 * k + D) * C + Rc], phi[k * C + Rc], pr[k]);
        } else {
          const R tl = zero_plus(dl * grad[(3 * k + D) * C + L]);
          const R trr = zero_plus(dr * grad[(3 * k + D) * C + Rc]);
          pl[k] += tl * phi[k * C + L];
          pr[k] += trr * phi[k * C + Rc];
        }
      }
    } else {
      const R dl[3] = {g.dL[f], g.dL[F + f], g.dL[2 * F + f]};
      const R dr[3] = {g.dR[f], g.dR[F + f], g.dR[2 * F + f]};
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        R tl = 0, trr = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          tl += dl[d] * grad[(3 * k + d) * C + L];
          trr += dr[d] * grad[(3 * k + d) * C + Rc];
        }
        pl[k] += tl * phi[k * C + L];
        pr[k] += trr * phi[k * C + Rc];
      }
    }
  }
  R flux[5];
  // Classes 0..5 have axis-aligned frames (axis cls % 3); class 6 takes the
  // general path.
  const int axis = cls < 6 ? cls % 3 : 3;
  if (axis == 0) face_flux_axis<R, VISC, 0>(t, g, grad, pl, pr, tr, f, L, Rc, flux);
  else if (axis == 1) face_flux_axis<R, VISC, 1>(t, g, grad, pl, pr, tr, f, L, Rc, flux);
  else if (axis == 2) face_flux_axis<R, VISC, 2>(t, g, grad, pl, pr, tr, f, L, Rc, flux);
  else {
    const FaceFrame<R> fr = load_frame<R>(g, f, F);
    roe_flux<R>(pl, pr, fr, flux);
    if (VISC) {
      R pf[5], gf[5][3], vf[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        pf[k] = R(0.5) * (pl[k] + pr[k]);
#pragma unroll
        for (int d = 0; d < 3; ++d) gf[k][d] = R(0.5) * (grad[(3 * k + d) * C + L] + grad[(3 * k + d) * C + Rc]);
      }
      viscous_flux<R>(gf, pf, fr.n, tr, vf);
#pragma unroll
      for (int k = 0; k < 5; ++k) flux[k] -= vf[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) fflux[static_cast<size_t>(f) * 5 + k] = flux[k];
}

// Boundary faces; each writes the contribution its cell adds to the residual.
template <class R>
__device__ __forceinline__ void bc_flux_face(const TopoView& t, const GeomView<R>& g, const R* __restrict__ W,
                                             const Transport& tr, const InflowState& inflow, R* __restrict__ fflux,
                                             int i) {
  const int C = t.C, F = t.F;
  const int f = t.Fi + i;
  const int c = t.fconn[f];
  const int e0 = t.nbc_type[0], e1 = e0 + t.nbc_type[1], e2 = e1 + t.nbc_type[2];
  R pl[5], pr[5], flux[5], out[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) pl[k] = W[k * C + c];
  const FaceFrame<R> fr = load_frame<R>(g, f, F);
  if (i < e0) {  // Extrapolate_BC.h:70-100
    roe_flux<R>(pl, pl, fr, flux);
#pragma unroll
    for (int k = 0; k < 5; ++k) out[k] = -flux[k];
  } else if (i < e1) {  // Tangent_BC.h:72-121
    reflect_state<R>(fr.n, fr.nn, pl, pr);
    roe_flux<R>(pl, pr, fr, flux);
#pragma unroll
    for (int k = 0; k < 5; ++k) out[k] = -flux[k];
  } else if (i < e2) {  // NoSlip_BC.h:77-155
    reflect_state<R>(fr.n, fr.nn, pl, pr);
    roe_flux<R>(pl, pr, fr, flux);
    R pf[5], gf[5][3], vf[5];
    pf[0] = pl[0]; pf[1] = R(0.0); pf[2] = R(0.0); pf[3] = R(0.0); pf[4] = pl[4];
    R dist = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const R dx = g.dL[d * F + f];
      dist += dx * dx;
    }
    const R inv_d = R(1.0) / dsqrt<R>(dist);
#pragma unroll
    for (int k = 0; k < 5; ++k)
#pragma unroll
      for (int d = 0; d < 3; ++d) gf[k][d] = (pf[k] - pl[k]) * fr.nu[d] * inv_d;
    viscous_flux<R>(gf, pf, fr.n, tr, vf);
#pragma unroll
    for (int k = 0; k < 5; ++k) out[k] = -flux[k] + vf[k];
  } else {  // Inflow_BC.h:73-109
    double vi[5];
    primitives(inflow.u, vi);
#pragma unroll
    for (int k = 0; k < 5; ++k) pr[k] = R(vi[k]);
    roe_flux<R>(pl, pr, fr, flux);
#pragma unroll
    for (int k = 0; k < 5; ++k) out[k] = -flux[k];
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) fflux[static_cast<size_t>(f) * 5 + k] = out[k];
}

// Ordered residual gather + RK4 update + primitives of the next stage state.
// cell_flux: the reference's -DCELL_FLUX reduction, r = 0 + sum over the
// slots (in slot order) of dt/V * flux (Flux.h:214-224), instead of
// r = 0 + dt/V * (0 + sum of the fluxes in the atomic order).
template <class R>
__device__ __forceinline__ void residual_cell(const TopoView& t, const R* __restrict__ fflux, double* __restrict__ Un,
                                              double* __restrict__ Unp1, R* __restrict__ W,
                                              double* __restrict__ res_out, double dt, int stage, bool cell_flux,
                                              int c) {
  const int C = t.C;
  // dt/V as the reference rounds it (div_by_recip returns the IEEE quotient);
  // the mixed form multiplies by 1/V.
  const double dtv = std::is_same<R, double>::value ? div_by_recip(dt, t.vol[c], t.vinv[c]) : dt * t.vinv[c];
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if constexpr (std::is_same<R, float>::value) {
    if (!cell_flux) {
      // Mixed form: each component's sum of the cell's FP32 face fluxes is
      // the exact sum rounded once to FP64 (exact_sum_f32, integer pipe), not
      // five FP64 additions; the FP64 pipe keeps the dt/V scaling and the
      // RK4 update.
      uint32_t bits[kMaxCellFaces][5];
#pragma unroll
      for (int s = 0; s < kMaxCellFaces; ++s) {
        const int code = t.csr_flux[s * C + c];
        const int f = code >> 1;
        const uint32_t flip = ((code & 1) && f < t.Fi) ? 0x80000000u : 0u;  // sign flip as a bit
        const R* fp = fflux + static_cast<size_t>(code < 0 ? 0 : f) * 5;
#pragma unroll
        for (int k = 0; k < 5; ++k) bits[s][k] = code < 0 ? 0u : (__float_as_uint(fp[k]) ^ flip);
      }
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const uint32_t u[kMaxCellFaces] = {bits[0][k], bits[1][k], bits[2][k], bits[3][k], bits[4][k], bits[5][k]};
        bool exact = true;
        acc[k] = exact_sum_f32(u, exact);
        if (!exact) {  // rare: a value far below the largest, or not finite
          double a = 0.0;
#pragma unroll
          for (int s = 0; s < kMaxCellFaces; ++s) a += widen_exact(__uint_as_float(u[s]));
          acc[k] = a;
        }
      }
    }
  }
#pragma unroll
  for (int s = 0; s < kMaxCellFaces; ++s) {
    if (std::is_same<R, float>::value && !cell_flux) break;  // summed above
    const int code = t.csr_flux[s * C + c];
    if (code < 0) continue;
    const int f = code >> 1;
    const bool neg = (code & 1) && f < t.Fi;
    const R* fp = fflux + static_cast<size_t>(f) * 5;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const double v = negate_if(to_double<R>(fp[k]), neg);  // sign flip on the integer pipe
      if (cell_flux) {
        acc[k] = acc[k] + dtv * v;
      } else {
        // the plain form adds to +0 as the reference does; with the first
        // slot present its term is 0 + v
        acc[k] = s == 0 ? zero_plus(v) : acc[k] + v;
      }
    }
  }
  // RK4 coefficients (TimeSolverExplicitRK4.h:188-195): beta of this stage and
  // alpha of the stage that follows (alpha[0] = 0 after the last stage).
  double beta, alpha_next;
  switch (stage) {
    case 0: beta = 1.0 / 6.0; alpha_next = 1.0 / 2.0; break;
    case 1: beta = 1.0 / 3.0; alpha_next = 1.0 / 2.0; break;
    case 2: beta = 1.0 / 3.0; alpha_next = 1.0; break;
    default: beta = 1.0 / 6.0; alpha_next = 0.0; break;
  }
  // The mixed form's ATOMICS_FLUX update takes the flux sum itself with the
  // coefficients beta dt/V and alpha dt/V (one multiply each instead of dt/V
  // times each of the 5 sums); the plain form keeps the reference's
  // res = 0 + (dt/V) sum and U + beta res.
  constexpr bool kPlain = std::is_same<R, double>::value;
  const bool fold = !kPlain && !cell_flux;
  const double cb = fold ? beta * dtv : beta;
  const double ca = fold ? alpha_next * dtv : alpha_next;
  double ut[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    // 0.0 + x as in apply_cell_flux (it only normalises a -0 result).
    const double r = cell_flux ? acc[k] : kPlain ? zero_plus(dtv * acc[k]) : acc[k];
    if (res_out) res_out[k * C + c] = fold ? dtv * acc[k] : r;
    // x + a*r: the plain form rounds the product and the sum as the
    // reference does; the mixed form (FP64 update, no reference bits to keep)
    // fuses them, an explicit fma that gives the same bits in every build.
    auto axpy = [&](double x, double a) { return kPlain ? x + a * r : fma(a, r, x); };
    // The plain form's alpha_next * r for stages 0-2: 0.5 r and 1 r, exact
    // without the FP64 multiply (the mixed form folds dt/V into ca instead).
    auto next = [&](double x) { return kPlain ? x + (stage == 2 ? r : halve(r)) : fma(ca, r, x); };
    if (stage == 0) {
      const double un = Un[k * C + c];
      Unp1[k * C + c] = axpy(un, cb);
      ut[k] = next(un);
    } else if (stage < 3) {
      const double un = Un[k * C + c];
      Unp1[k * C + c] = axpy(Unp1[k * C + c], cb);
      ut[k] = next(un);
    } else {
      const double u1 = axpy(Unp1[k * C + c], cb);
      Un[k * C + c] = u1;
      ut[k] = kPlain ? u1 + alpha_next * r : u1;  // alpha_next = 0
    }
  }
  store_primitives<R>(ut, W, C, c);
}


// ---- single-mesh kernels: one thread per cell / face ----
template <class R, int MODE>
__global__ void __launch_bounds__(kCellBlock, kSweepMinBlocks<R>) k_sweep1(TopoView t, GeomView<R> g, const R* __restrict__ W,
                                                       R* __restrict__ grad, R* __restrict__ phi) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < t.C) sweep1_cell<R, MODE>(t, g, W, grad, phi, c);
}

template <class R, bool SECOND, bool VISC>
__global__ void __launch_bounds__(kFaceBlock, kFluxMinBlocks<R, SECOND, VISC>) k_internal_flux(TopoView t, GeomView<R> g, const R* __restrict__ W,
                                                              const R* __restrict__ grad, const R* __restrict__ phi,
                                                              Transport tr, R* __restrict__ fflux) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < t.Fi) internal_flux_face<R, SECOND, VISC>(t, g, W, grad, phi, tr, fflux, f);
}

template <class R>
__global__ void __launch_bounds__(kFaceBlock) k_bc_flux(TopoView t, GeomView<R> g, const R* __restrict__ W,
                                                        Transport tr, InflowState inflow, R* __restrict__ fflux) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < t.Fb) bc_flux_face<R>(t, g, W, tr, inflow, fflux, i);
}

template <class R>
__global__ void __launch_bounds__(kCellBlock, kResidualMinBlocks<R>) k_residual(TopoView t, const R* __restrict__ fflux,
                                                         double* __restrict__ Un, double* __restrict__ Unp1,
                                                         R* __restrict__ W, double* __restrict__ res_out, double dt,
                                                         int stage, bool cell_flux) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < t.C) residual_cell<R>(t, fflux, Un, Unp1, W, res_out, dt, stage, cell_flux, c);
}

// ---- batched kernels: persistent grid over chunks of (segment, first item) ----
// Each block takes whole chunks; a chunk holds blockDim.x consecutive items of
// one segment. The chunk count is read from device memory so that a captured
// graph stays valid when the batch membership changes.
template <class R, int MODE>
__global__ void __launch_bounds__(256, std::is_same<R, double>::value ? 2 : 0) kb_sweep1(const Segment<R>* __restrict__ segs, const int2* __restrict__ chunks,
                                                 const int* __restrict__ nchunks) {
  const int n = *nchunks;
  for (int ch = blockIdx.x; ch < n; ch += gridDim.x) {
    const int2 cs = chunks[ch];
    const Segment<R>& sg = segs[cs.x];
    const int c = cs.y + threadIdx.x;
    if constexpr (kWarpVenkat<R, MODE, true>) {
      sweep1_cell<R, MODE, true>(sg.t, sg.g, sg.b.W, sg.b.grad, sg.b.phi, c < sg.t.C ? c : sg.t.C - 1, c < sg.t.C);
    } else if (c < sg.t.C) {
      sweep1_cell<R, MODE>(sg.t, sg.g, sg.b.W, sg.b.grad, sg.b.phi, c);
    }
  }
}

template <class R, bool SECOND, bool VISC>
__global__ void __launch_bounds__(256) kb_internal_flux(const Segment<R>* __restrict__ segs,
                                                        const int2* __restrict__ chunks,
                                                        const int* __restrict__ nchunks, Transport tr) {
  const int n = *nchunks;
  for (int ch = blockIdx.x; ch < n; ch += gridDim.x) {
    const int2 cs = chunks[ch];
    const Segment<R>& sg = segs[cs.x];
    const int f = cs.y + threadIdx.x;
    if (f < sg.t.Fi) internal_flux_face<R, SECOND, VISC>(sg.t, sg.g, sg.b.W, sg.b.grad, sg.b.phi, tr, sg.b.fflux, f);
  }
}

template <class R>
__global__ void __launch_bounds__(256) kb_bc_flux(const Segment<R>* __restrict__ segs, const int2* __restrict__ chunks,
                                                  const int* __restrict__ nchunks, Transport tr) {
  const int n = *nchunks;
  for (int ch = blockIdx.x; ch < n; ch += gridDim.x) {
    const int2 cs = chunks[ch];
    const Segment<R>& sg = segs[cs.x];
    const int i = cs.y + threadIdx.x;
    if (i < sg.t.Fb) bc_flux_face<R>(sg.t, sg.g, sg.b.W, tr, sg.inflow, sg.b.fflux, i);
  }
}

template <class R>
__global__ void __launch_bounds__(256) kb_residual(const Segment<R>* __restrict__ segs, const int2* __restrict__ chunks,
                                                   const int* __restrict__ nchunks, int stage, bool cell_flux) {
  const int n = *nchunks;
  for (int ch = blockIdx.x; ch < n; ch += gridDim.x) {
    const int2 cs = chunks[ch];
    const Segment<R>& sg = segs[cs.x];
    const int c = cs.y + threadIdx.x;
    if (c < sg.t.C)
      residual_cell<R>(sg.t, sg.b.fflux, sg.s.Un, sg.s.Unp1, sg.b.W, sg.s.res, sg.dt, stage, cell_flux, c);
  }
}

// ---- one launch for whole batch steps: phases separated by a grid barrier ----
// The batch's kernels of one RK stage become phases of one persistent
// kernel: (A) Green-Gauss/limiter sweep and boundary-face flux, (B)
// internal-face flux, (C) residual and RK4 update; a grid-wide barrier
// separates the phases and the stages, so a whole ma_batch_step is one
// launch. It is launched cooperatively (all blocks resident, checked by the
// runtime at launch), so every barrier completes; each wait is still bounded
// (kGridBarrierTimeoutNs): a block that waits longer sets *err, every block
// then leaves at its next barrier, and the host reports the error. Every
// item is computed by the device functions of the per-kind kernels, so the
// bits are the same.
constexpr unsigned long long kGridBarrierTimeoutNs = 5000000000ull;  // 5 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Sense by generation: the last block to arrive resets the count and bumps
// the generation; the others wait for the bump. Returns false when the
// barrier gave up (timeout here or in another block).
__device__ __forceinline__ bool grid_barrier(unsigned* count, unsigned* gen, int* err,
                                             unsigned long long timeout_ns = kGridBarrierTimeoutNs) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = gen;
    volatile int* verr = err;
    const unsigned g = *vgen;
    __threadfence();
    int ok = *verr == 0;
    if (atomicAdd(count, 1u) + 1u == gridDim.x) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      unsigned spins = 0;
      while (ok && *vgen == g) {
        __nanosleep(64);
        if (*verr != 0) ok = 0;
        // The time limit, and an iteration limit that holds even if the
        // timer did not advance (2^28 sleeps of at least 64 ns: over 17 s).
        else if (global_ns() - t0 > timeout_ns || ++spins > (1u << 28)) {
          atomicExch(err, 1);
          ok = 0;
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

struct GridSync {
  unsigned* count;
  unsigned* gen;
  int* err;
};

// FP64: two resident blocks of 256 (128 registers, 56-84 bytes spilled to L1)
// instead of one at 166 registers: 234.6 -> 243.0 Mcell-stage/s on the
// 64-box Sod ensemble.
template <class R, int MODE, bool SECOND, bool VISC>
__global__ void __launch_bounds__(256, std::is_same<R, double>::value ? 2 : 0) kb_steps(const Segment<R>* segs, const int2* c_sweep, const int2* c_flux,
                                                const int2* c_bc, const int2* c_res, const int* nchunks, Transport tr,
                                                bool cell_flux, int nsteps, GridSync gs) {
  // The sweep phase exists for second-order or viscous runs only; without it
  // the kernel carries no sweep code (fewer registers, more resident blocks).
  constexpr bool has_sweep = SECOND || VISC;
  const int n0 = nchunks[0], n1 = nchunks[1], n2 = nchunks[2], n3 = nchunks[3];
  for (int step = 0; step < nsteps; ++step) {
    for (int stage = 0; stage < 4; ++stage) {
      if constexpr (has_sweep) {
        for (int ch = blockIdx.x; ch < n0; ch += gridDim.x) {
          const int2 cs = c_sweep[ch];
          const Segment<R>& sg = segs[cs.x];
          const int c = cs.y + threadIdx.x;
          if constexpr (kWarpVenkat<R, MODE, true>) {
            sweep1_cell<R, MODE, true>(sg.t, sg.g, sg.b.W, sg.b.grad, sg.b.phi, c < sg.t.C ? c : sg.t.C - 1,
                                       c < sg.t.C);
          } else if (c < sg.t.C) {
            sweep1_cell<R, MODE>(sg.t, sg.g, sg.b.W, sg.b.grad, sg.b.phi, c);
          }
        }
      }
      for (int ch = blockIdx.x; ch < n2; ch += gridDim.x) {
        const int2 cs = c_bc[ch];
        const Segment<R>& sg = segs[cs.x];
        const int i = cs.y + threadIdx.x;
        if (i < sg.t.Fb) bc_flux_face<R>(sg.t, sg.g, sg.b.W, tr, sg.inflow, sg.b.fflux, i);
      }
      // The internal-face flux reads the sweep's gradients and limiter; with
      // no sweep it shares the first phase.
      if (has_sweep && !grid_barrier(gs.count, gs.gen, gs.err)) return;
      for (int ch = blockIdx.x; ch < n1; ch += gridDim.x) {
        const int2 cs = c_flux[ch];
        const Segment<R>& sg = segs[cs.x];
        const int f = cs.y + threadIdx.x;
        if (f < sg.t.Fi)
          internal_flux_face<R, SECOND, VISC>(sg.t, sg.g, sg.b.W, sg.b.grad, sg.b.phi, tr, sg.b.fflux, f);
      }
      if (!grid_barrier(gs.count, gs.gen, gs.err)) return;
      for (int ch = blockIdx.x; ch < n3; ch += gridDim.x) {
        const int2 cs = c_res[ch];
        const Segment<R>& sg = segs[cs.x];
        const int c = cs.y + threadIdx.x;
        if (c < sg.t.C)
          residual_cell<R>(sg.t, sg.b.fflux, sg.s.Un, sg.s.Unp1, sg.b.W, sg.s.res, sg.dt, stage, cell_flux, c);
      }
      const bool last = step == nsteps - 1 && stage == 3;
      if (!last && !grid_barrier(gs.count, gs.gen, gs.err)) return;
    }
  }
}

template <class R>
cudaError_t launch_batch_steps_impl(const PathConfig& cfg, const Segment<R>* segs, const BatchLaunch& bl,
                                    int nsteps, unsigned* barrier_words, int* err, int block, int grid,
                                    cudaStream_t stream) {
  const Transport tr = cfg.transport;
  const int mode = !cfg.second_order ? 0 : (cfg.limiter == 1 ? 2 : 1);
  GridSync gs{barrier_words, barrier_words + 1, err};
  const int2* c0 = bl.chunks[0];
  const int2* c1 = bl.chunks[1];
  const int2* c2 = bl.chunks[2];
  const int2* c3 = bl.chunks[3];
  const int* nc = bl.nchunks;
  bool cf = cfg.cell_flux;
  void* args[] = {(void*)&segs, (void*)&c0, (void*)&c1, (void*)&c2, (void*)&c3, (void*)&nc, (void*)&tr,
                  (void*)&cf, (void*)&nsteps, (void*)&gs};
  const void* fn = nullptr;
  if (mode == 0) {
    fn = cfg.viscous ? (const void*)kb_steps<R, 0, false, true> : (const void*)kb_steps<R, 0, false, false>;
  } else if (mode == 1) {
    fn = cfg.viscous ? (const void*)kb_steps<R, 1, true, true> : (const void*)kb_steps<R, 1, true, false>;
  } else {
    fn = cfg.viscous ? (const void*)kb_steps<R, 2, true, true> : (const void*)kb_steps<R, 2, true, false>;
  }
  const size_t smem = (mode == 1 && std::is_same<R, double>::value) ? block / 32 * kVenkatBufBytes : 0;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), args, smem, stream);
}

// Resident blocks per SM of the single-launch kernel for this configuration.
template <class R>
cudaError_t batch_steps_occupancy_impl(const PathConfig& cfg, int block, int* blocks_per_sm) {
  const int mode = !cfg.second_order ? 0 : (cfg.limiter == 1 ? 2 : 1);
  const void* fn = nullptr;
  if (mode == 0) {
    fn = cfg.viscous ? (const void*)kb_steps<R, 0, false, true> : (const void*)kb_steps<R, 0, false, false>;
  } else if (mode == 1) {
    fn = cfg.viscous ? (const void*)kb_steps<R, 1, true, true> : (const void*)kb_steps<R, 1, true, false>;
  } else {
    fn = cfg.viscous ? (const void*)kb_steps<R, 2, true, true> : (const void*)kb_steps<R, 2, true, false>;
  }
  const size_t smem = (mode == 1 && std::is_same<R, double>::value) ? block / 32 * kVenkatBufBytes : 0;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, block, smem);
}

// Failure path of the grid barrier: block 0 waits at a barrier that block 1
// never reaches (it returns at once), so the wait runs out after timeout_ns;
// out[0] = whether block 0 passed the barrier (0 expected), out[1] = the
// error word afterwards (1 expected).
__global__ void k_debug_barrier_timeout(unsigned* words, int* err, unsigned long long timeout_ns, int* out) {
  if (blockIdx.x != 0) return;
  const bool passed = grid_barrier(words, words + 1, err, timeout_ns);
  if (threadIdx.x == 0) {
    out[0] = passed ? 1 : 0;
    out[1] = *static_cast<volatile int*>(err);
  }
}

// Primitives of U_n + 0 * res with res = 0 (first stage after set_state).
template <class R>
__global__ void k_init_primitives(int C, const double* __restrict__ Un, R* __restrict__ W, double zero) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  double ut[5], v[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) ut[k] = Un[k * C + c] + 0.0 * zero;
  (void)v;
  store_primitives<R>(ut, W, C, c);
}

inline unsigned blocks_for(int n, int bs) { return static_cast<unsigned>((n + bs - 1) / bs); }

template <class R>
cudaError_t launch_init_primitives_impl(const TopoView& t, const StateBuffers& s, const StageBuffers<R>& b,
                                        cudaStream_t stream) {
  if (t.C == 0) return cudaSuccess;
  k_init_primitives<R><<<blocks_for(t.C, kCellBlock), kCellBlock, 0, stream>>>(t.C, s.Un, b.W, 0.0);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_stage_impl(const TopoView& t, const GeomView<R>& g, const PathConfig& cfg, const StateBuffers& s,
                              const StageBuffers<R>& b, int stage, cudaStream_t stream, unsigned kernels) {
  if (t.C == 0) return cudaSuccess;
  const unsigned gc = blocks_for(t.C, kCellBlock);
  if (!(kernels & kSweep1)) {
  } else if (cfg.second_order) {
    if (cfg.limiter == 1)
      k_sweep1<R, 2><<<gc, kCellBlock, 0, stream>>>(t, g, b.W, b.grad, b.phi);
    else
      k_sweep1<R, 1><<<gc, kCellBlock, 0, stream>>>(t, g, b.W, b.grad, b.phi);
  } else if (cfg.viscous) {
    k_sweep1<R, 0><<<gc, kCellBlock, 0, stream>>>(t, g, b.W, b.grad, b.phi);
  }
  if (t.Fi > 0 && (kernels & kInternalFlux)) {
    const unsigned gf = blocks_for(t.Fi, kFaceBlock);
    if (cfg.second_order) {
      if (cfg.viscous)
        k_internal_flux<R, true, true><<<gf, kFaceBlock, 0, stream>>>(t, g, b.W, b.grad, b.phi, cfg.transport, b.fflux);
      else
        k_internal_flux<R, true, false><<<gf, kFaceBlock, 0, stream>>>(t, g, b.W, b.grad, b.phi, cfg.transport, b.fflux);
    } else {
      if (cfg.viscous)
        k_internal_flux<R, false, true><<<gf, kFaceBlock, 0, stream>>>(t, g, b.W, b.grad, b.phi, cfg.transport, b.fflux);
      else
        k_internal_flux<R, false, false><<<gf, kFaceBlock, 0, stream>>>(t, g, b.W, b.grad, b.phi, cfg.transport, b.fflux);
    }
  }
  if (t.Fb > 0 && (kernels & kBcFlux)) {
    InflowState inflow;
    for (int k = 0; k < 5; ++k) inflow.u[k] = cfg.inflow[k];
    k_bc_flux<R><<<blocks_for(t.Fb, kFaceBlock), kFaceBlock, 0, stream>>>(t, g, b.W, cfg.transport, inflow, b.fflux);
  }
  if (kernels & kResidual) {
    // Meshes of up to two blocks of 256 cells per SM (152 SMs): 32-cell blocks
    // spread the cells over every SM; 256-cell blocks would leave SMs idle.
    const int rb = t.C <= kSmallMeshCells ? 32 : kCellBlock;
    k_residual<R><<<blocks_for(t.C, rb), rb, 0, stream>>>(t, b.fflux, s.Un, s.Unp1, b.W, s.res, cfg.dt, stage,
                                                         cfg.cell_flux);
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_batch_stage_impl(const PathConfig& cfg, const Segment<R>* segs, const BatchLaunch& bl, int stage,
                                    cudaStream_t stream, unsigned kernels) {
  const Transport tr = cfg.transport;
  if ((kernels & kSweep1) && (cfg.second_order || cfg.viscous)) {
    const dim3 g(bl.grid[0]), b(bl.block[0]);
    if (!cfg.second_order)
      kb_sweep1<R, 0><<<g, b, 0, stream>>>(segs, bl.chunks[0], bl.nchunks + 0);
    else if (cfg.limiter == 1)
      kb_sweep1<R, 2><<<g, b, 0, stream>>>(segs, bl.chunks[0], bl.nchunks + 0);
    else
      kb_sweep1<R, 1><<<g, b, kWarpVenkat<R, 1, true> ? bl.block[0] / 32 * kVenkatBufBytes : 0, stream>>>(
          segs, bl.chunks[0], bl.nchunks + 0);
  }
  if (kernels & kInternalFlux) {
    const dim3 g(bl.grid[1]), b(bl.block[1]);
    if (cfg.second_order) {
      if (cfg.viscous)
        kb_internal_flux<R, true, true><<<g, b, 0, stream>>>(segs, bl.chunks[1], bl.nchunks + 1, tr);
      else
        kb_internal_flux<R, true, false><<<g, b, 0, stream>>>(segs, bl.chunks[1], bl.nchunks + 1, tr);
    } else {
      if (cfg.viscous)
        kb_internal_flux<R, false, true><<<g, b, 0, stream>>>(segs, bl.chunks[1], bl.nchunks + 1, tr);
      else
        kb_internal_flux<R, false, false><<<g, b, 0, stream>>>(segs, bl.chunks[1], bl.nchunks + 1, tr);
    }
  }
  if (kernels & kBcFlux) kb_bc_flux<R><<<bl.grid[2], bl.block[2], 0, stream>>>(segs, bl.chunks[2], bl.nchunks + 2, tr);
  if (kernels & kResidual)
    kb_residual<R><<<bl.grid[3], bl.block[3], 0, stream>>>(segs, bl.chunks[3], bl.nchunks + 3, stage, cfg.cell_flux);
  return cudaGetLastError();
}

}  // namespace
}  // namespace dev
}  // namespace miniaero
