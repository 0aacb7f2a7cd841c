// eval.cuh -- pair-evaluation kernels: s, ds/dx, virial, ds/dR_0, ds/dD_0.
//
// Each kernel is templated on an EvalMode (kargs.h): EVAL_S accumulates s
// only (the cheap forward under autograd), EVAL_DERIV adds the per-atom
// derivatives and the virial (CoordinationBase::calculate), EVAL_PARAM also
// the switching-parameter gradients.  The backward pass is EVAL_PARAM with the
// derivatives scaled by dV/ds in the finalize kernel.
//
// Parameter gradient of one pair inside d_max (x = (r - d0)/r0, S = stretch):
//   dsigma/dR_0 = -dfunc r (r - d0) / r0 + c_r0 (sigma - 1)
//   dsigma/dD_0 = -dfunc r               + c_d0 (sigma - 1)
// with dfunc = S f'(x)/(r0 r) the reference's dfunc and c_p the dependence of
// the stretch constants on p (host_setup.cpp).
#pragma once
#include <type_traits>

#include "kernels.cuh"

namespace coordgpu {
namespace {
// CONTACT_MATRIX's weights (adjmat/ContactMatrix.h:99-107): no bond when
// r^2 < epsilon ("atoms can't be bonded to themselves") and none, nor a
// derivative, when sigma < epsilon; epsilon is DBL_EPSILON (tools/Tools.h).
constexpr double kBondEps = 2.220446049250313e-16;


__device__ __forceinline__ void vir_sub(double v[kPartials], const double dd[3], const double d[3]) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) v[1 + 3 * i + j] -= dd[i] * d[j];
}

__device__ __forceinline__ void param_acc64(const SwitchParams &sw, double r2, double sig, double df, double part[]) {
  if (r2 <= sw.dmax_2) {
    const double r = sqrt(r2);
    part[10] += -df * r * (r - sw.d0) * sw.invr0 + sw.c_r0 * (sig - 1.0);
    part[11] += -df * r + sw.c_d0 * (sig - 1.0);
  }
}

// ---------------------------------------------------------------------------
// neighbour list, FP64: one thread per row (rank), warp = slice
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256) k_eval_nl64(KArgs a, SwitchParams sw) {
  const int f = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const size_t fo = (size_t)f * a.ns;
  double part[kPartials];
#pragma unroll
  for (int k = 0; k < kPartials; k++) part[k] = 0.0;
  if (r < a.ns) {
    const FrameConst &fc = a.fc[f];
    const int len = a.row_len[fo + r];
    const double4 xr4 = a.x64[fo + r];  // .w: the row's upstream g in EVAL_VJP
    const double xr[3] = {xr4.x, xr4.y, xr4.z};
    double accr[3] = {0.0, 0.0, 0.0};
    double accw = 0.0;
    const uint32_t *e = a.ell + ((size_t)f * a.nslices + (r >> 5)) * (size_t)a.cap * 32 + lane;
    for (int k = 0; k < len; k++) {
      const uint32_t ent = __ldg(e + (size_t)k * 32);
      const int p = (int)(ent & kRankMask);
      const bool rfirst = (ent & kOrientBit) != 0;
      const double4 xp4 = a.x64[fo + p];
      const double xp[3] = {xp4.x, xp4.y, xp4.z};
      double d[3], df;
      int sr = 0, sp = 0;  // slots, for the sibling CVs' per-atom data
      if (a.cv != COORD_CV_COORDINATION) {
        sr = a.slot_of_rank[fo + r];
        sp = a.slot_of_rank[fo + p];
      }
      double sig = rfirst ? pair_fp64(a, sw, fc, xr, xp, sr, sp, d, df) : pair_fp64(a, sw, fc, xp, xr, sp, sr, d, df);
      if (MODE >= EVAL_PERATOM && (mod2(d) < kBondEps || sig < kBondEps)) {
        sig = 0.0;
        df = 0.0;
      }
      if (MODE == EVAL_VJP) df *= xr4.w + xp4.w;
      if (MODE == EVAL_PERATOM && sig != 0.0) {
        atomicAdd(a.accw64 + fo + p, sig);
        accw += sig;
      }
      part[0] += sig;
      if (MODE >= EVAL_DERIV && df != 0.0) {  // a pair beyond d_max adds nothing
        const double dd[3] = {df * d[0], df * d[1], df * d[2]};
        double *accp = a.acc64 + (fo + p) * 3;
        // deriv[first] -= dd; deriv[second] += dd  (CoordinationBase.cpp:196-206)
        const double sgn = rfirst ? 1.0 : -1.0;
        for (int q = 0; q < 3; q++) {
          accr[q] -= sgn * dd[q];
          atomicAdd(accp + q, sgn * dd[q]);
        }
        vir_sub(part, dd, d);
      }
      if (MODE == EVAL_PARAM) param_acc64(sw, mod2(d), sig, df, part);
    }
    if (MODE >= EVAL_DERIV) {
      double *acc = a.acc64 + (fo + r) * 3;
      for (int q = 0; q < 3; q++) atomicAdd(acc + q, accr[q]);
    }
    if (MODE == EVAL_PERATOM && accw != 0.0) atomicAdd(a.accw64 + fo + r, accw);
  }
  block_partials_finish(a, f, part, gridDim.x);
}

// ---------------------------------------------------------------------------
// neighbour list, FP64, COORDINATION on orthorhombic frames: the drop-in's
// fast form.  One warp per slice.  Each lane screens its row's entries with
// the FP32 distance of the fixed-point positions; an entry whose FP32 r^2 is
// above d_max^2 (1 + 2e-6) has an FP64 r^2 above d_max^2 (the FP32 value is
// within about 4e-7 of it), so the reference gives it sigma = dfunc = 0 and
// it adds nothing.  The other entries go to a queue in shared memory, and
// the warp evaluates them 32 at a time with every lane busy, in FP64 with the
// reference's operations (pair_fp64, as k_eval_nl64).  Both atoms'
// derivatives go to the FP64 accumulators by atomic adds; s, the virial and
// the parameter sums stay in the evaluating lane.  The FP64 pipe runs only
// for queued pairs and never idles lanes on a divergent branch.
// ---------------------------------------------------------------------------
// The reference's minimum-image difference v2 - v1 along one orthorhombic
// axis, d = ((v2 - v1) * invBox + 100 - t) * box with t = int(x + 0.5) of
// Tools::pbc (Tools.h:557-563), given the image shift n = round((v2 - v1) /
// L) as an integer: t = 100 + n then, and it is formed exactly in FP64 from
// the integer by the 1.5 * 2^52 bias (no integer-to-double conversion).  The
// operations on the values are the reference's, in its order, so the result
// is bit-identical; only the conversions of Tools::pbc are avoided.
__device__ __forceinline__ double pbc_axis_shift(double v1, double v2, double invbox, double box, int n) {
  const double x = (v2 - v1) * invbox + 100.0;
  const double t = __longlong_as_double(0x4338000000000000LL + (long long)(100 + n)) - 6755399441055744.0;
  return (x - t) * box;
}

// round((v_b - v_a) / L) along one axis from the 64-bit fixed-point positions
// (high word ha/hb, low word qa/qb), exact while |v_b - v_a| < 0.45 L
__device__ __forceinline__ int image_shift(int ha, uint32_t qa, int hb, uint32_t qb) {
  const long long low = (long long)qb - (long long)qa;           // in (-2^32, 2^32)
  const long long carry = (low - (long long)(int)(qb - qa)) >> 32;  // -1, 0 or 1
  return hb - ha + (int)carry;
}

// fixedRational<2 NH>::calculateSqr (SwitchingFunction.cpp:203-215) with N
// known at compile time: the operations of sw_calculate_sqr, in its order.
template <int NH> __device__ __forceinline__ double ratfix_sqr(const SwitchParams &s, double d2, double &df) {
  if (!(d2 <= s.dmax_2)) {
    df = 0.0;
    return 0.0;
  }
  const double rdist = d2 * s.invr0_2;
  VD<double> r = rational_fixed<double>(NH, rdist);
  r.d *= 2.0 * s.invr0_2;
  r.f = r.f * s.stretch + s.shift;
  r.d *= s.stretch;
  df = r.d;
  return r.f;
}

template <int MODE, int kU, int NH>
__global__ void __launch_bounds__(256) k_eval_nl64q(KArgs a, SwitchParams sw, SwitchF32 s32) {
  const int f = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slice = blockIdx.x * 8 + warp;
  const size_t fo = (size_t)f * a.ns;
  const FrameConst &fc = a.fc[f];
  __shared__ uint2 queue[8][64];  // (list entry, row lane); at most 31 + 32 waiting
  double part[kPartials];
#pragma unroll
  for (int k = 0; k < kPartials; k++) part[k] = 0.0;
  if (slice < a.nslices) {  // warp-uniform
    const int r = slice * 32 + lane;
    const bool active = r < a.ns;
    const bool near_only = near_rows_only(a, f);
    const int len = active ? (near_only ? a.row_near[fo + r] : a.row_len[fo + r]) : 0;
    const int w = (near_only ? a.slice_wn : a.slice_w)[(size_t)f * a.nslices + slice];
    const uint4 *__restrict__ q = a.q + fo;
    const uint4 qr = active ? q[r] : make_uint4(0u, 0u, 0u, 0u);
    const float sx = fc.scale[0], sy = fc.scale[1], sz = fc.scale[2];
    const uint32_t *__restrict__ e = a.ell + ((size_t)f * a.nslices + slice) * (size_t)a.cap * 32 + lane;
    uint2 *const qu = queue[warp];
    const unsigned below = (1u << lane) - 1u;
    int qn = 0;  // queued entries (warp-uniform)
    // evaluates qu[0 .. n) one per lane
    auto evaluate = [&](int n) {
      if (lane >= n) return;
      const uint2 it = qu[lane];
      const int rr = slice * 32 + (int)it.y;
      const int p = (int)(it.x & kRankMask);
      const bool rfirst = (it.x & kOrientBit) != 0;
      const double4 xr4 = a.x64[fo + rr], xp4 = a.x64[fo + p];
      const double xr[3] = {xr4.x, xr4.y, xr4.z}, xp[3] = {xp4.x, xp4.y, xp4.z};
      double d[3], df, sig;
      if (fc.shift_ok && a.qhi) {
        // the reference's d = pbc(x[second] - x[first]) with the image shifts
        // taken from the integer fixed-point positions
        const uint4 qa = q[rr], qb = q[p];
        const int4 ha = a.qhi[fo + rr], hb = a.qhi[fo + p];
        const int n0 = image_shift(ha.x, qa.x, hb.x, qb.x), n1 = image_shift(ha.y, qa.y, hb.y, qb.y),
                  n2 = image_shift(ha.z, qa.z, hb.z, qb.z);
        const double *v1 = rfirst ? xr : xp, *v2 = rfirst ? xp : xr;
        const int sg = rfirst ? 1 : -1;
        d[0] = pbc_axis_shift(v1[0], v2[0], fc.pbc.invbox[0], fc.pbc.box[0], sg * n0);
        d[1] = pbc_axis_shift(v1[1], v2[1], fc.pbc.invbox[4], fc.pbc.box[4], sg * n1);
        d[2] = pbc_axis_shift(v1[2], v2[2], fc.pbc.invbox[8], fc.pbc.box[8], sg * n2);
        if constexpr (NH > 0) {
          sig = ratfix_sqr<NH>(sw, mod2(d), df);
        } else {
          const VD<double> v = sw_calculate_sqr<double>(sw, mod2(d));
          sig = v.f;
          df = v.d;
        }
      } else if constexpr (NH > 0) {
        // fixedRational<2 NH> only: the reference's distance, then the same switch
        if (rfirst)
          pbc_distance(fc.pbc, xr, xp, d);
        else
          pbc_distance(fc.pbc, xp, xr, d);
        sig = ratfix_sqr<NH>(sw, mod2(d), df);
      } else {
        sig = rfirst ? pair_fp64(a, sw, fc, xr, xp, 0, 0, d, df) : pair_fp64(a, sw, fc, xp, xr, 0, 0, d, df);
      }
      if (MODE >= EVAL_PERATOM && (mod2(d) < kBondEps || sig < kBondEps)) {
        sig = 0.0;
        df = 0.0;
      }
      if (MODE == EVAL_VJP) df *= xr4.w + xp4.w;
      if (MODE == EVAL_PERATOM && sig != 0.0) {
        atomicAdd(a.accw64 + fo + p, sig);
        atomicAdd(a.accw64 + fo + rr, sig);
      }
      part[0] += sig;
      if (MODE >= EVAL_DERIV && df != 0.0) {
        const double dd[3] = {df * d[0], df * d[1], df * d[2]};
        // deriv[first] -= dd; deriv[second] += dd  (CoordinationBase.cpp:196-206)
        const double sgn = rfirst ? 1.0 : -1.0;
        double *accp = a.acc64 + (fo + p) * 3, *accr = a.acc64 + (fo + rr) * 3;
        for (int k = 0; k < 3; k++) {
          atomicAdd(accp + k, sgn * dd[k]);
          atomicAdd(accr + k, -sgn * dd[k]);
        }
        // virial -= dd (x) d: dd = dfunc d, so the tensor is symmetric; the
        // six distinct entries by fused multiply-adds, mirrored at the end
        part[1] = fma(-dd[0], d[0], part[1]);
        part[2] = fma(-dd[0], d[1], part[2]);
        part[3] = fma(-dd[0], d[2], part[3]);
        part[5] = fma(-dd[1], d[1], part[5]);
        part[6] = fma(-dd[1], d[2], part[6]);
        part[9] = fma(-dd[2], d[2], part[9]);
      }
      if (MODE == EVAL_PARAM) param_acc64(sw, mod2(d), sig, df, part);
    };
    for (int k = 0; k < w; k += kU) {
      uint32_t en[kU];
      uint4 qp[kU];
#pragma unroll
      for (int u = 0; u < kU; u++) en[u] = (k + u < len) ? __ldcs(e + (size_t)(k + u) * 32) : 0xffffffffu;
#pragma unroll
      for (int u = 0; u < kU; u++) qp[u] = (en[u] != 0xffffffffu) ? __ldg(q + (en[u] & kRankMask)) : qr;
#pragma unroll
      for (int u = 0; u < kU; u++) {
        const float dx = fixed_delta(qr.x, qp[u].x, sx);
        const float dy = fixed_delta(qr.y, qp[u].y, sy);
        const float dz = fixed_delta(qr.z, qp[u].z, sz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool cand = en[u] != 0xffffffffu && r2 <= s32.dmax2_hi;
        const unsigned b = __ballot_sync(0xffffffffu, cand);
        if (cand) qu[qn + __popc(b & below)] = make_uint2(en[u], (uint32_t)lane);
        qn += __popc(b);
        if (qn >= 32) {
          __syncwarp();
          evaluate(32);
          __syncwarp();
          if (lane < qn - 32) qu[lane] = qu[32 + lane];
          __syncwarp();
          qn -= 32;
        }
      }
    }
    __syncwarp();
    evaluate(qn);
  }
  part[4] = part[2];
  part[7] = part[3];
  part[8] = part[6];
  block_partials_finish(a, f, part, gridDim.x);
}

// ---------------------------------------------------------------------------
// mixed precision: FP32 pair math from fixed-point positions, FP32 per-thread
// accumulation (Kahan for s), FP64 compensated block/grid sums.  NH = N/2 of
// fixedRational<N>; NH == 0 evaluates any switch type in FP32.
// ---------------------------------------------------------------------------
template <int NH>
__device__ __forceinline__ void sw32(const SwitchParams &sw, const SwitchF32 &s, float r2, float &sig, float &df) {
  if constexpr (NH > 0) {
    const float x = r2 * s.invr0_2;
    float xp = 1.0f;
#pragma unroll
    for (int i = 0; i < NH - 1; i++) xp *= x;
    // 1/(1 + x^N): the hardware's approximate reciprocal (the argument is
    // >= 1), then one Newton-Raphson step r += r (1 - y r), which leaves it
    // within about half an ulp and without the approximation's bias (the CV
    // is a sum of millions of these values, so a bias of one ulp shows as a
    // relative error of 1e-7 in s)
    const float y = fmaf(xp, x, 1.0f);
    float s0 = __fdividef(1.0f, y);
    s0 = fmaf(s0, fmaf(-y, s0, 1.0f), s0);
    sig = fmaf(s0, s.stretch, s.shift);
    df = s.c * xp * s0 * s0;
  } else {
    VD<float> v = sw_calculate_sqr<float>(sw, r2);
    sig = v.f;
    df = v.d;
  }
}

// Quantities a lane sums per slice in FP32 and totals in FP64: s, the six
// independent virial components, ds/dR_0, ds/dD_0.
constexpr int kSliceSums = 9;
// Slices a lane sums in FP32 before adding the sums to its FP64 totals.
constexpr int kFlushSlices = 4;

// Per-thread FP32 accumulators of one pair kernel.
struct Acc32 {
  float cv = 0.f, cvc = 0.f;
  float vxx = 0.f, vyy = 0.f, vzz = 0.f, vxy = 0.f, vxz = 0.f, vyz = 0.f;
  float pr0 = 0.f, pd0 = 0.f;
  // the neighbour-list pass: a plain FP32 sum over one slice's pairs of a
  // row (tens of terms), flushed into an FP64 lane total after every slice
  float cvs = 0.f;
  double cv64 = 0.0;
  // FP64 totals of the virial and parameter sums, for kernels that flush
  // their FP32 sums after every tile (flush_tile)
  double vt[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, pt[2] = {0.0, 0.0};
  template <int MODE> __device__ __forceinline__ void flush_tile() {
    if (MODE >= EVAL_DERIV) {
      vt[0] += (double)vxx;
      vt[1] += (double)vyy;
      vt[2] += (double)vzz;
      vt[3] += (double)vxy;
      vt[4] += (double)vxz;
      vt[5] += (double)vyz;
      vxx = vyy = vzz = vxy = vxz = vyz = 0.f;
    }
    if (MODE == EVAL_PARAM) {
      pt[0] += (double)pr0;
      pt[1] += (double)pd0;
      pr0 = pd0 = 0.f;
    }
  }
  __device__ __forceinline__ void add_s_slice(float sig) { cvs += sig; }
  __device__ __forceinline__ void flush_s() {
    cv64 += (double)cvs;
    cvs = 0.f;
  }
  // The warp's FP32 sums of the last slices (s in cvs, the virial, the
  // parameter gradients): summed over the warp's lanes in FP32 (a fixed
  // butterfly, so every lane holds the same value), added by lane 0 to the
  // warp's FP64 totals wt[kSliceSums], then cleared.
  template <int MODE> __device__ __forceinline__ void flush_warp(double *wt, int lane) {
    constexpr int nq = (MODE == EVAL_S) ? 1 : (MODE == EVAL_PARAM ? 9 : 7);
    float v[9] = {cvs, vxx, vyy, vzz, vxy, vxz, vyz, pr0, pd0};
#pragma unroll
    for (int k = 0; k < nq; k++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < nq; k++) wt[k] += (double)v[k];
    cvs = 0.f;
    vxx = vyy = vzz = vxy = vxz = vyz = 0.f;
    pr0 = pd0 = 0.f;
  }
  __device__ __forceinline__ void add_s(float sig) {
    const float yk = sig - cvc;
    const float tk = cv + yk;
    cvc = (tk - cv) - yk;
    cv = tk;
  }
  __device__ __forceinline__ void add_vir(float ddx, float ddy, float ddz, float dx, float dy, float dz) {
    vxx = fmaf(-ddx, dx, vxx);
    vyy = fmaf(-ddy, dy, vyy);
    vzz = fmaf(-ddz, dz, vzz);
    vxy = fmaf(-ddx, dy, vxy);
    vxz = fmaf(-ddx, dz, vxz);
    vyz = fmaf(-ddy, dz, vyz);
  }
  __device__ __forceinline__ void add_param(const SwitchF32 &s, float r2, float sig, float df) {
    const float r = sqrtf(r2);
    pr0 = fmaf(-df * r, (r - s.d0) * s.invr0, fmaf(s.c_r0, sig - 1.f, pr0));
    pd0 = fmaf(-df, r, fmaf(s.c_d0, sig - 1.f, pd0));
  }
  __device__ __forceinline__ void to_partials(double part[kPartials]) const {
    part[0] = ((double)cv - (double)cvc) + (cv64 + (double)cvs);
    const double xx = vt[0] + vxx, yy = vt[1] + vyy, zz = vt[2] + vzz, xy = vt[3] + vxy, xz = vt[4] + vxz,
                 yz = vt[5] + vyz;
    part[1] = xx;
    part[2] = xy;
    part[3] = xz;
    part[4] = xy;
    part[5] = yy;
    part[6] = yz;
    part[7] = xz;
    part[8] = yz;
    part[9] = zz;
    part[10] = pt[0] + pr0;
    part[11] = pt[1] + pd0;
  }
};

// The reference's inclusive d_max test, r^2 = modulo2(pbc.distance(x1, x2))
// <= d_max^2 in FP64 (CoordinationBase.cpp:187-190, SwitchingFunction.cpp:
// 206), for the rare pair whose FP32 r^2 falls in the band around d_max^2
// (a stretched switch is zero at d_max but its derivative is not, so the
// decision must match).  x1 is the reference's first atom; every operation is
// an explicitly rounded intrinsic, so no contraction changes the result.
// Generic boxes: Pbc::distance's reduced-lattice branch (Pbc.cpp:392-413),
// each matmul summed j = 0, 1, 2 from zero as Vector.h's matmul does.
__device__ __noinline__ void pbc_generic_rn(const PbcParams *pbc, double d[3]) {
  double sc[3];
  for (int i = 0; i < 3; i++) {
    double acc = 0.0;
    for (int j = 0; j < 3; j++) acc = __dadd_rn(acc, __dmul_rn(d[j], pbc->invreduced[j * 3 + i]));
    const double x = __dadd_rn(acc, 100.0);  // Tools::pbc (Tools.h:557-563)
    const double t = (x >= 0) ? (double)__double2int_rz(__dadd_rn(x, 0.5)) : (double)__double2int_rz(__dsub_rn(x, 0.5));
    sc[i] = __dsub_rn(x, t);
  }
  for (int i = 0; i < 3; i++) {
    double acc = 0.0;
    for (int j = 0; j < 3; j++) acc = __dadd_rn(acc, __dmul_rn(sc[j], pbc->reduced[j * 3 + i]));
    d[i] = acc;
  }
  if (__dadd_rn(__dadd_rn(fabs(sc[0]), fabs(sc[1])), fabs(sc[2])) > 0.5) {
    const int o = 4 * (sc[0] > 0 ? 1 : 0) + 2 * (sc[1] > 0 ? 1 : 0) + (sc[2] > 0 ? 1 : 0);
    double best[3] = {d[0], d[1], d[2]};
    double lbest = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
    for (int i = 0; i < pbc->nshift[o]; i++) {
      double t[3];
      for (int k = 0; k < 3; k++) t[k] = __dadd_rn(d[k], pbc->shift[o][i][k]);
      const double l = __dadd_rn(__dadd_rn(__dmul_rn(t[0], t[0]), __dmul_rn(t[1], t[1])), __dmul_rn(t[2], t[2]));
      if (l < lbest) {
        lbest = l;
        best[0] = t[0];
        best[1] = t[1];
        best[2] = t[2];
      }
    }
    for (int k = 0; k < 3; k++) d[k] = best[k];
  }
}
__device__ __forceinline__ bool dmax_exact(const double *x1, const double *x2, const PbcParams *pbc, int do_pbc,
                                        double dmax_2) {
  double d[3];
  for (int k = 0; k < 3; k++) d[k] = __dsub_rn(x2[k], x1[k]);
  if (do_pbc && pbc->type == PBC_GENERIC) pbc_generic_rn(pbc, d);
  if (do_pbc && pbc->type == PBC_ORTHO) {
    for (int k = 0; k < 3; k++) {
      // Tools::pbc (Tools.h:557-563) of d * invBox(k,k), times box(k,k)
      double x = __dadd_rn(__dmul_rn(d[k], pbc->invbox[4 * k]), 100.0);
      const double t = (x >= 0) ? (double)__double2int_rz(__dadd_rn(x, 0.5))
                                : (double)__double2int_rz(__dsub_rn(x, 0.5));
      d[k] = __dmul_rn(__dsub_rn(x, t), pbc->box[4 * k]);
    }
  }
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
  return r2 <= dmax_2;
}

// FP32 displacement x_b - x_a of two fixed-point positions under the frame's
// periodic boundary conditions (the mixed path's pair geometry).
// Orthorhombic (or no) box: the wrapped difference per axis times L / 2^32.
// Generic box: the wrapped differences are the reduced scaled distance after
// Tools::pbc; Pbc::distance takes it back through the reduced cell and, when
// |s0| + |s1| + |s2| > 0.5, tries the shifts of the octant for a shorter
// image (Pbc.cpp:392-413), here in FP32 (the shift test compares the
// fixed-point sum with 2^31).
__device__ __noinline__ void tric_shift32(const FrameConst *fc, float t0, float t1, float t2, float *d) {
  const int o = 4 * (t0 > 0.f ? 1 : 0) + 2 * (t1 > 0.f ? 1 : 0) + (t2 > 0.f ? 1 : 0);
  float b0 = d[0], b1 = d[1], b2 = d[2];
  float lb = fmaf(b0, b0, fmaf(b1, b1, b2 * b2));
  for (int i = 0; i < fc->pbc.nshift[o]; i++) {
    const float x = d[0] + (float)fc->pbc.shift[o][i][0], y = d[1] + (float)fc->pbc.shift[o][i][1],
                z = d[2] + (float)fc->pbc.shift[o][i][2];
    const float l = fmaf(x, x, fmaf(y, y, z * z));
    if (l < lb) {
      lb = l;
      b0 = x;
      b1 = y;
      b2 = z;
    }
  }
  d[0] = b0;
  d[1] = b1;
  d[2] = b2;
}
template <bool TRIC> struct Geo32 {
  float sx, sy, sz;
  __device__ __forceinline__ explicit Geo32(const FrameConst &fc)
      : sx(fc.scale[0]), sy(fc.scale[1]), sz(fc.scale[2]) {}
  __device__ __forceinline__ void delta(const uint4 &a, const uint4 &b, float &dx, float &dy, float &dz) const {
    dx = fixed_delta(a.x, b.x, sx);
    dy = fixed_delta(a.y, b.y, sy);
    dz = fixed_delta(a.z, b.z, sz);
  }
};
template <> struct Geo32<true> {
  const FrameConst *fc;
  float m[9];
  __device__ __forceinline__ explicit Geo32(const FrameConst &f) : fc(&f) {
#pragma unroll
    for (int k = 0; k < 9; k++) m[k] = f.red32[k];
  }
  __device__ __forceinline__ void delta(const uint4 &a, const uint4 &b, float &dx, float &dy, float &dz) const {
    const float t0 = (float)(int)(b.x - a.x), t1 = (float)(int)(b.y - a.y), t2 = (float)(int)(b.z - a.z);
    dx = fmaf(t0, m[0], fmaf(t1, m[3], t2 * m[6]));
    dy = fmaf(t0, m[1], fmaf(t1, m[4], t2 * m[7]));
    dz = fmaf(t0, m[2], fmaf(t1, m[5], t2 * m[8]));
    if (fabsf(t0) + fabsf(t1) + fabsf(t2) > 2147483648.0f) {
      float d[3] = {dx, dy, dz};
      tric_shift32(fc, t0, t1, t2, d);
      dx = d[0];
      dy = d[1];
      dz = d[2];
    }
  }
};

// Asks the TMA engine to bring [p, p + bytes) into L2 (no registers, no
// completion to wait for); p 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void prefetch_l2_bulk(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Fire-and-forget vector reduction into a float4 accumulator (16-byte aligned);
// w carries the per-atom sums of sigma in EVAL_PERATOM.
__device__ __forceinline__ void red_add_v4(float4 *p, float x, float y, float z, float w = 0.f) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(x), "f"(y), "f"(z), "f"(w)
               : "memory");
}


// Bytes per frame of band_flag: slices rounded up to 32 (16-byte vector loads).
__device__ __forceinline__ size_t band_stride(const KArgs &a) { return ((size_t)a.nslices + 31) & ~(size_t)31; }

// Persistent warps: warp w of the frame's grid takes slices w, w + nw, ...;
// the per-thread accumulators carry across slices and one block reduction
// closes the kernel.  Inside a slice the loop runs to the slice width (warp
// uniform); entries and partner positions are loaded kUnroll at a time before
// any is used, so kUnroll gathers are in flight per lane.  Entries are
// streamed once per step (ld.global.cs: evict first) so that the fixed-point
// positions, gathered many times, stay resident in L2.  (A grid that visits
// the frames in order, for L2 locality, measured 2x slower: the per-frame
// block barrier costs more than the locality gains.)
// (four resident blocks of 256 threads per SM: a 64-register budget, which
// the latency of the partner gathers needs more than registers)
// Queues one band pair for k_band_fix and flags its slice (out of line: the
// pair kernel's loop keeps its registers for the partner gathers).
__device__ __noinline__ void band_push(unsigned *qn, uint4 *qbuf, int cap, unsigned *overflow,
                                      unsigned char *slice_flag, uint4 item) {
  const unsigned i = atomicAdd(qn, 1u);
  if (i < (unsigned)cap)
    qbuf[i] = item;
  else
    *overflow = 1u;
  *slice_flag = 1;
}

template <int NH, int MODE, int kUnroll, bool TRIC = false>
__global__ void __launch_bounds__(256, 4) k_eval_nl32(KArgs a, SwitchParams sw, SwitchF32 s32) {
  const int f = blockIdx.y + a.frame0;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  // each warp's FP64 totals of its FP32 sums (s, the six virial components,
  // the two parameter gradients): a lane sums the pairs of its rows over
  // kFlushSlices slices (about 150 pairs) in FP32, the warp sums its lanes
  // in FP32, and lane 0 adds the result here in FP64, so no FP32 sum runs
  // longer.  (Per-lane FP64 totals in shared memory measured 4 % slower:
  // their 21 KB per block came out of L1, which holds the partners.)
  __shared__ double wtot[8][kSliceSums];
  double *const mytot = wtot[threadIdx.x >> 5];
  if (lane < kSliceSums) mytot[lane] = 0.0;
  __syncwarp();
  const int nw = gridDim.x * wpb;
  const size_t fo = (size_t)f * a.ns;
  const Geo32<TRIC> geo(a.fc[f]);
  const uint4 *__restrict__ q = a.q + fo;
  float4 *__restrict__ acc4 = a.acc32 + fo;
  Acc32 acc;
  const size_t slice_words = (size_t)a.cap * 32;
  const uint32_t *ell_f = a.ell + (size_t)f * a.nslices * slice_words;
  // rows read to their near parts while the atoms have moved less than half
  // the skin since the rebuild (near_rows_only), else in full
  const bool near_only = near_rows_only(a, f);
  const int *sw_f = (near_only ? a.slice_wn : a.slice_w) + (size_t)f * a.nslices;
  const int *rl_f = (near_only ? a.row_near : a.row_len) + fo;
  int pending = 0;  // slices summed in FP32 since the last flush
  {
    // this warp's first slice: its entries (w rows of 32 words) into L2
    const int s0 = blockIdx.x * wpb + (threadIdx.x >> 5);
    if (lane == 0 && s0 < a.nslices) {
      const int w0 = sw_f[s0];
      if (w0 > 0) prefetch_l2_bulk(ell_f + (size_t)s0 * slice_words, (uint32_t)w0 * 128u);
    }
  }
  for (int slice = blockIdx.x * wpb + (threadIdx.x >> 5); slice < a.nslices; slice += nw) {
    const int r = slice * 32 + lane;
    const bool active = r < a.ns;
    const int len = active ? rl_f[r] : 0;
    const int w = sw_f[slice];
    if (lane == 0 && slice + nw < a.nslices) {
      // the next slice's entries stream into L2 while this one is evaluated
      const int wn = sw_f[slice + nw];
      if (wn > 0) prefetch_l2_bulk(ell_f + (size_t)(slice + nw) * slice_words, (uint32_t)wn * 128u);
    }
    const uint4 qr = active ? q[r] : make_uint4(0u, 0u, 0u, 0u);
    float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
    const float gr = __uint_as_float(qr.w);  // EVAL_VJP: the row's upstream g
    const uint32_t *__restrict__ e = a.ell + ((size_t)f * a.nslices + slice) * (size_t)a.cap * 32 + lane;
    // one pair inside d_max: s, the two derivatives (d = x_p - x_r:
    // deriv[r] -= df d, deriv[p] += df d, either orientation), the virial;
    // gpw: the partner's q.w
    auto pair = [&](int p, float dx, float dy, float dz, float r2, uint32_t gpw) {
      float sig, df;
      sw32<NH>(sw, s32, r2, sig, df);
      if (MODE >= EVAL_PERATOM && (r2 < (float)kBondEps || sig < (float)kBondEps)) {
        sig = 0.f;
        df = 0.f;
      }
      if (MODE == EVAL_VJP) df *= gr + __uint_as_float(gpw);
      acc.add_s_slice(sig);
      if (MODE >= EVAL_DERIV) {
        const float ddx = df * dx, ddy = df * dy, ddz = df * dz;
        ax -= ddx;
        ay -= ddy;
        az -= ddz;
        if (MODE == EVAL_PERATOM) {
          aw += sig;
          red_add_v4(acc4 + p, ddx, ddy, ddz, sig);
        } else {
          red_add_v4(acc4 + p, ddx, ddy, ddz);
        }
        acc.add_vir(ddx, ddy, ddz, dx, dy, dz);
      }
      if (MODE == EVAL_PARAM) acc.add_param(s32, r2, sig, df);
    };
    // pairs whose FP32 r^2 lies in (dmax2_lo, dmax2_hi] cannot decide the
    // reference's inclusive test r^2 <= d_max^2: they are queued for the
    // FP64 fix-up pass (k_band_fix), and their slice flagged in case the
    // queue is full.  bits(r^2) - bits(lo) - 1 is below the band width
    // exactly for them (r^2 >= 0 orders like its bits; pairs below lo and
    // dead entries, r^2 = 0, wrap to large values).
    const uint32_t band_lo = __float_as_uint(s32.dmax2_lo) + 1u;
    const uint32_t band_w = __float_as_uint(s32.dmax2_hi) - __float_as_uint(s32.dmax2_lo);
    // kUnroll entries of every lane's row from entry k; kChecked: some rows
    // may end before k + kUnroll (entries past a row's end read as ~0)
    auto entries = [&](int k, auto checked) {
      constexpr bool kChecked = decltype(checked)::value;
      uint32_t en[kUnroll];  // list entries (partner rank | orientation)
      uint4 qp[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; u++)
        en[u] = (!kChecked || k + u < len) ? __ldcs(e + (size_t)(k + u) * 32) : 0xffffffffu;
#pragma unroll
      for (int u = 0; u < kUnroll; u++)
        qp[u] = (!kChecked || en[u] != 0xffffffffu) ? __ldg(q + (en[u] & kRankMask)) : qr;
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        float dx, dy, dz;
        geo.delta(qr, qp[u], dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if ((!kChecked || en[u] != 0xffffffffu) && r2 <= s32.dmax2_lo) {
          pair((int)(en[u] & kRankMask), dx, dy, dz, r2, qp[u].w);
        } else if (__float_as_uint(r2) - band_lo < band_w) {
          band_push(a.band_qn + f, a.band_q + (size_t)f * a.band_qcap, a.band_qcap, a.band_qn + a.disp2_frames,
                    a.band_flag + (size_t)f * band_stride(a) + slice, make_uint4((unsigned)f, (unsigned)r, en[u], 0u));
        }
      }
    };
    // up to the slice's shortest row no entry needs the row-end test
    const int kfast = (int)(__reduce_min_sync(0xffffffffu, (unsigned)len) / kUnroll) * kUnroll;
    for (int k = 0; k < kfast; k += kUnroll) entries(k, std::false_type{});
    for (int k = kfast; k < w; k += kUnroll) entries(k, std::true_type{});
    if (MODE >= EVAL_DERIV && len > 0) red_add_v4(acc4 + r, ax, ay, az, aw);
    if (++pending == kFlushSlices) {
      acc.flush_warp<MODE>(mytot, lane);
      pending = 0;
    }
  }
  acc.flush_warp<MODE>(mytot, lane);
  // the block's record: the warps' totals summed in warp order
  __syncthreads();
  if (threadIdx.x < kPartials) {
    // record layout (s, virial row-major, ds/dR_0, ds/dD_0) from the totals
    // (s, xx, yy, zz, xy, xz, yz, ds/dR_0, ds/dD_0): total index of record
    // entry k is nibble k of 0x873656245410
    const int src = (int)((0x873656245410ull >> (4 * threadIdx.x)) & 15ull);
    double v = 0.0;
    for (int w2 = 0; w2 < wpb; w2++) v += wtot[w2][src];
    a.partials[((size_t)f * a.max_blocks + blockIdx.x) * kPartials + threadIdx.x] = v;
  }
  block_records_finish(a, f, gridDim.x);
}

// One band pair of the mixed NL pass (queued or found again in its row):
// the reference's own FP64 test (dmax_exact, in the pair's orientation) and,
// if kept, the pair evaluated at d_max^2 (both sides of the FP32 rounding
// agree there).  The partner's derivative goes out by a vector reduction; the
// row's is added to (ax, ay, az, aw); s / virial / parameter sums into acc.
template <int NH, int MODE, bool TRIC>
__device__ __forceinline__ void band_pair(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32,
                                          const FrameConst &fc, size_t fo, int r, uint4 qr, uint32_t en, uint4 qq,
                                          Acc32 &acc, float &ax, float &ay, float &az, float &aw) {
  float dx, dy, dz;
  Geo32<TRIC>(fc).delta(qr, qq, dx, dy, dz);
  const int p = (int)(en & kRankMask);
  const double *xr = a.pos + (fo + a.slot_of_rank[fo + r]) * 3;
  const double *xp = a.pos + (fo + a.slot_of_rank[fo + p]) * 3;
  const bool in = (en & kOrientBit) ? dmax_exact(xr, xp, &fc.pbc, a.do_pbc, s32.dmax_2)
                                    : dmax_exact(xp, xr, &fc.pbc, a.do_pbc, s32.dmax_2);
  if (!in) return;
  float sig, df;
  sw32<NH>(sw, s32, s32.dmax2, sig, df);
  if (MODE >= EVAL_PERATOM && sig < (float)kBondEps) {
    sig = 0.f;
    df = 0.f;
  }
  if (MODE == EVAL_VJP) df *= __uint_as_float(qr.w) + __uint_as_float(qq.w);
  acc.add_s(sig);
  if (MODE >= EVAL_DERIV) {
    const float ddx = df * dx, ddy = df * dy, ddz = df * dz;
    ax -= ddx;
    ay -= ddy;
    az -= ddz;
    aw += sig;
    red_add_v4(a.acc32 + fo + p, ddx, ddy, ddz, MODE == EVAL_PERATOM ? sig : 0.f);
    acc.add_vir(ddx, ddy, ddz, dx, dy, dz);
  }
  if (MODE == EVAL_PARAM) acc.add_param(s32, s32.dmax2, sig, df);
}

// Adds a frame's fix-up sums (s, virial row-major, ds/dR_0, ds/dD_0) to its
// results: every old value loaded before any store, so the twelve
// read-modify-writes overlap instead of waiting on one another.
__device__ __forceinline__ void add_frame_results(const KArgs &a, int f, const double v[kPartials]) {
  double o[kPartials];
  o[0] = a.out_s ? __ldcg(a.out_s + f) : 0.0;
#pragma unroll
  for (int k = 0; k < 9; k++) o[1 + k] = a.out_virial ? __ldcg(a.out_virial + (size_t)f * 9 + k) : 0.0;
#pragma unroll
  for (int k = 0; k < 2; k++) o[10 + k] = a.out_dparam ? __ldcg(a.out_dparam + (size_t)f * 2 + k) : 0.0;
  if (a.out_s) a.out_s[f] = o[0] + v[0];
  if (a.out_virial)
#pragma unroll
    for (int k = 0; k < 9; k++) a.out_virial[(size_t)f * 9 + k] = o[1 + k] + v[1 + k];
  if (a.out_dparam)
#pragma unroll
    for (int k = 0; k < 2; k++) a.out_dparam[(size_t)f * 2 + k] = o[10 + k] + v[10 + k];
}

// Queue order: frame, row, partner (a total order: a row lists a partner once).
__device__ __forceinline__ bool band_less(const uint4 &x, const uint4 &y) {
  if (x.x != y.x) return x.x < y.x;
  if (x.y != y.y) return x.y < y.y;
  return (x.z & kRankMask) < (y.z & kRankMask);
}

// FP64 fix-up of the mixed NL pass.  The pair kernel queued, per frame, the
// pairs whose FP32 r^2 lies in the band around d_max^2 (about a hundred per
// frame among 1e7 at 262,144 atoms).  With every frame's pairs in its queue,
// a frame's blocks evaluate them one per thread (band_pair) into a record
// per pair and clear the slices' flags; the frame's last block sorts the
// frame's queue (bitonic, in shared memory) and adds the records to the
// frame's results in that order, so the sums do not depend on the order the
// pairs were queued in.  When some frame's queue overflowed, every block
// takes the flagged slices instead: their rows are scanned again, each band
// pair evaluated, a record per slice, and the frame's last block adds the
// records in slice order.  Each frame's last block resets its queue.
template <int NH, int MODE, bool TRIC = false>
__global__ void __launch_bounds__(256) k_band_fix(KArgs a, SwitchParams sw, SwitchF32 s32) {
  // the queue's sort (kBandQueueCap entries) or the slice path's reduction
  __shared__ __align__(16) unsigned char smem[kPartials * 256 * sizeof(double)];
  static_assert(kBandQueueCap * sizeof(uint4) <= sizeof(smem), "fix-up shared memory");
  if (__ldcg(a.band_qn + a.disp2_frames) == 0u) {  // every frame's band pairs are in its queue
    const int f = blockIdx.y + a.frame0;
    const unsigned nq = __ldcg(a.band_qn + f);
    const uint4 *qf = a.band_q + (size_t)f * a.band_qcap;
    double *rf = a.band_qrec + (size_t)f * a.band_qcap * kPartials;
    // the frame's blocks: its queued pairs one per thread, a record each,
    // dealt round-robin over the blocks (their FP64 work spread over the SMs)
    for (unsigned i = blockIdx.x + gridDim.x * threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
      const uint4 t = __ldcg(qf + i);
      const int r = (int)t.y;
      const size_t fo = (size_t)f * a.ns;
      const FrameConst &fc = a.fc[f];
      const uint4 qr = a.q[fo + r];
      Acc32 acc;
      float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
      band_pair<NH, MODE, TRIC>(a, sw, s32, fc, fo, r, qr, t.z, a.q[fo + (t.z & kRankMask)], acc, ax, ay, az, aw);
      if (MODE >= EVAL_DERIV && (ax != 0.f || ay != 0.f || az != 0.f || aw != 0.f))
        red_add_v4(a.acc32 + fo + r, ax, ay, az, MODE == EVAL_PERATOM ? aw : 0.f);
      double part[kPartials];
      acc.to_partials(part);
#pragma unroll
      for (int k = 0; k < kPartials; k++) rf[(size_t)i * kPartials + k] = part[k];
      a.band_flag[(size_t)f * band_stride(a) + r / 32] = 0;
    }
    // the frame's last block: its queue sorted (row, partner) with each
    // pair's record index, the records added in that order
    __shared__ bool last_q;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last_q = atomicAdd(&a.band_tickets[f], 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!last_q) return;
    __threadfence();
    uint4 *sq = reinterpret_cast<uint4 *>(smem);
    unsigned m = 1;
    while (m < nq) m <<= 1;
    for (unsigned i = threadIdx.x; i < m; i += blockDim.x) {
      uint4 t = i < nq ? __ldcg(qf + i) : make_uint4(~0u, ~0u, ~0u, ~0u);
      t.w = i;
      sq[i] = t;
    }
    __syncthreads();
    for (unsigned k = 2; k <= m; k <<= 1)
      for (unsigned j = k >> 1; j > 0; j >>= 1) {
        for (unsigned i = threadIdx.x; i < m; i += blockDim.x) {
          const unsigned l = i ^ j;
          if (l > i) {
            const uint4 x = sq[i], y = sq[l];
            if (band_less(y, x) == ((i & k) == 0)) {
              sq[i] = y;
              sq[l] = x;
            }
          }
        }
        __syncthreads();
      }
    // warp w sums the sorted records w, w + 8, ... lane by lane (lane l:
    // records w + 8 (l + 32 i)), then a fixed shuffle tree, then the warps'
    // sums in warp order: an order set by the sorted queue alone
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double v[kPartials];
#pragma unroll
    for (int k = 0; k < kPartials; k++) v[k] = 0.0;
    for (unsigned j = warp + nw * lane; j < nq; j += nw * 32)
#pragma unroll
      for (int k = 0; k < kPartials; k++) v[k] += __ldcg(rf + (size_t)sq[j].w * kPartials + k);
#pragma unroll
    for (int k = 0; k < kPartials; k++) v[k] = warp_sum(v[k]);
    __syncthreads();  // the records' reads are done with sq; its memory takes the warps' sums
    double(*ws)[kPartials] = reinterpret_cast<double(*)[kPartials]>(smem);
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < kPartials; k++) ws[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
      double t[kPartials];
#pragma unroll
      for (int k = 0; k < kPartials; k++) t[k] = 0.0;
      for (int w = 0; w < nw; w++)
#pragma unroll
        for (int k = 0; k < kPartials; k++) t[k] += ws[w][k];
      if (nq > 0) add_frame_results(a, f, t);
      a.band_qn[f] = 0u;
      a.band_tickets[f] = 0u;
    }
    return;
  }
  const int f = blockIdx.y + a.frame0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const size_t fo = (size_t)f * a.ns;
  const FrameConst &fc = a.fc[f];
  const Geo32<TRIC> geo(fc);
  const uint4 *__restrict__ q = a.q + fo;
  unsigned char *flag = a.band_flag + (size_t)f * band_stride(a);
  const uint32_t band_lo = __float_as_uint(s32.dmax2_lo) + 1u;
  const uint32_t band_w = __float_as_uint(s32.dmax2_hi) - __float_as_uint(s32.dmax2_lo);
  // each warp takes 32 consecutive slices: one coalesced load of their flags
  for (int chunk = blockIdx.x * nwarps + warp; chunk * 32 < a.nslices; chunk += gridDim.x * nwarps) {
    const int s_l = chunk * 32 + lane;
    unsigned todo = __ballot_sync(0xffffffffu, s_l < a.nslices && flag[s_l] != 0);
    while (todo) {
    const int slice = chunk * 32 + __ffs(todo) - 1;
    todo &= todo - 1u;
    const int r = slice * 32 + lane;
    const bool active = r < a.ns;
    const int len = active ? a.row_len[fo + r] : 0;
    const uint4 qr = active ? q[r] : make_uint4(0u, 0u, 0u, 0u);
    const uint32_t *e = a.ell + ((size_t)f * a.nslices + slice) * (size_t)a.cap * 32 + lane;
    Acc32 acc;
    float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
    constexpr int kU = 8;  // entries and partner positions in flight per lane
    for (int k0 = 0; k0 < len; k0 += kU) {
      uint32_t en[kU];
      uint4 qq[kU];
#pragma unroll
      for (int u = 0; u < kU; u++) en[u] = (k0 + u < len) ? e[(size_t)(k0 + u) * 32] : 0xffffffffu;
#pragma unroll
      for (int u = 0; u < kU; u++) qq[u] = (en[u] != 0xffffffffu) ? q[en[u] & kRankMask] : qr;
#pragma unroll
      for (int u = 0; u < kU; u++) {
        float dx, dy, dz;
        geo.delta(qr, qq[u], dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        if ((__float_as_uint(r2) - band_lo) >= band_w) continue;  // dead entries: r2 = 0, never in the band
        band_pair<NH, MODE, TRIC>(a, sw, s32, fc, fo, r, qr, en[u], qq[u], acc, ax, ay, az, aw);
      }
    }
    if (MODE >= EVAL_DERIV && (ax != 0.f || ay != 0.f || az != 0.f || aw != 0.f))
      red_add_v4(a.acc32 + fo + r, ax, ay, az, MODE == EVAL_PERATOM ? aw : 0.f);
    double part[kPartials];
    acc.to_partials(part);
    double *rec = a.band_rec + ((size_t)f * a.nslices + slice) * kPartials;
#pragma unroll
    for (int k = 0; k < kPartials; k++) {
      const double v = warp_sum(part[k]);  // fixed shuffle tree
      if (lane == 0) rec[k] = v;
    }
    }
  }
  // the frame's last block: records of the flagged slices, in slice order
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = atomicAdd(&a.band_tickets[f], 1u) == gridDim.x - 1u;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // thread t: slices [32 t', 32 t' + 32) for t' = t, t + 256, ... in order,
  // their flags as two 16-byte loads
  double v[kPartials];
#pragma unroll
  for (int k = 0; k < kPartials; k++) v[k] = 0.0;
  bool any = false;
  for (int c0 = threadIdx.x * 32; c0 < a.nslices; c0 += blockDim.x * 32) {
    uint4 *fv = reinterpret_cast<uint4 *>(flag + c0);
    const uint4 f0 = __ldcg(fv), f1 = __ldcg(fv + 1);
    if ((f0.x | f0.y | f0.z | f0.w | f1.x | f1.y | f1.z | f1.w) == 0u) continue;
    any = true;
    for (int sl = c0; sl < min(c0 + 32, a.nslices); sl++) {
      if (!flag[sl]) continue;
      const double *rec = a.band_rec + ((size_t)f * a.nslices + sl) * kPartials;
#pragma unroll
      for (int k = 0; k < kPartials; k++) v[k] += __ldcg(rec + k);
    }
    fv[0] = make_uint4(0u, 0u, 0u, 0u);
    fv[1] = make_uint4(0u, 0u, 0u, 0u);
  }
  double(*red)[256] = reinterpret_cast<double(*)[256]>(smem);
  __shared__ int any_block;
  if (threadIdx.x == 0) any_block = 0;
  __syncthreads();
  if (any) atomicOr(&any_block, 1);
#pragma unroll
  for (int k = 0; k < kPartials; k++) red[k][threadIdx.x] = v[k];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int k = 0; k < kPartials; k++) red[k][threadIdx.x] += red[k][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.band_tickets[f] = 0u;
    if (any_block) {
      double v[kPartials];
#pragma unroll
      for (int k = 0; k < kPartials; k++) v[k] = red[k][0];
      add_frame_results(a, f, v);
    }
    // the frame's queue count; the launch's last frame resets the overflow flag
    a.band_qn[f] = 0u;
    __threadfence();
    if (atomicAdd(&a.band_qn[a.disp2_frames + 1], 1u) == gridDim.y - 1u) {
      a.band_qn[a.disp2_frames + 1] = 0u;
      a.band_qn[a.disp2_frames] = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// every pair (no NLIST): tiles of TILE i-slots against TILE j-slots, a
// persistent grid striding over tile pairs.  j-side derivatives accumulate in
// shared memory with a staggered order (thread t visits j = (t+step) mod
// TILE) so no two threads hit one address in the same step.  Single list:
// tiles (I,J), J>=I, j>i inside a diagonal tile; two lists: A x B tiles.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tile_pair(int t, int nTi, int nTj, bool tri, int &I, int &J) {
  if (!tri) {
    I = t / nTj;
    J = t % nTj;
    return;
  }
  int i = 0, rem = t;
  while (rem >= nTi - i) {
    rem -= nTi - i;
    i++;
  }
  I = i;
  J = i + rem;
}

template <int TILE, int MODE>
__global__ void __launch_bounds__(TILE) k_allpairs64(KArgs a, SwitchParams sw, int nTi, int nTj, int ntp) {
  const int f = blockIdx.z;
  const bool tri = a.mode == MODE_SINGLE;
  const int iend = tri ? a.ns : a.nA, jbase0 = tri ? 0 : a.nA, jend = a.ns;
  const size_t fo = (size_t)f * a.ns;
  const FrameConst &fc = a.fc[f];
  __shared__ double xj[TILE][3];
  __shared__ double accj[TILE][3];
  __shared__ long long absj[TILE];
  double part[kPartials];
#pragma unroll
  for (int k = 0; k < kPartials; k++) part[k] = 0.0;
  for (int t = blockIdx.x; t < ntp; t += gridDim.x) {
    int I, J;
    tile_pair(t, nTi, nTj, tri, I, J);
    const int i = I * TILE + threadIdx.x;
    const int jb = jbase0 + J * TILE;
    __syncthreads();
    {
      const int j = jb + threadIdx.x;
      if (j < jend) {
        const double *p = a.pos + (fo + j) * 3;
        xj[threadIdx.x][0] = p[0];
        xj[threadIdx.x][1] = p[1];
        xj[threadIdx.x][2] = p[2];
        absj[threadIdx.x] = a.abs_of_slot[j];
      }
      accj[threadIdx.x][0] = accj[threadIdx.x][1] = accj[threadIdx.x][2] = 0.0;
    }
    __syncthreads();
    double acci[3] = {0.0, 0.0, 0.0};
    if (i < iend) {
      const double *pi = a.pos + (fo + i) * 3;
      const double xi[3] = {pi[0], pi[1], pi[2]};
      const long long absi = a.abs_of_slot[i];
      const bool diag = tri && (I == J);
      for (int s = 0; s < TILE; s++) {
        const int jl = (threadIdx.x + s) & (TILE - 1);
        const int j = jb + jl;
        if (j >= jend || (diag && jl <= (int)threadIdx.x) || absj[jl] == absi) continue;
        double d[3], df;
        const double xjj[3] = {xj[jl][0], xj[jl][1], xj[jl][2]};
        const double sig = pair_fp64(a, sw, fc, xi, xjj, i, j, d, df);
        part[0] += sig;
        if (MODE >= EVAL_DERIV) {
          const double dd[3] = {df * d[0], df * d[1], df * d[2]};
          for (int q = 0; q < 3; q++) {
            acci[q] -= dd[q];
            if (dd[q] != 0.0) atomicAdd(&accj[jl][q], dd[q]);
          }
          vir_sub(part, dd, d);
        }
        if (MODE == EVAL_PARAM) param_acc64(sw, mod2(d), sig, df, part);
      }
      if (MODE >= EVAL_DERIV)
        for (int q = 0; q < 3; q++)
          if (acci[q] != 0.0) atomicAdd(a.acc64 + (fo + i) * 3 + q, acci[q]);
    }
    __syncthreads();
    if (MODE >= EVAL_DERIV) {
      const int j = jb + threadIdx.x;
      if (j < jend)
        for (int q = 0; q < 3; q++)
          if (accj[threadIdx.x][q] != 0.0) atomicAdd(a.acc64 + (fo + j) * 3 + q, accj[threadIdx.x][q]);
    }
  }
  block_partials_finish(a, f, part, gridDim.x);
}

template <int TILE, int NH, int MODE, bool TRIC = false>
__global__ void __launch_bounds__(TILE) k_allpairs32(KArgs a, SwitchParams sw, SwitchF32 s32, int nTi, int nTj,
                                                     int ntp) {
  const int f = blockIdx.z;
  const bool tri = a.mode == MODE_SINGLE;
  const int iend = tri ? a.ns : a.nA, jbase0 = tri ? 0 : a.nA, jend = a.ns;
  const size_t fo = (size_t)f * a.ns;
  const FrameConst &fc = a.fc[f];
  const Geo32<TRIC> geo(fc);
  __shared__ uint4 qj[TILE];
  __shared__ float accj[TILE][3];
  __shared__ long long absj[TILE];
  Acc32 acc;
  for (int t = blockIdx.x; t < ntp; t += gridDim.x) {
    int I, J;
    tile_pair(t, nTi, nTj, tri, I, J);
    const int i = I * TILE + threadIdx.x;
    const int jb = jbase0 + J * TILE;
    __syncthreads();
    {
      const int j = jb + threadIdx.x;
      if (j < jend) {
        qj[threadIdx.x] = a.q[fo + j];
        absj[threadIdx.x] = a.abs_of_slot[j];
      }
      accj[threadIdx.x][0] = accj[threadIdx.x][1] = accj[threadIdx.x][2] = 0.f;
    }
    __syncthreads();
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (i < iend) {
      const uint4 qi = a.q[fo + i];
      const long long absi = a.abs_of_slot[i];
      const bool diag = tri && (I == J);
      for (int s = 0; s < TILE; s++) {
        const int jl = (threadIdx.x + s) & (TILE - 1);
        const int j = jb + jl;
        if (j >= jend || (diag && jl <= (int)threadIdx.x) || absj[jl] == absi) continue;
        const uint4 qp = qj[jl];
        float dx, dy, dz;
        geo.delta(qi, qp, dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        bool in = r2 <= s32.dmax2_lo;
        if (!in && r2 <= s32.dmax2_hi)  // band: slot i is the reference's first atom
          in = dmax_exact(a.pos + (fo + i) * 3, a.pos + (fo + j) * 3, &fc.pbc, a.do_pbc, s32.dmax_2);
        if (in) {
          float sig, df;
          sw32<NH>(sw, s32, fminf(r2, s32.dmax2), sig, df);
          acc.add_s(sig);
          if (MODE >= EVAL_DERIV) {
            const float ddx = df * dx, ddy = df * dy, ddz = df * dz;
            ax -= ddx;
            ay -= ddy;
            az -= ddz;
            atomicAdd(&accj[jl][0], ddx);
            atomicAdd(&accj[jl][1], ddy);
            atomicAdd(&accj[jl][2], ddz);
            acc.add_vir(ddx, ddy, ddz, dx, dy, dz);
          }
          if (MODE == EVAL_PARAM) acc.add_param(s32, fminf(r2, s32.dmax2), sig, df);
        }
      }
      if (MODE >= EVAL_DERIV && (ax != 0.f || ay != 0.f || az != 0.f))
        atomicAdd(a.acc32 + fo + i, make_float4(ax, ay, az, 0.f));
      acc.flush_tile<MODE>();
    }
    __syncthreads();
    if (MODE >= EVAL_DERIV) {
      const int j = jb + threadIdx.x;
      const float *v = accj[threadIdx.x];
      if (j < jend && (v[0] != 0.f || v[1] != 0.f || v[2] != 0.f))
        atomicAdd(a.acc32 + fo + j, make_float4(v[0], v[1], v[2], 0.f));
    }
  }
  double part[kPartials];
  acc.to_partials(part);
  block_partials_finish(a, f, part, gridDim.x);
}

// ---------------------------------------------------------------------------
// PAIR: pair i is (slot i, slot i+nA); every slot belongs to one pair, so
// derivatives are written without atomics.  With NLIST only flagged pairs.
// ---------------------------------------------------------------------------
template <int MODE> __global__ void k_pairs64(KArgs a, SwitchParams sw, int use_flags) {
  const int f = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t fo = (size_t)f * a.ns;
  double part[kPartials];
#pragma unroll
  for (int k = 0; k < kPartials; k++) part[k] = 0.0;
  if (i < a.nA && (!use_flags || a.pair_flag[(size_t)f * a.nA + i]) && a.abs_of_slot[i] != a.abs_of_slot[i + a.nA]) {
    const double *p0 = a.pos + (fo + i) * 3, *p1 = a.pos + (fo + i + a.nA) * 3;
    const double v1[3] = {p0[0], p0[1], p0[2]}, v2[3] = {p1[0], p1[1], p1[2]};
    double d[3], df;
    part[0] = pair_fp64(a, sw, a.fc[f], v1, v2, i, i + a.nA, d, df);
    if (MODE >= EVAL_DERIV) {
      const double dd[3] = {df * d[0], df * d[1], df * d[2]};
      for (int q = 0; q < 3; q++) {
        a.acc64[(fo + i) * 3 + q] -= dd[q];
        a.acc64[(fo + i + a.nA) * 3 + q] += dd[q];
      }
      vir_sub(part, dd, d);
    }
    if (MODE == EVAL_PARAM) param_acc64(sw, mod2(d), part[0], df, part);
  }
  block_partials_finish(a, f, part, gridDim.x);
}

template <int NH, int MODE, bool TRIC = false>
__global__ void k_pairs32(KArgs a, SwitchParams sw, SwitchF32 s32, int use_flags) {
  const int f = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const size_t fo = (size_t)f * a.ns;
  Acc32 acc;
  if (i < a.nA && (!use_flags || a.pair_flag[(size_t)f * a.nA + i]) && a.abs_of_slot[i] != a.abs_of_slot[i + a.nA]) {
    const FrameConst &fc = a.fc[f];
    const uint4 q0 = a.q[fo + i], q1 = a.q[fo + i + a.nA];
    float dx, dy, dz;
    Geo32<TRIC>(fc).delta(q0, q1, dx, dy, dz);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    bool in = r2 <= s32.dmax2_lo;
    if (!in && r2 <= s32.dmax2_hi)  // band: pair i is (slot i, slot i+nA) in the reference's orientation
      in = dmax_exact(a.pos + (fo + i) * 3, a.pos + (fo + i + a.nA) * 3, &fc.pbc, a.do_pbc, s32.dmax_2);
    if (in) {
      float sig, df;
      sw32<NH>(sw, s32, fminf(r2, s32.dmax2), sig, df);
      acc.add_s(sig);
      if (MODE >= EVAL_DERIV) {
        const float ddx = df * dx, ddy = df * dy, ddz = df * dz;
        float4 &a0 = a.acc32[fo + i], &a1 = a.acc32[fo + i + a.nA];
        a0.x -= ddx;
        a0.y -= ddy;
        a0.z -= ddz;
        a1.x += ddx;
        a1.y += ddy;
        a1.z += ddz;
        acc.add_vir(ddx, ddy, ddz, dx, dy, dz);
      }
      if (MODE == EVAL_PARAM) acc.add_param(s32, fminf(r2, s32.dmax2), sig, df);
    }
  }
  double part[kPartials];
  acc.to_partials(part);
  block_partials_finish(a, f, part, gridDim.x);
}

// ---------------------------------------------------------------------------
// backward epilogue: box and parameter gradients of V from this pass's virial
// B and parameter sums: dV/dh = g * (-(h^T)^{-1} B)  (scaled coordinates held
// fixed; the box-derivative convention of ActionAtomistic.cpp:221-265).
// ---------------------------------------------------------------------------
__global__ void k_grad_post(KArgs a, const double *vir, const double *dpar, double *grad_box, double *grad_param) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.nframes) return;
  const double g = a.g ? a.g[f] : 1.0;
  const FrameConst &fc = a.fc[f];
  if (grad_box) {
    const double *B = vir + (size_t)f * 9;
    const double *ib = fc.pbc.invbox;
    const bool has_box = fc.pbc.type != PBC_UNSET;
    for (int k = 0; k < 3; k++)
      for (int b = 0; b < 3; b++) {
        double s = 0.0;
        for (int q = 0; q < 3; q++) s += ib[q * 3 + k] * B[q * 3 + b];
        grad_box[(size_t)f * 9 + k * 3 + b] = has_box ? -g * s : 0.0;
      }
  }
  if (grad_param) {
    grad_param[(size_t)f * 2] = g * dpar[(size_t)f * 2];
    grad_param[(size_t)f * 2 + 1] = g * dpar[(size_t)f * 2 + 1];
  }
}

} // namespace
} // namespace coordgpu
