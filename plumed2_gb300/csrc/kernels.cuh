// kernels.cuh -- sm_103a kernels of the COORDINATION hot path.
//
// Included by two translation units:
//   k_fp64.cu   compiled with -fmad=false: neighbour-list build (the exact
//               FP64 cutoff test must not be contracted) and the FP64 pair
//               kernels, whose per-pair arithmetic repeats the reference's
//               operations in order (Pbc::distance + modulo2 +
//               SwitchingFunction::calculateSqr, CoordinationBase.cpp:187-206)
//   k_mixed.cu  FP32 pair kernels (FMA allowed) with compensated FP64 sums
//
// Data layout (per frame f; frames = walkers or trajectory frames):
//   slots     GROUPA then GROUPB, the order positions arrive in
//   ranks     slots sorted by neighbour-list cell (x fastest) and, inside a
//             cell, by slot index: spatially coherent rows for the pair kernels
//   ell       neighbour list as a sliced ELL: 32 consecutive ranks form a
//             slice (one warp); entry k of lane l sits at
//             ell[(slice*cap + k)*32 + l]; bits 0-30 partner rank, bit 31 set
//             when the row atom is the first atom of the pair in the
//             reference's orientation (NeighborList.cpp:158-163,252-266).
//             Each pair is stored once (half list), owned by the lower rank
//             when ranks sum to even, else by the higher (balanced rows).
//   q         mixed path positions as 32-bit fixed-point fractions of the box
//             (orthorhombic) or of a bounding frame (no pbc): differences
//             wrap modulo 2^32, which is exactly the minimum image.
#pragma once
#include "coordgpu.h"
#include "coord_internal.h"
#include "switch_eval.cuh"
#include "kargs.h"
#include <cstdint>

namespace coordgpu {

namespace {  // kernels have internal linkage: each .cu instantiates what it launches

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// The frame's last block (atomic ticket, no waiting) sums every block's record
// of kPartials doubles in block order with Neumaier compensation; the final
// values land in out_s / out_virial / out_dparam of the frame.  Called by
// every thread after the block's record has been written.
__device__ void block_records_finish(const KArgs &a, int frame, int nblocks_frame) {
  __shared__ bool is_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(&a.tickets[frame], 1u);
    is_last = (t == (unsigned)nblocks_frame - 1u);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // Quantity k is summed by warp k % nwarps: each lane a Neumaier-compensated
  // sum over records lane, lane+32, ...; the lanes' (sum, compensation) pairs
  // then meet in a fixed shuffle tree with exact two-sums, so the result does
  // not depend on timing and the loads of a quantity are spread over 32 lanes.
  const double *base = a.partials + (size_t)frame * a.max_blocks * kPartials;
  for (int k = warp; k < kPartials; k += nwarps) {
    double s = 0.0, c = 0.0;
    for (int b = lane; b < nblocks_frame; b += 32) {
      const double x = __ldcg(base + (size_t)b * kPartials + k);
      const double t = s + x;
      c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
      s = t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double s2 = __shfl_xor_sync(0xffffffffu, s, o), c2 = __shfl_xor_sync(0xffffffffu, c, o);
      // the lower lane of each exchange orders the operands, so both lanes agree bit for bit
      const double x = (lane & o) ? s2 : s, y = (lane & o) ? s : s2;
      const double t = x + y, bv = t - x;
      c = ((lane & o) ? c2 + c : c + c2) + ((x - (t - bv)) + (y - bv));
      s = t;
    }
    if (lane == 0) {
      const double v = s + c;
      if (k == 0) {
        if (a.out_s) a.out_s[frame] = v;
      } else if (k <= 9) {
        if (a.out_virial) a.out_virial[(size_t)frame * 9 + (k - 1)] = v;
      } else {
        if (a.out_dparam) a.out_dparam[(size_t)frame * 2 + (k - 10)] = v;
      }
    }
  }
  if (threadIdx.x == 0) a.tickets[frame] = 0u;
}

// Sums 16 doubles per lane over the warp as a reduce-scatter: at each level a
// lane keeps half of its quantities and adds its partner's copy of them, so
// 16 FP64 additions per lane (8 + 4 + 2 + 1 + 1) instead of 5 per quantity.
// Afterwards lanes 2q and 2q+1 hold the warp's sum of quantity q in x[0].
// (The FP64 pipe is narrow on this part: the additions, not the shuffles,
// are the cost.)
__device__ __forceinline__ void warp_reduce_scatter16(double x[16], int lane) {
#pragma unroll
  for (int lvl = 0, half = 8, o = 16; lvl < 4; lvl++, half >>= 1, o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      if (i >= half) break;
      const double mine = up ? x[half + i] : x[i], other = up ? x[i] : x[half + i];
      x[i] = mine + __shfl_xor_sync(0xffffffffu, other, o);
    }
  }
  x[0] += __shfl_xor_sync(0xffffffffu, x[0], 1);
}

// Block-reduces kPartials doubles (one set per thread) into the block's
// record, then block_records_finish.
__device__ void block_partials_finish(const KArgs &a, int frame, double v[kPartials], int nblocks_frame) {
  __shared__ double red[kPartials][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
  double x[16];
#pragma unroll
  for (int k = 0; k < 16; k++) x[k] = k < kPartials ? v[k] : 0.0;
  warp_reduce_scatter16(x, lane);
  if ((lane & 1) == 0 && (lane >> 1) < kPartials) red[lane >> 1][warp] = x[0];
  __syncthreads();
  double *rec = a.partials + ((size_t)frame * a.max_blocks + blockIdx.x) * kPartials;
  if (threadIdx.x < kPartials) {
    double s = 0.0;
    for (int w = 0; w < nwarps; w++) s += red[threadIdx.x][w];
    rec[threadIdx.x] = s;
  }
  block_records_finish(a, frame, nblocks_frame);
}

// ---------------------------------------------------------------------------
// fixed-point positions (mixed path and the FP32 neighbour-list prefilter)
// ---------------------------------------------------------------------------
// q = rn((x - lo) / L * 2^32) mod 2^32 per coordinate: the fraction of the
// frame, wrapped as frac() would.  Orthorhombic frames (and no PBC) take it
// in integer arithmetic (fixed_v64), generic boxes through the reduced cell
// in FP64, and fixed_of_hi (the FP64 pass's image shifts need the high word
// of the same rounding) as one FP64 FMA and one conversion per coordinate.
__device__ __forceinline__ uint4 fixed_of(const FrameConst &fc, const double *x) {
  if (fc.tric) {  // reduced fractional coordinates: three FMAs per component
    uint32_t v[3];
#pragma unroll
    for (int i = 0; i < 3; i++)
      v[i] = (uint32_t)(unsigned long long)__double2ll_rn(
          fma(x[0], fc.fx_m[i], fma(x[1], fc.fx_m[3 + i], x[2] * fc.fx_m[6 + i])));
    return make_uint4(v[0], v[1], v[2], 0u);
  }
  // rn((x - lo) inv_l 2^32) mod 2^32 in integer arithmetic (fixed_v64)
  uint32_t v[3];
#pragma unroll
  for (int k = 0; k < 3; k++)
    v[k] = (uint32_t)((fixed_v64(x[k], fc.fxi_m[k], fc.fxi_e[k]) + fc.fxi_c[k] + 0x80000000ull) >> 32);
  return make_uint4(v[0], v[1], v[2], 0u);
}
// The same fixed-point positions with their high words: the 64-bit value
// rn(x * 2^32 / L) is (box image) * 2^32 + q.
__device__ __forceinline__ uint4 fixed_of_hi(const FrameConst &fc, const double *x, int4 &hi) {
  long long v[3];
#pragma unroll
  for (int k = 0; k < 3; k++) v[k] = __double2ll_rn(fma(x[k], fc.fx_s[k], fc.fx_c[k]));
  hi = make_int4((int)(v[0] >> 32), (int)(v[1] >> 32), (int)(v[2] >> 32), 0);
  return make_uint4((uint32_t)v[0], (uint32_t)v[1], (uint32_t)v[2], 0u);
}
// float -> double by re-biasing the exponent (exact, as the conversion
// instruction is, without the FP64 pipe that bounds the O(N) kernels that
// widen accumulators); subnormals, infinities and NaNs take the instruction.
__device__ __forceinline__ double f2d_int(float v) {
  const uint32_t b = __float_as_uint(v);
  if ((b << 1) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);  // +-0
  const uint32_t e = (b >> 23) & 0xffu;
  if (e - 1u >= 254u) return (double)v;
  return __hiloint2double((int)((b & 0x80000000u) | (((b >> 3) & 0x0fffffffu) + 0x38000000u)), (int)(b << 29));
}
__device__ __forceinline__ float fixed_delta(uint32_t a, uint32_t b, float scale) {
  return (float)(int)(b - a) * scale;  // wraps modulo 2^32: minimum image
}
// The largest d2 of the block's threads (valid ones) into *step and
// *interval: warp maxima, a shared maximum, then one atomic pair per block
// (unsigned bits of a non-negative float order like the floats).  Every
// thread of the block calls it.  (Atomics per warp on the frame's one
// address measured 50 % slower for the gather.)
__device__ __forceinline__ void disp_max_block(unsigned *step, unsigned *interval, float d2, bool valid) {
  __shared__ unsigned bmax;
  if (threadIdx.x == 0) bmax = 0u;
  __syncthreads();
  const unsigned v = __reduce_max_sync(0xffffffffu, valid ? __float_as_uint(d2) : 0u);
  if ((threadIdx.x & 31) == 0 && v) atomicMax(&bmax, v);
  __syncthreads();
  if (threadIdx.x == 0 && bmax) {
    atomicMax(step, bmax);
    atomicMax(interval, bmax);
  }
}
// Squared displacement since the rebuild of a rank whose new fixed-point
// position is qq (wrapped: the minimum image in a periodic box).
__device__ __forceinline__ float disp2_of(const FrameConst &fc, uint4 qb, uint4 qq) {
  const float dx = fixed_delta(qb.x, qq.x, fc.scale[0]), dy = fixed_delta(qb.y, qq.y, fc.scale[1]),
              dz = fixed_delta(qb.z, qq.z, fc.scale[2]);
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// ---------------------------------------------------------------------------
// cells: binning, scan, scatter, per-cell ordering
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cell_index_of(const FrameConst &fc, const double *x, int nl_kind, int do_pbc) {
  const GridParams &g = fc.grid;
  int c[3];
  if (nl_kind == 2) {
    // LinkCells::findMyCell (LinkCells.cpp:255-266): scaled coordinates of
    // (x - origin) through invBox^T, then floor((pbc(s)+0.5)*n).
    double xm[3] = {x[0] - g.lo[0], x[1] - g.lo[1], x[2] - g.lo[2]};
    const double *ib = fc.pbc.invbox;
    for (int i = 0; i < 3; i++) {
      double s = 0.0;
      for (int j = 0; j < 3; j++) s += ib[j * 3 + i] * xm[j];
      int ci = (int)floor((tools_pbc(s) + 0.5) * g.nc[i]);
      c[i] = min(max(ci, 0), g.nc[i] - 1);
    }
  } else if (g.wrap) {
    for (int k = 0; k < 3; k++) {
      if (fc.fxi_m[k]) {
        // floor(frac(x / L) * n) in integer arithmetic: the top 32 bits of
        // (x / L) 2^64 mod 2^64 (fixed_v64) times n, high word (the O(N)
        // binning is otherwise bound by the FP64 pipe)
        const unsigned long long v = fixed_v64(x[k], fc.fxi_m[k], fc.fxi_e[k]);
        c[k] = min((int)(((v >> 32) * (unsigned long long)g.nc[k]) >> 32), g.nc[k] - 1);
      } else {
        double f = x[k] * fc.pbc.invbox[4 * k];
        f = f - floor(f);
        c[k] = min(max((int)(f * g.nc[k]), 0), g.nc[k] - 1);
      }
    }
  } else {
    for (int k = 0; k < 3; k++) {
      const double f = (x[k] - g.lo[k]) * g.inv_width[k];
      c[k] = min(max((int)floor(f * g.nc[k]), 0), g.nc[k] - 1);
    }
  }
  (void)do_pbc;
  return (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
}

// min/max of positions per frame (no-pbc bounding frames)
__device__ __forceinline__ unsigned long long ordered_bits(double v) {
  unsigned long long b = __double_as_longlong(v);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_ordered(unsigned long long b) {
  b = (b & 0x8000000000000000ull) ? (b & 0x7fffffffffffffffull) : ~b;
  return __longlong_as_double(b);
}

__global__ void k_bounds(KArgs a, unsigned long long *mm /*[nframes][6]*/) {
  const int f = blockIdx.y;
  const double *pos = a.pos + (size_t)f * a.ns * 3;
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < a.ns; s += gridDim.x * blockDim.x)
    for (int k = 0; k < 3; k++) {
      unsigned long long b = ordered_bits(pos[3 * (size_t)s + k]);
      lo[k] = min(lo[k], b);
      hi[k] = max(hi[k], b);
    }
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; k++) {
      atomicMin(&mm[f * 6 + k], lo[k]);
      atomicMax(&mm[f * 6 + 3 + k], hi[k]);
    }
}

// Completes the no-pbc frame of every frame: bounding-box origin and widths
// for binning and the fixed-point frame; cell counts bounded by ncell_cap.
// For NLISTCELLS this is LinkCells::setupCells(pos) (LinkCells.cpp:48-68).
__global__ void k_bounds_finish(KArgs a, const unsigned long long *mm, double cutoff, int linkcells) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= a.nframes) return;
  FrameConst &fc = a.fc[f];
  double lo[3], hi[3];
  for (int k = 0; k < 3; k++) {
    lo[k] = from_ordered(mm[f * 6 + k]);
    hi[k] = from_ordered(mm[f * 6 + 3 + k]);
    if (a.ns == 0) lo[k] = hi[k] = 0.0;
  }
  if (linkcells) {
    double box[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 3; k++) {
      if (cutoff < 1.3407807929942596e154)
        box[4 * k] = cutoff * (1 + ceil((hi[k] - lo[k]) / cutoff));
      else
        box[4 * k] = hi[k] - lo[k] + 1;
      fc.grid.lo[k] = (lo[k] + hi[k]) / 2;
    }
    // Pbc::setBox of the diagonal bounding box: invBox = inverse(box)
    const double det = box[0] * box[4] * box[8];
    const double invdet = 1.0 / det;
    for (int i = 0; i < 9; i++) fc.pbc.invbox[i] = 0.0;
    fc.pbc.invbox[0] = invdet * (box[4] * box[8]);
    fc.pbc.invbox[4] = invdet * (box[0] * box[8]);
    fc.pbc.invbox[8] = invdet * (box[0] * box[4]);
    long long ncell = 1;
    for (int k = 0; k < 3; k++) {
      const double r = fc.pbc.invbox[4 * k];
      int n = (int)floor(1.0 / sqrt(r * r) / cutoff);
      if (n == 0) n = 1;
      fc.grid.nc[k] = n;
      ncell *= n;
    }
    if (ncell > a.ncell_cap) {
      // more link cells than were allocated: report instead of binning
      fc.grid.ncells = 0;
      a.nl_count[f * 4 + 3] = 1ull;
    } else {
      fc.grid.ncells = (int)ncell;
    }
  } else {
    int nc[3];
    double width[3];
    for (int k = 0; k < 3; k++) {
      width[k] = (hi[k] - lo[k]) > 0 ? (hi[k] - lo[k]) : 1.0;
      double n = floor(width[k] / (cutoff * (1.0 + 1e-9)));
      nc[k] = (int)fmin(fmax(n, 1.0), 1024.0);
    }
    while ((long long)nc[0] * nc[1] * nc[2] > a.ncell_cap) {
      int kmax = (nc[0] >= nc[1] && nc[0] >= nc[2]) ? 0 : (nc[1] >= nc[2] ? 1 : 2);
      nc[kmax] = max(1, nc[kmax] / 2);
    }
    for (int k = 0; k < 3; k++) {
      fc.grid.nc[k] = nc[k];
      fc.grid.lo[k] = lo[k];
      fc.grid.inv_width[k] = 1.0 / width[k];
    }
    fc.grid.ncells = nc[0] * nc[1] * nc[2];
  }
  // fixed-point frame: twice the span so differences never wrap.  With
  // NLISTCELLS grid.lo stays the LinkCells origin (the box centre); the
  // fixed-point differences are modular, so any origin works.
  double spanmax = 0.0;
  for (int k = 0; k < 3; k++) {
    const double span = fmax(hi[k] - lo[k], 1e-3) * 2.0 + 1e-3;
    if (!linkcells) fc.grid.lo[k] = lo[k];
    fc.inv_l[k] = 1.0 / span;
    fc.scale[k] = (float)(span / 4294967296.0);
    spanmax = fmax(spanmax, span);
  }
  fixed_frame_finish(fc);
  // FP32 prefilter band around cutoff^2 (covers quantisation and rounding)
  const double band = 1e-4 * fc.cut2 + 8.0 * cutoff * spanmax / 4294967296.0 + 1e-12;
  fc.cut2_lo = (float)(fc.cut2 - band);
  fc.cut2_hi = (float)(fc.cut2 + band);
}

__global__ void k_bin(KArgs a) {
  const int f = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.ns) return;
  const FrameConst &fc = a.fc[f];
  if (fc.grid.ncells <= 0 || fc.grid.ncells > a.ncell_cap) return;
  const int c = cell_index_of(fc, a.pos + ((size_t)f * a.ns + s) * 3, a.nl_kind, a.do_pbc);
  a.cell_of_slot[(size_t)f * a.ns + s] = c;
  atomicAdd(&a.cell_count[(size_t)f * a.ncell_cap + c], 1);
}

// exclusive scan of the cell counts, one block per frame
__global__ void k_scan_cells(KArgs a) {
  const int f = blockIdx.x;
  const int n = min(max(a.fc[f].grid.ncells, 0), a.ncell_cap);
  int *cnt = a.cell_count + (size_t)f * a.ncell_cap;
  int *start = a.cell_start + (size_t)f * (a.ncell_cap + 1);
  int *fill = a.cell_fill + (size_t)f * a.ncell_cap;
  __shared__ int warp_tot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(lo + per, n);
  int local = 0;
  for (int i = lo; i < hi; i++) local += cnt[i];
  // block exclusive scan of 'local'
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += y;
    }
    warp_tot[lane] = v;
  }
  __syncthreads();
  int run = incl - local + (warp > 0 ? warp_tot[warp - 1] : 0);
  for (int i = lo; i < hi; i++) {
    start[i] = run;
    run += cnt[i];
    cnt[i] = 0;  // reset for the next build
    fill[i] = 0;
  }
  if (threadIdx.x == blockDim.x - 1) start[n] = run;
}

__global__ void k_scatter(KArgs a) {
  const int f = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.ns) return;
  if (a.fc[f].grid.ncells <= 0) return;
  const int c = a.cell_of_slot[(size_t)f * a.ns + s];
  const int p = a.cell_start[(size_t)f * (a.ncell_cap + 1) + c] + atomicAdd(&a.cell_fill[(size_t)f * a.ncell_cap + c], 1);
  if (p < a.ns) a.scatter_tmp[(size_t)f * a.ns + p] = s;
}

// Orders each cell's members by slot index (rank = number of smaller
// members), which makes the sorted order independent of atomic timing.  One
// warp per cell: a cell of up to 32 members ranks them by shuffles, a larger
// one by a loop over its members.
__global__ void __launch_bounds__(256) k_cell_sort(KArgs a) {
  const int f = blockIdx.y;
  const int n = min(max(a.fc[f].grid.ncells, 0), a.ncell_cap);
  const int *start = a.cell_start + (size_t)f * (a.ncell_cap + 1);
  const int *tmp = a.scatter_tmp + (size_t)f * a.ns;
  int *out = a.slot_of_rank + (size_t)f * a.ns;
  int *inv = a.rank_of_slot + (size_t)f * a.ns;
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int c = blockIdx.x * nw + (threadIdx.x >> 5); c < n; c += gridDim.x * nw) {  // warp-uniform
    const int b = start[c], m = start[c + 1] - b;
    if (m <= 32) {
      const int v = lane < m ? tmp[b + lane] : 0x7fffffff;
      int r = 0;
      for (int j = 0; j < m; j++) r += (__shfl_sync(0xffffffffu, v, j) < v) ? 1 : 0;
      if (lane < m) {
        out[b + r] = v;
        inv[v] = b + r;
      }
    } else {
      for (int i = lane; i < m; i += 32) {
        const int v = tmp[b + i];
        int r = 0;
        for (int j = 0; j < m; j++) r += (tmp[b + j] < v);
        out[b + r] = v;
        inv[v] = b + r;
      }
    }
  }
}

// Block-staged contiguous copies between a slot-ordered AoS array of 3
// doubles per slot and shared memory: every warp access covers 32
// consecutive doubles (whole lines, also across a CPU-GPU link), where one
// thread per slot touching its own 3 doubles would leave holes in every
// access.
constexpr int kSlotBlock = 256;
__device__ __forceinline__ void stage_in3(double *sh, const double *src, int nb) {
  for (int k = threadIdx.x; k < 3 * nb; k += blockDim.x) sh[k] = src[k];
}
__device__ __forceinline__ void stage_out3(double *dst, const double *sh, int nb) {
  for (int k = threadIdx.x; k < 3 * nb; k += blockDim.x) dst[k] = sh[k];
}

// Host-array calls on devices that access pageable host memory in place:
// positions read from the caller's array in slot order (coalesced across the
// link) and written as fixed-point values straight to rank order, replacing
// a copy and k_gather; derivatives read through rank_of_slot and written to
// the caller's array in slot order, replacing k_finalize32 and a copy.
__global__ void __launch_bounds__(kSlotBlock) k_prep_host(KArgs a, const double *__restrict__ hpos, int rank_order) {
  const int f = blockIdx.y + a.frame0;
  const int s0 = blockIdx.x * kSlotBlock;
  const int nb = min(kSlotBlock, a.ns - s0);
  if (nb <= 0) return;
  const size_t fo = (size_t)f * a.ns;
  __shared__ double sx[3 * kSlotBlock];
  stage_in3(sx, hpos + (fo + s0) * 3, nb);
  __syncthreads();
  const int t = threadIdx.x;
  float d2 = 0.f;
  if (t < nb) {
    const int s = s0 + t;
    const double xx[3] = {sx[3 * t], sx[3 * t + 1], sx[3 * t + 2]};
    const int r = rank_order ? a.rank_of_slot[fo + s] : s;
    const uint4 qq = fixed_of(a.fc[f], xx);
    a.q[fo + r] = qq;
    if (a.disp2) d2 = disp2_of(a.fc[f], a.q_build[fo + r], qq);
  }
  if (a.disp2) disp_max_block(a.disp2 + f, a.disp2 + a.disp2_frames + f, d2, t < nb);
}
__global__ void __launch_bounds__(kSlotBlock) k_finalize_host32(KArgs a, double *__restrict__ hderiv, int rank_order) {
  const int f = blockIdx.y + a.frame0;
  const int s0 = blockIdx.x * kSlotBlock;
  const int nb = min(kSlotBlock, a.ns - s0);
  if (nb <= 0) return;
  const size_t fo = (size_t)f * a.ns;
  __shared__ double sd[3 * kSlotBlock];
  const int t = threadIdx.x;
  if (t < nb) {
    const int s = s0 + t;
    const int r = rank_order ? a.rank_of_slot[fo + s] : s;
    const float4 v = a.acc32[fo + r];
    if (a.g) {  // backward: scaled by the frame's upstream dV/ds
      const double g = __ldg(a.g + f);
      if (fabs(g) > 1e-30 && fabs(g) < 1e30) {
        // in FP32 (the accumulators hold FP32-accurate derivatives; the
        // product adds at most 2^-24 relative), off the narrow FP64 pipe
        const float gf = (float)g;
        sd[3 * t] = f2d_int(gf * v.x);
        sd[3 * t + 1] = f2d_int(gf * v.y);
        sd[3 * t + 2] = f2d_int(gf * v.z);
      } else {
        sd[3 * t] = g * f2d_int(v.x);
        sd[3 * t + 1] = g * f2d_int(v.y);
        sd[3 * t + 2] = g * f2d_int(v.z);
      }
    } else {
      sd[3 * t] = f2d_int(v.x);
      sd[3 * t + 1] = f2d_int(v.y);
      sd[3 * t + 2] = f2d_int(v.z);
    }
    if (!a.keep_acc) a.acc32[fo + r] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();
  stage_out3(hderiv + (fo + s0) * 3, sd, nb);
}

// Force application from a saved forward (Colvar::apply, core/Colvar.cpp:50-60,
// with the daxpy of ActionWithValue::checkForForces, ActionWithValue.cpp:
// 337-411, and ActionAtomistic::setForcesOnAtoms, ActionAtomistic.cpp:502-541):
// atom_forces[frame][abs(slot)] += ff[frame] * ds/dx(slot), taken straight
// from the kept accumulators (rank order through rank_of_slot), which are
// cleared; atomics only when an absolute index occupies two slots.
template <typename Acc>
__global__ void k_apply_forces(KArgs a, int rank_order, const double *__restrict__ ff, long long n_atoms,
                               double *__restrict__ atom_forces) {
  const int f = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.ns) return;
  const size_t fo = (size_t)f * a.ns;
  const int r = rank_order ? a.rank_of_slot[fo + s] : s;
  double v[3];
  if constexpr (sizeof(Acc) == sizeof(float4)) {
    float4 *acc = reinterpret_cast<float4 *>(a.acc32) + fo + r;
    const float4 x = *acc;
    v[0] = x.x, v[1] = x.y, v[2] = x.z;
    *acc = make_float4(0.f, 0.f, 0.f, 0.f);
  } else {
    double *acc = a.acc64 + (fo + r) * 3;
    v[0] = acc[0], v[1] = acc[1], v[2] = acc[2];
    acc[0] = acc[1] = acc[2] = 0.0;
  }
  const double g = ff[f];
  double *o = atom_forces + ((size_t)f * n_atoms + a.abs_of_slot[s]) * 3;
  if (a.has_dup) {
    for (int k = 0; k < 3; k++) atomicAdd(o + k, g * v[k]);
  } else {
    for (int k = 0; k < 3; k++) o[k] += g * v[k];
  }
}
__global__ void k_apply_box_forces(int nframes, const double *__restrict__ ff, const double *__restrict__ vir,
                                   double *__restrict__ box_forces) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nframes * 9) return;
  box_forces[i] += ff[i / 9] * vir[i];
}

// FP64 positions in rank order (and the fixed-point copy for the NL prefilter
// and the mixed kernels).  rank_order==0: slot order.
// k_gather's work for rank r of frame f; returns the squared displacement
// since the rebuild when it is measured (0 otherwise).
__device__ __forceinline__ float gather_one(const KArgs &a, int f, int r, int rank_order, int want64, int wantq,
                                            int wantcell) {
  const int s = rank_order ? a.slot_of_rank[(size_t)f * a.ns + r] : r;
  if (wantcell) a.cell_of_rank[(size_t)f * a.ns + r] = a.cell_of_slot[(size_t)f * a.ns + s];
  const double *x = a.pos + ((size_t)f * a.ns + s) * 3;
  const double x0 = x[0], x1 = x[1], x2 = x[2];
  // the per-atom backward's upstream g rides in the spare fourth component
  const double gw = a.gslot ? a.gslot[(size_t)f * a.ns + s] : 0.0;
  if (want64) a.x64[(size_t)f * a.ns + r] = make_double4(x0, x1, x2, gw);
  if (wantq) {
    const double xx[3] = {x0, x1, x2};
    uint4 qq;
    if (a.qhi) {
      int4 hi;
      qq = fixed_of_hi(a.fc[f], xx, hi);
      a.qhi[(size_t)f * a.ns + r] = hi;
    } else {
      qq = fixed_of(a.fc[f], xx);
    }
    qq.w = __float_as_uint((float)gw);
    a.q[(size_t)f * a.ns + r] = qq;
    if (a.disp2) return disp2_of(a.fc[f], a.q_build[(size_t)f * a.ns + r], qq);
  }
  return 0.f;
}

__global__ void k_gather(KArgs a, int rank_order, int want64, int wantq, int wantcell) {
  const int f = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  float d2 = 0.f;
  if (r < a.ns) d2 = gather_one(a, f, r, rank_order, want64, wantq, wantcell);
  if (wantq && a.disp2) disp_max_block(a.disp2 + f, a.disp2 + a.disp2_frames + f, d2, r < a.ns);
}

// Orders each row of a rebuilt list near part first: entries whose FP32
// distance at the rebuild is within a.near_r2 (d_max + skin, squared, with a
// margin), then the rest.  A warp streams its slice's rows in lock step, kU
// entries and partner positions in flight per lane as in the pair pass: near
// entries are written back compacted to the front of the row (never ahead of
// what has been read), far ones to the row's column of a scratch list, and
// the far entries then follow the near ones.  Records the near counts, the
// slices' longest near parts, the rebuild positions, and zero displacements
// (this step's and the interval's).  One warp per slice, one lane per row.
template <int kU>
__global__ void __launch_bounds__(256) k_nl_partition(KArgs a) {
  const int f = blockIdx.y;
  const int lane = threadIdx.x & 31;
  const int slice = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (slice >= a.nslices) return;  // warp-uniform
  const size_t fo = (size_t)f * a.ns;
  const FrameConst &fc = a.fc[f];
  const int r = slice * 32 + lane;
  const bool active = r < a.ns;
  const size_t base = ((size_t)f * a.nslices + slice) * (size_t)a.cap * 32 + lane;
  uint32_t *row = a.ell + base, *far = a.ell_far + base;
  const int len = active ? a.row_len[fo + r] : 0;
  const int w = a.slice_w[(size_t)f * a.nslices + slice];
  const uint4 qr = active ? a.q[fo + r] : make_uint4(0u, 0u, 0u, 0u);
  if (active) a.q_build[fo + r] = qr;
  int nn = 0, nf = 0;
  for (int k = 0; k < w; k += kU) {
    uint32_t e[kU];
    uint4 qp[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) e[u] = (k + u < len) ? row[(size_t)(k + u) * 32] : 0xffffffffu;
#pragma unroll
    for (int u = 0; u < kU; u++) qp[u] = (e[u] != 0xffffffffu) ? a.q[fo + (e[u] & kRankMask)] : qr;
#pragma unroll
    for (int u = 0; u < kU; u++) {
      if (e[u] == 0xffffffffu) continue;
      const float dx = fixed_delta(qr.x, qp[u].x, fc.scale[0]), dy = fixed_delta(qr.y, qp[u].y, fc.scale[1]),
                  dz = fixed_delta(qr.z, qp[u].z, fc.scale[2]);
      if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= a.near_r2)
        row[(size_t)(nn++) * 32] = e[u];
      else
        far[(size_t)(nf++) * 32] = e[u];
    }
  }
  // the far entries after the near ones, four loads in flight
  for (int i = 0; i < nf; i += 4) {
    uint32_t t[4];
#pragma unroll
    for (int u = 0; u < 4; u++) t[u] = (i + u < nf) ? far[(size_t)(i + u) * 32] : 0u;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (i + u < nf) row[(size_t)(nn + i + u) * 32] = t[u];
  }
  if (active) a.row_near[fo + r] = nn;
  const int wmax = warp_max(nn);
  if (lane == 0) {
    a.slice_wn[(size_t)f * a.nslices + slice] = wmax;
    if (slice == 0 && a.disp2) {
      a.disp2[f] = 0u;
      a.disp2[a.disp2_frames + f] = 0u;
    }
  }
}

// Whether frame f's rows may be read up to their near parts: the skin is on
// and every atom has moved less than half of it since the rebuild, so an
// entry of a far part (beyond d_max + skin then) lies beyond d_max now,
// where every switching function is exactly zero.
__device__ __forceinline__ bool near_rows_only(const KArgs &a, int f) {
  return a.row_near != nullptr && a.disp2 != nullptr && a.disp_ok2 >= 0.f &&
         __uint_as_float(a.disp2[f]) <= a.disp_ok2;
}

// ---------------------------------------------------------------------------
// neighbour-list search: one thread per row (rank); exact pair set
// ---------------------------------------------------------------------------
// The cells a cell must look at: LinkCells::addRequiredCells
// (LinkCells.cpp:184-231) -- with at least 3 cells per periodic dimension
// this is the 27-cell stencil; with fewer, duplicates are avoided by the
// same min/max rules the reference uses.
__device__ __forceinline__ void cell_range(int c, int n, int wrap, int &lo, int &hi) {
  lo = c + ((n < 2) ? 0 : -1);
  hi = c + ((n < 3 && wrap) ? 1 : 2);
  if (!wrap) {
    lo = max(lo, 0);
    hi = min(hi, n);
  }
}
__device__ __forceinline__ int wrap_cell(int v, int n) { return (v < 0) ? n - 1 : v % n; }

// Candidate p of row r: ownership, cutoff test, group; stores the entry.
// Ordered so the common case (a candidate beyond the cutoff) costs an
// ownership test and an FP32 fixed-point distance; the slot, orientation,
// absolute indices and FP64 positions are read only for candidates that
// survive (about one in ten).
__device__ __forceinline__ void nl_candidate(const KArgs &a, const FrameConst &fc, int f, size_t fo, int r, int sr,
                                             bool ra, const uint4 &qr, int p, int sp, const uint4 &qp,
                                             size_t slice_base, int &n) {
  if (p == r) return;
  // ownership: even rank sum -> lower rank, odd -> higher rank
  if (((r + p) & 1) ? (r < p) : (r > p)) return;
  bool need_exact = true, accept = true;
  if (a.nl_kind != 2) {
    if (fc.fixed_ok) {
      const float dx = fixed_delta(qr.x, qp.x, fc.scale[0]);
      const float dy = fixed_delta(qr.y, qp.y, fc.scale[1]);
      const float dz = fixed_delta(qr.z, qp.z, fc.scale[2]);
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 > fc.cut2_hi) return;
      need_exact = !(r2 < fc.cut2_lo);
    }
  } else {
    need_exact = false;  // NLISTCELLS: every pair of neighbouring cells (NeighborList.cpp:194-231)
  }
  bool r_first;
  if (a.mode == MODE_TWO) {
    if (ra == (sp < a.nA)) return;
    r_first = ra;
  } else {
    r_first = sr < sp;
  }
  if (need_exact) {
    // the reference's own test: modulo2(pbc.distance(x[first], x[second])) <= cutoff^2
    const double4 xr4 = a.x64[fo + r], xp4 = a.x64[fo + p];
    const double va[3] = {xr4.x, xr4.y, xr4.z}, vb[3] = {xp4.x, xp4.y, xp4.z};
    double d[3];
    const double *v1 = r_first ? va : vb, *v2 = r_first ? vb : va;
    if (a.do_pbc)
      pbc_distance(fc.pbc, v1, v2, d);
    else
      for (int k = 0; k < 3; k++) d[k] = v2[k] - v1[k];
    accept = mod2(d) <= fc.cut2;
  }
  if (!accept) return;
  if (a.has_dup && a.abs_of_slot[sp] == a.abs_of_slot[sr]) {
    // a self pair: counted in the list size, skipped by the CV loop
    // (CoordinationBase.cpp:183); kept aside for coord_get_pairs
    unsigned long long k = atomicAdd(&a.nl_count[f * 4 + 1], 1ull);
    if (k < (unsigned long long)a.self_cap) {
      a.self_pairs[((size_t)f * a.self_cap + k) * 2] = r_first ? sr : sp;
      a.self_pairs[((size_t)f * a.self_cap + k) * 2 + 1] = r_first ? sp : sr;
    }
    return;
  }
  if (n < a.cap) a.ell[slice_base + (size_t)n * 32] = (uint32_t)p | (r_first ? kOrientBit : 0u);
  n++;
}

// x-adjacency of cells cx and cxp in a row of nc cells: the required-cell
// rule of LinkCells::addRequiredCells for one dimension.
__device__ __forceinline__ bool x_adjacent(int cx, int cxp, int nc, int wrap) {
  const int d = abs(cxp - cx);
  if (wrap) return nc < 3 || d <= 1 || d == nc - 1;
  return d <= 1;
}

constexpr int kSearchWarps = 4;

// The reference's own cutoff test for ranks (first, second) in its orientation:
// modulo2(pbc.distance(x[first], x[second])) <= cutoff^2
// (NeighborList.cpp:190-200).  Out of line: taken only inside the band.
__device__ __noinline__ bool nl_exact(const double4 *x64, const FrameConst *fc, int do_pbc, int first, int second) {
  const double4 x1 = x64[first], x2 = x64[second];
  const double v1[3] = {x1.x, x1.y, x1.z}, v2[3] = {x2.x, x2.y, x2.z};
  double d[3];
  if (do_pbc)
    pbc_distance(fc->pbc, v1, v2, d);
  else
    for (int k = 0; k < 3; k++) d[k] = v2[k] - v1[k];
  return mod2(d) <= fc->cut2;
}

// A candidate that passed the FP32 prefilter (r2 <= cut2_hi) of a classic
// list: group and orientation, the reference's own FP64 test when r2 lies in
// the band around cutoff^2 (in_band: r2 >= cut2_lo), self pairs, store.
__device__ __forceinline__ void nl_accept(const KArgs &a, const FrameConst &fc, int f, size_t fo, int r, int sr,
                                          bool ra, int p, int sp, bool in_band, size_t slice_base, int &n) {
  bool r_first;
  if (a.mode == MODE_TWO) {
    if (ra == (sp < a.nA)) return;
    r_first = ra;
  } else {
    r_first = sr < sp;
  }
  if (in_band && !nl_exact(a.x64 + fo, &fc, a.do_pbc, r_first ? r : p, r_first ? p : r)) return;
  if (a.has_dup && a.abs_of_slot[sp] == a.abs_of_slot[sr]) {
    // a self pair: counted in the list size, skipped by the CV loop
    // (CoordinationBase.cpp:183); kept aside for coord_get_pairs
    unsigned long long k = atomicAdd(&a.nl_count[f * 4 + 1], 1ull);
    if (k < (unsigned long long)a.self_cap) {
      a.self_pairs[((size_t)f * a.self_cap + k) * 2] = r_first ? sr : sp;
      a.self_pairs[((size_t)f * a.self_cap + k) * 2 + 1] = r_first ? sp : sr;
    }
    return;
  }
  if (n < a.cap) a.ell[slice_base + (size_t)n * 32] = (uint32_t)p | (r_first ? kOrientBit : 0u);
  n++;
}

// bit i of v to bit 2i (i < 16)
__device__ __forceinline__ uint32_t spread_even16(uint32_t v) {
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  return (v | (v << 1)) & 0x55555555u;
}

// Stores the accepted candidates of one staged batch (hit: bit j) in the
// lane's row, in j order; every check that can drop a hit has been made.
__device__ __forceinline__ int nl_store_row(const KArgs &a, uint32_t hit, int base, const uint4 *stage, int n, int sr,
                                            bool ra, size_t slice_base) {
  uint32_t *row = a.ell + slice_base;
  const bool two = a.mode == MODE_TWO;
  const int cap = a.cap;
  for (; hit; hit &= hit - 1u) {
    const int j = __ffs(hit) - 1;
    const bool r_first = two ? ra : (sr < (int)stage[j].w);
    if (n < cap) row[n * 32] = (uint32_t)(base + j) | (r_first ? kOrientBit : 0u);
    n++;
  }
  return n;
}

// Classic lists with a fixed-point frame (orthorhombic box or no PBC).  The
// slice's rows are processed one x-row of cells at a time; the candidates of a
// row pass are the ranks of at most 9 row segments (ranks are cell-major, x
// fastest), staged 32 at a time in shared memory and tested by every lane of
// the row.  kRel: candidates are staged as FP32 coordinates relative to the
// pass's first row (an exact integer difference of fixed-point positions, one
// rounding), so a test is three subtractions and a squared norm; otherwise
// each test takes the wrapped fixed-point difference itself.  Ownership (even
// rank sum -> lower rank, odd -> higher) selects every other candidate of a
// batch that lies wholly above or below the lane's rank.
template <bool kRel>
__device__ __forceinline__ int nl_row_pass(const KArgs &a, const FrameConst &fc, int f, size_t fo, int r, int sr, bool ra,
                                        uint4 qr, bool mine, int ry, int rz, int nint, int xa0, int xb0, int xa1,
                                        int xb1, uint4 qref, size_t slice_base, int lane, int n) {
  __shared__ uint4 stage_w[kSearchWarps][32];
  uint4 *stage = stage_w[threadIdx.x >> 5];
  const GridParams &g = fc.grid;
  const int *start = a.cell_start + (size_t)f * (a.ncell_cap + 1);
  const int *slot_of_rank = a.slot_of_rank + fo;
  const float sx = fc.scale[0], sy = fc.scale[1], sz = fc.scale[2];
  const float hi2 = fc.cut2_hi, lo2 = fc.cut2_lo;
  float mx = 0.f, my = 0.f, mz = 0.f;
  if (kRel) {
    mx = fixed_delta(qref.x, qr.x, sx);
    my = fixed_delta(qref.y, qr.y, sy);
    mz = fixed_delta(qref.z, qr.z, sz);
  }
  const int cwrap = g.wrap;
  int y0, y1, z0, z1;
  cell_range(ry, g.nc[1], cwrap, y0, y1);
  cell_range(rz, g.nc[2], cwrap, z0, z1);
  for (int ny = y0; ny < y1; ++ny)
    for (int nz = z0; nz < z1; ++nz) {
      const int rowcell = wrap_cell(ny, g.nc[1]) * g.nc[0] + wrap_cell(nz, g.nc[2]) * g.nc[0] * g.nc[1];
      for (int it = 0; it < nint; it++) {
        const int rb = start[rowcell + (it ? xa1 : xa0)], re = start[rowcell + (it ? xb1 : xb0) + 1];
        for (int base = rb; base < re; base += 32) {
          const int m = min(32, re - base);
          int sp = 0;
          if (lane < m) {
            const int p = base + lane;
            const uint4 qp = a.q[fo + p];
            sp = slot_of_rank[p];
            if (kRel)
              stage[lane] = make_uint4(__float_as_uint(fixed_delta(qref.x, qp.x, sx)),
                                       __float_as_uint(fixed_delta(qref.y, qp.y, sy)),
                                       __float_as_uint(fixed_delta(qref.z, qp.z, sz)), (uint32_t)sp);
            else
              stage[lane] = make_uint4(qp.x, qp.y, qp.z, (uint32_t)sp);
          }
          // two lists: the batch's candidates of GROUPB (bit j)
          const uint32_t in_b = __ballot_sync(0xffffffffu, lane < m && sp >= a.nA);
          __syncwarp();
          // branch-free tests record the candidates within cut2_hi (hit) and
          // those inside the band (band) as bits of j; the accepted ones are
          // stored afterwards by the whole warp
          uint32_t hit = 0u, band = 0u;
          if (mine) {
            auto test = [&](int j) {
              const uint4 c = stage[j];
              float dx, dy, dz;
              if (kRel) {
                dx = __uint_as_float(c.x) - mx;
                dy = __uint_as_float(c.y) - my;
                dz = __uint_as_float(c.z) - mz;
              } else {
                dx = fixed_delta(qr.x, c.x, sx);
                dy = fixed_delta(qr.y, c.y, sy);
                dz = fixed_delta(qr.z, c.z, sz);
              }
              const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
              hit |= (r2 <= hi2 ? 1u : 0u) << j;
              band |= (r2 < lo2 ? 0u : 1u) << j;
            };
            if (r < base || r >= base + m) {
              // the whole batch lies above r (owned when r + p is even) or
              // below it (owned when r + p is odd): every other candidate
              const int j0 = (r < base) ? ((r - base) & 1) : ((r - base + 1) & 1);
              if (m == 32) {
                // a full batch: 16 independent tests at j0 + 2i with
                // compile-time bit positions, spread to bit j afterwards
                uint32_t h16 = 0u, b16 = 0u;
#pragma unroll
                for (int i = 0; i < 16; i++) {
                  const uint4 c = stage[j0 + 2 * i];
                  float dx, dy, dz;
                  if (kRel) {
                    dx = __uint_as_float(c.x) - mx;
                    dy = __uint_as_float(c.y) - my;
                    dz = __uint_as_float(c.z) - mz;
                  } else {
                    dx = fixed_delta(qr.x, c.x, sx);
                    dy = fixed_delta(qr.y, c.y, sy);
                    dz = fixed_delta(qr.z, c.z, sz);
                  }
                  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                  h16 |= (r2 <= hi2 ? 1u : 0u) << i;
                  b16 |= (r2 < lo2 ? 0u : 1u) << i;
                }
                hit = spread_even16(h16) << j0;
                band = (h16 & b16) ? spread_even16(h16 & b16) << j0 : 0u;
              } else {
                int j = j0;
                for (; j + 2 < m; j += 4) {
                  test(j);
                  test(j + 2);
                }
                if (j < m) test(j);
              }
            } else {
              for (int j = 0; j < m; j++) {
                const int p = base + j;
                if (p == r || ((((r + p) & 1) != 0) ? (r < p) : (r > p))) continue;
                test(j);
              }
            }
            if (a.mode == MODE_TWO) hit &= ra ? in_b : ~in_b;
            // hits inside the band: the reference's own FP64 test decides
            for (uint32_t bh = hit & band; bh; bh &= bh - 1u) {
              const int j = __ffs(bh) - 1;
              const int p = base + j, sp_j = (int)stage[j].w;
              const bool r_first = (a.mode == MODE_TWO) ? ra : (sr < sp_j);
              if (!nl_exact(a.x64 + fo, &fc, a.do_pbc, r_first ? r : p, r_first ? p : r)) hit &= ~(1u << j);
            }
            if (a.has_dup) {
              // duplicated atoms: self pairs are set aside one by one
              for (; hit; hit &= hit - 1u) {
                const int j = __ffs(hit) - 1;
                nl_accept(a, fc, f, fo, r, sr, ra, base + j, (int)stage[j].w, false, slice_base, n);
              }
            }
          }
          if (hit) n = nl_store_row(a, hit, base, stage, n, sr, ra, slice_base);
          __syncwarp();
        }
      }
    }
  return n;
}

// x intervals (at most two) of the cells within one cell of [cxa, cxb] in a
// row of nc cells, each cell once.
__device__ __forceinline__ int x_intervals(int cxa, int cxb, int nc, int cwrap, int *xi0, int *xi1) {
  if (cxb - cxa + 3 >= nc) {
    xi0[0] = 0;
    xi1[0] = nc - 1;
    return 1;
  }
  if (cwrap) {
    const int lo = cxa - 1, hi = cxb + 1;
    if (lo < 0) {
      xi0[0] = nc - 1;
      xi1[0] = nc - 1;
      xi0[1] = 0;
      xi1[1] = hi;
      return 2;
    }
    if (hi >= nc) {
      xi0[0] = lo;
      xi1[0] = nc - 1;
      xi0[1] = 0;
      xi1[1] = hi - nc;
      return 2;
    }
    xi0[0] = lo;
    xi1[0] = hi;
    return 1;
  }
  xi0[0] = max(cxa - 1, 0);
  xi1[0] = min(cxb + 1, nc - 1);
  return 1;
}

// Per-warp bookkeeping of a search: slice width, list size, overflow.
__device__ __forceinline__ void nl_slice_done(const KArgs &a, int f, int slice, int lane, bool active, int n) {
  const int wmax = warp_max(active ? n : 0);
  unsigned long long tot = active ? (unsigned long long)n : 0ull;
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (lane == 0 && slice < a.nslices) {
    a.slice_w[(size_t)f * a.nslices + slice] = min(wmax, a.cap);
    atomicAdd(&a.nl_count[f * 4 + 0], tot);
    if (wmax > a.cap) atomicMax(&a.nl_count[f * 4 + 2], (unsigned long long)wmax);
  }
}

// Classic lists (NLIST) over frames with a fixed-point frame (orthorhombic
// box or no PBC): one warp per slice of 32 ranks, one nl_row_pass per x-row of
// cells that the slice's rows occupy (usually one).
__global__ void __launch_bounds__(kSearchWarps * 32, 8) k_nl_search(KArgs a) {
  const int f = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slice = blockIdx.x * kSearchWarps + warp;
  const int r = slice * 32 + lane;
  const bool active = r < a.ns && slice < a.nslices;
  const FrameConst &fc = a.fc[f];
  const GridParams &g = fc.grid;
  const size_t fo = (size_t)f * a.ns;
  int n = 0;
  if (slice < a.nslices && g.ncells > 0) {
    const int sr = active ? a.slot_of_rank[fo + r] : 0;
    const bool ra = sr < a.nA;
    const int cr = active ? a.cell_of_rank[fo + r] : 0;
    const uint4 qr = active ? a.q[fo + r] : make_uint4(0, 0, 0, 0);
    const size_t slice_base = ((size_t)f * a.nslices + slice) * (size_t)a.cap * 32 + lane;
    const int last = min(31, a.ns - 1 - slice * 32);  // last active lane
    const int myrow = cr / g.nc[0];
    const double cut = sqrt(fc.cut2);
    int lo = 0;
    while (lo <= last) {  // warp-uniform passes over the x-rows of the slice
      const int row = __shfl_sync(0xffffffffu, myrow, lo);
      const unsigned inrow = __ballot_sync(0xffffffffu, active && myrow == row);
      const int hi = 31 - __clz(inrow);
      const int cxa = __shfl_sync(0xffffffffu, cr, lo) % g.nc[0];
      const int cxb = __shfl_sync(0xffffffffu, cr, hi) % g.nc[0];
      const uint4 qref = make_uint4(__shfl_sync(0xffffffffu, qr.x, lo), __shfl_sync(0xffffffffu, qr.y, lo),
                                    __shfl_sync(0xffffffffu, qr.z, lo), 0u);
      int xi0[2] = {0, 0}, xi1[2] = {0, 0};
      const int nint = x_intervals(cxa, cxb, g.nc[0], g.wrap, xi0, xi1);
      const int ry = row % g.nc[1], rz = row / g.nc[1];
      // relative FP32 coordinates are exact enough (error << the prefilter
      // band) while every offset from the reference row stays within 8
      // cutoffs, and give the minimum image while offsets stay below half the
      // box
      const double cw0 = g.wrap ? fc.pbc.box[0] / g.nc[0] : 1.0 / (g.inv_width[0] * g.nc[0]);
      const double cw1 = g.wrap ? fc.pbc.box[4] / g.nc[1] : 1.0 / (g.inv_width[1] * g.nc[1]);
      const double cw2 = g.wrap ? fc.pbc.box[8] / g.nc[2] : 1.0 / (g.inv_width[2] * g.nc[2]);
      const int spanx = cxb - cxa + 2;
      bool rel = fmax(spanx * cw0, 2.0 * fmax(cw1, cw2)) <= 8.0 * cut;
      if (g.wrap) rel = rel && 2 * spanx <= g.nc[0] && g.nc[1] >= 4 && g.nc[2] >= 4 && (cxb - cxa + 3 < g.nc[0]);
      const bool mine = active && lane >= lo && lane <= hi;
      if (rel)
        n = nl_row_pass<true>(a, fc, f, fo, r, sr, ra, qr, mine, ry, rz, nint, xi0[0], xi1[0], xi0[1], xi1[1], qref,
                              slice_base, lane, n);
      else
        n = nl_row_pass<false>(a, fc, f, fo, r, sr, ra, qr, mine, ry, rz, nint, xi0[0], xi1[0], xi0[1], xi1[1], qref,
                               slice_base, lane, n);
      lo = hi + 1;
    }
    if (active) a.row_len[fo + r] = min(n, a.cap);
  }
  nl_slice_done(a, f, slice, lane, active, n);
}

// NLISTCELLS (every pair of neighbouring link cells), or a classic list in a
// generic (triclinic) box: one warp per slice.  When the slice lies in one
// x-row the candidates are staged as in k_nl_search, with the x-adjacency test
// of the link cells; otherwise each lane walks its own 27 cells.
__global__ void __launch_bounds__(kSearchWarps * 32) k_nl_search_cells(KArgs a) {
  const int f = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slice = blockIdx.x * kSearchWarps + warp;
  const int r = slice * 32 + lane;
  const bool active = r < a.ns && slice < a.nslices;
  const FrameConst &fc = a.fc[f];
  const GridParams &g = fc.grid;
  const size_t fo = (size_t)f * a.ns;
  const int *slot_of_rank = a.slot_of_rank + fo;
  const int *start = a.cell_start + (size_t)f * (a.ncell_cap + 1);
  __shared__ uint4 sq[kSearchWarps][32];
  __shared__ int sslot[kSearchWarps][32];
  __shared__ int scx[kSearchWarps][32];
  int n = 0;
  if (slice < a.nslices && g.ncells > 0) {
    const int sr = active ? slot_of_rank[r] : 0;
    const bool ra = sr < a.nA;
    const int cr = active ? a.cell_of_rank[fo + r] : 0;
    const uint4 qr = active ? a.q[fo + r] : make_uint4(0, 0, 0, 0);
    const size_t slice_base = ((size_t)f * a.nslices + slice) * (size_t)a.cap * 32 + lane;
    const int last = min(31, a.ns - 1 - slice * 32);  // last active lane
    const int cx = cr % g.nc[0], cy = (cr / g.nc[0]) % g.nc[1], cz = cr / (g.nc[0] * g.nc[1]);
    const int cwrap = (a.nl_kind == 2) ? a.do_pbc : g.wrap;
    const bool cells_kind = a.nl_kind == 2;
    const int cfirst = __shfl_sync(0xffffffffu, cr, 0), clast = __shfl_sync(0xffffffffu, cr, last);
    const int rowfirst = cfirst / g.nc[0], rowlast = clast / g.nc[0];
    if (rowfirst == rowlast) {
      // every loop bound below is warp-uniform (taken from the slice's row,
      // not the lane's cell), so lanes past the end of a partial last slice
      // stage the same segments and meet every __syncwarp
      const int cxa = cfirst % g.nc[0], cxb = clast % g.nc[0];
      const int ry = rowfirst % g.nc[1], rz = rowfirst / g.nc[1];
      int xi0[2] = {0, 0}, xi1[2] = {0, 0};
      const int nint = x_intervals(cxa, cxb, g.nc[0], cwrap, xi0, xi1);
      int y0, y1, z0, z1;
      cell_range(ry, g.nc[1], cwrap, y0, y1);
      cell_range(rz, g.nc[2], cwrap, z0, z1);
      for (int ny = y0; ny < y1; ++ny)
        for (int nz = z0; nz < z1; ++nz) {
          const int rowcell = wrap_cell(ny, g.nc[1]) * g.nc[0] + wrap_cell(nz, g.nc[2]) * g.nc[0] * g.nc[1];
          for (int it = 0; it < nint; it++) {
            const int rb = start[rowcell + xi0[it]], re = start[rowcell + xi1[it] + 1];
            for (int base = rb; base < re; base += 32) {
              const int m = min(32, re - base);
              if (lane < m) {
                const int p = base + lane;
                sq[warp][lane] = a.q[fo + p];
                sslot[warp][lane] = slot_of_rank[p];
                if (cells_kind) scx[warp][lane] = a.cell_of_rank[fo + p] % g.nc[0];
              }
              __syncwarp();
              if (active)
                for (int j = 0; j < m; j++) {
                  if (cells_kind && !x_adjacent(cx, scx[warp][j], g.nc[0], cwrap)) continue;
                  nl_candidate(a, fc, f, fo, r, sr, ra, qr, base + j, sslot[warp][j], sq[warp][j], slice_base, n);
                }
              __syncwarp();
            }
          }
        }
    } else if (active) {
      int x0, x1, y0, y1, z0, z1;
      cell_range(cx, g.nc[0], cwrap, x0, x1);
      cell_range(cy, g.nc[1], cwrap, y0, y1);
      cell_range(cz, g.nc[2], cwrap, z0, z1);
      for (int nx = x0; nx < x1; ++nx)
        for (int ny = y0; ny < y1; ++ny)
          for (int nz = z0; nz < z1; ++nz) {
            const int c = wrap_cell(nx, g.nc[0]) + wrap_cell(ny, g.nc[1]) * g.nc[0] +
                          wrap_cell(nz, g.nc[2]) * g.nc[0] * g.nc[1];
            const int pe = start[c + 1];
            for (int p = start[c]; p < pe; p++)
              nl_candidate(a, fc, f, fo, r, sr, ra, qr, p, slot_of_rank[p], a.q[fo + p], slice_base, n);
          }
    }
    if (active) a.row_len[fo + r] = min(n, a.cap);
  }
  nl_slice_done(a, f, slice, lane, active, n);
}

// PAIR mode list: pair i kept when |d(i, i+nA)| <= cutoff (NeighborList.cpp:150-152,252-266)
__global__ void k_pair_flags(KArgs a) {
  const int f = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nA) return;
  const FrameConst &fc = a.fc[f];
  const double *p0 = a.pos + ((size_t)f * a.ns + i) * 3;
  const double *p1 = a.pos + ((size_t)f * a.ns + i + a.nA) * 3;
  double d[3];
  if (a.do_pbc)
    pbc_distance(fc.pbc, p0, p1, d);
  else
    for (int k = 0; k < 3; k++) d[k] = p1[k] - p0[k];
  const bool keep = mod2(d) <= fc.cut2;
  a.pair_flag[(size_t)f * a.nA + i] = keep ? 1 : 0;
  unsigned long long c = keep ? 1ull : 0ull;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(&a.nl_count[f * 4 + 0], c);
}

// ---------------------------------------------------------------------------
// finalize: sorted/slot accumulators -> FP64 derivatives in slot order; the
// accumulators are zeroed for the next step.
// ---------------------------------------------------------------------------
__global__ void k_finalize64(KArgs a, int rank_order) {
  const int f = blockIdx.y;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.ns) return;
  const size_t fo = (size_t)f * a.ns;
  const int s = rank_order ? a.slot_of_rank[fo + r] : r;
  double *acc = a.acc64 + (fo + r) * 3;
  if (a.out_deriv) {
    // backward: scaled by the upstream dV/ds of the frame
    const double g = a.g ? a.g[f] : 1.0;
    double *o = a.out_deriv + (fo + s) * 3;
    o[0] = g * acc[0];
    o[1] = g * acc[1];
    o[2] = g * acc[2];
  }
  if (a.out_peratom) {
    a.out_peratom[fo + s] = a.accw64[fo + r];
    a.accw64[fo + r] = 0.0;
  }
  if (!a.keep_acc) {
    acc[0] = 0.0;
    acc[1] = 0.0;
    acc[2] = 0.0;
  }
}
// Slot-major: each thread reads its slot's accumulator at the slot's rank;
// the block writes its 256 slots' derivatives as one contiguous range.
__global__ void __launch_bounds__(kSlotBlock) k_finalize32(KArgs a, int rank_order) {
  const int f = blockIdx.y + a.frame0;
  const int s0 = blockIdx.x * kSlotBlock;
  const int nb = min(kSlotBlock, a.ns - s0);
  if (nb <= 0) return;
  const size_t fo = (size_t)f * a.ns;
  __shared__ double sd[3 * kSlotBlock];
  const int t = threadIdx.x;
  if (t < nb) {
    const int s = s0 + t;
    const int r = rank_order ? a.rank_of_slot[fo + s] : s;
    const float4 v = a.acc32[fo + r];
    if (a.g) {  // backward: scaled by the frame's upstream dV/ds
      const double g = __ldg(a.g + f);
      if (fabs(g) > 1e-30 && fabs(g) < 1e30) {
        // in FP32 (the accumulators hold FP32-accurate derivatives; the
        // product adds at most 2^-24 relative), off the narrow FP64 pipe
        const float gf = (float)g;
        sd[3 * t] = f2d_int(gf * v.x);
        sd[3 * t + 1] = f2d_int(gf * v.y);
        sd[3 * t + 2] = f2d_int(gf * v.z);
      } else {
        sd[3 * t] = g * f2d_int(v.x);
        sd[3 * t + 1] = g * f2d_int(v.y);
        sd[3 * t + 2] = g * f2d_int(v.z);
      }
    } else {
      sd[3 * t] = f2d_int(v.x);
      sd[3 * t + 1] = f2d_int(v.y);
      sd[3 * t + 2] = f2d_int(v.z);
    }
    if (a.out_peratom) a.out_peratom[fo + s] = (double)v.w;
    if (!a.keep_acc) a.acc32[fo + r] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (!a.out_deriv) return;  // uniform
  __syncthreads();
  stage_out3(a.out_deriv + (fo + s0) * 3, sd, nb);
}


// ---------------------------------------------------------------------------
// FP64 pair math of one (first, second) pair: the reference's operations.
// Returns sigma; d, dfunc out.
// ---------------------------------------------------------------------------
// pairing(distance2, dfunc, i, j) of the sibling CVs of CoordinationBase,
// slots s1 = first, s2 = second of the pair (the operation order of the
// reference, built without FMA contraction):
//   DHENERGY  DHEnergy::pairing (DHEnergy.cpp:128-142)
//   GHBFIX    GHBFIX::pairing (GHBFIX.cpp:178-218)
__device__ __noinline__ double sibling_pairing(const KArgs &a, double distance2, int s1, int s2, double &dfunc) {
  if (a.cv == COORD_CV_DHENERGY) {
    const double distance = sqrt(distance2);
    const double invdistance = 1.0 / distance;
    const double tmp = exp(-a.dh_k * distance) * invdistance * a.dh_const * a.charge[s1] * a.charge[s2] / a.dh_eps;
    const double dtmp = -(a.dh_k + invdistance) * tmp;
    dfunc = dtmp * invdistance;
    return tmp;
  }
  const double scale = a.eta[a.n_types * a.ptype[s1] + a.ptype[s2]];
  if (distance2 > a.gh_dmax_sq) {
    dfunc = 0.0;
    return 0.;
  }
  const double distance = sqrt(distance2);
  const double rdist = distance - a.gh_d0;
  double result = -1., df = 0.0;
  if (rdist > 0.) {
    if (rdist > a.gh_c_dmax2) {
      result += (a.gh_A + a.gh_B * rdist + a.gh_C * rdist * rdist);
      df += a.gh_B + 2 * a.gh_C * rdist;
    } else {
      result += a.gh_D * (rdist * rdist);
      df += 2 * a.gh_D * rdist;
    }
    df /= distance;
  }
  dfunc = df * scale;
  return result * scale;
}

// One pair of the FP64 path in the reference's orientation: d = min-image
// of v2 - v1, the CV's pairing of r^2 = |d|^2.  s1, s2: slots of the first
// and second atom (read only by the sibling CVs).
__device__ __forceinline__ double pair_fp64(const KArgs &a, const SwitchParams &sw, const FrameConst &fc,
                                            const double v1[3], const double v2[3], int s1, int s2, double d[3],
                                            double &dfunc) {
  if (a.do_pbc)
    pbc_distance(fc.pbc, v1, v2, d);
  else
    for (int k = 0; k < 3; k++) d[k] = v2[k] - v1[k];
  if (a.cv != COORD_CV_COORDINATION) return sibling_pairing(a, mod2(d), s1, s2, dfunc);
  VD<double> r = sw_calculate_sqr<double>(sw, mod2(d));
  dfunc = r.d;
  return r.f;
}

// ds/dR_0 and ds/dD_0 of one pair (for COORD_FLAG_DR0 and the backward).
// sigma is a function of (r - d0)/r0 (stretched); the stretch/shift depend on
// R_0 and D_0 through sigma(0) and sigma(d_max), and for the R_0= syntax d_max
// itself is d0 + r0*1e-5^(1/(n-m)).  Derivatives are taken by central
// differences of the closed form in (r0, d0) at fixed r -- see
// param_grad_host() which precomputes the stretch sensitivities.
struct ParamGrad {
  double dstretch_dr0, dshift_dr0, dstretch_dd0, dshift_dd0;  // of the stretch/shift constants
};

} // namespace
} // namespace coordgpu
