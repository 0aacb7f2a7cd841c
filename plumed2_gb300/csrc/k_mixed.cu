// k_mixed.cu -- FP32 pair kernels of the mixed-precision path.
#include "launch.h"
#include "eval.cuh"

namespace coordgpu {

static inline dim3 grid1(int n, int block, int frames) { return dim3((n + block - 1) / block > 0 ? (n + block - 1) / block : 1, frames); }

int mixed_nh(const SwitchParams &sw) {
  if (sw.type == SW_RATFIX && (sw.nn == 2 || sw.nn == 4 || sw.nn == 6 || sw.nn == 8 || sw.nn == 10 || sw.nn == 12))
    return sw.nn / 2;
  return 0;
}

// N/2 of fixedRational<N> compiled as its own kernel; other N and every other
// switch type use the generic FP32 evaluator (NH = 0).
#define NH_MODE_DISPATCH(NHV, M, CALL)       \
  do {                                       \
    const int nh_ = (NHV), m_ = (M);         \
    if (m_ == EVAL_S) {                      \
      if (nh_ == 3) CALL(3, EVAL_S);         \
      else if (nh_ == 2) CALL(2, EVAL_S);    \
      else if (nh_ == 4) CALL(4, EVAL_S);    \
      else if (nh_ == 6) CALL(6, EVAL_S);    \
      else CALL(0, EVAL_S);                  \
    } else if (m_ == EVAL_PARAM) {           \
      if (nh_ == 3) CALL(3, EVAL_PARAM);     \
      else if (nh_ == 2) CALL(2, EVAL_PARAM); \
      else if (nh_ == 4) CALL(4, EVAL_PARAM); \
      else if (nh_ == 6) CALL(6, EVAL_PARAM); \
      else CALL(0, EVAL_PARAM);              \
    } else {                                 \
      if (nh_ == 3) CALL(3, EVAL_DERIV);     \
      else if (nh_ == 2) CALL(2, EVAL_DERIV); \
      else if (nh_ == 4) CALL(4, EVAL_DERIV); \
      else if (nh_ == 6) CALL(6, EVAL_DERIV); \
      else CALL(0, EVAL_DERIV);              \
    }                                        \
  } while (0)

// The neighbour-list kernels also run the per-atom modes, compiled for
// fixedRational<6> and the generic evaluator only.
#define NH_MODE_DISPATCH_NL(NHV, M, CALL)                 \
  do {                                                   \
    const int nhn_ = (NHV), mn_ = (M);                   \
    if (mn_ == EVAL_PERATOM) {                           \
      if (nhn_ == 3) CALL(3, EVAL_PERATOM);              \
      else CALL(0, EVAL_PERATOM);                        \
    } else if (mn_ == EVAL_VJP) {                        \
      if (nhn_ == 3) CALL(3, EVAL_VJP);                  \
      else CALL(0, EVAL_VJP);                            \
    } else {                                             \
      NH_MODE_DISPATCH(nhn_, mn_, CALL);                 \
    }                                                    \
  } while (0)

static int nh_compiled(const SwitchParams &sw) {
  const int nh = mixed_nh(sw);
  return (nh == 2 || nh == 3 || nh == 4 || nh == 6) ? nh : 0;
}

void launch_eval_nl32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int nblocks,
                      int unroll, cudaStream_t s) {
  if (a.tric_band > 0.f) return launch_eval_nl32_tric(a, sw, s32, mode, nblocks, s);
  // persistent: nblocks blocks over all frames, at least one per frame, at
  // most one per 8 slices of a frame (8 warps per block)
  // (at most a.max_blocks: the records of a frame's blocks)
  const int per_frame =
      std::max(1, std::min(std::min((nblocks + a.nframes - 1) / a.nframes, (a.nslices + 7) / 8), a.max_blocks));
  const dim3 g(per_frame, a.nframes);
  if (unroll >= 8) {
#define CALL(N, M) k_eval_nl32<N, M, 8><<<g, 256, 0, s>>>(a, sw, s32)
    NH_MODE_DISPATCH_NL(nh_compiled(sw), mode, CALL);
#undef CALL
  } else if (unroll <= 2) {
#define CALL(N, M) k_eval_nl32<N, M, 2><<<g, 256, 0, s>>>(a, sw, s32)
    NH_MODE_DISPATCH_NL(nh_compiled(sw), mode, CALL);
#undef CALL
  } else {
#define CALL(N, M) k_eval_nl32<N, M, 4><<<g, 256, 0, s>>>(a, sw, s32)
    NH_MODE_DISPATCH_NL(nh_compiled(sw), mode, CALL);
#undef CALL
  }
  g_launches += 1;
}

void launch_band_fix(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, cudaStream_t s) {
  if (!(s32.dmax2_lo < s32.dmax2_hi)) return;  // no d_max: nothing to decide
  if (a.tric_band > 0.f) return launch_band_fix_tric(a, sw, s32, mode, s);
  const int chunks = (a.nslices + 31) / 32;  // one warp per 32 slices
  const dim3 g(std::max(1, std::min((chunks + 7) / 8, 8)), a.nframes);  // 8 blocks per frame: one wave
#define CALL(N, M) k_band_fix<N, M><<<g, 256, 0, s>>>(a, sw, s32)
  NH_MODE_DISPATCH_NL(nh_compiled(sw), mode, CALL);
#undef CALL
  g_launches += 1;
}

void launch_allpairs32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int tile, int nblocks,
                       cudaStream_t s) {
  if (a.tric_band > 0.f) return launch_allpairs32_tric(a, sw, s32, mode, tile, nblocks, s);
  const bool tri = a.mode == MODE_SINGLE;
  const int ni = tri ? a.ns : a.nA, nj = tri ? a.ns : a.ns - a.nA;
  const int nTi = (ni + tile - 1) / tile, nTj = (nj + tile - 1) / tile;
  const long long ntp = tri ? (long long)nTi * (nTi + 1) / 2 : (long long)nTi * nTj;
  const int nb = (int)std::max(1ll, std::min<long long>(ntp, nblocks));
  dim3 g(nb, 1, a.nframes);
  if (tile == 64) {
#define CALL(N, M) k_allpairs32<64, N, M><<<g, 64, 0, s>>>(a, sw, s32, nTi, nTj, (int)ntp)
    NH_MODE_DISPATCH(nh_compiled(sw), mode, CALL);
#undef CALL
  } else {
#define CALL(N, M) k_allpairs32<128, N, M><<<g, 128, 0, s>>>(a, sw, s32, nTi, nTj, (int)ntp)
    NH_MODE_DISPATCH(nh_compiled(sw), mode, CALL);
#undef CALL
  }
  g_launches += 1;
}

void launch_pairs32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int use_flags,
                    cudaStream_t s) {
  if (a.tric_band > 0.f) return launch_pairs32_tric(a, sw, s32, mode, use_flags, s);
#define CALL(N, M) k_pairs32<N, M><<<grid1(a.nA, 256, a.nframes), 256, 0, s>>>(a, sw, s32, use_flags)
  NH_MODE_DISPATCH(nh_compiled(sw), mode, CALL);
#undef CALL
  g_launches += 1;
}

void launch_prep_host(const KArgs &a, const double *hpos, int rank_order, cudaStream_t s) {
  k_prep_host<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, hpos, rank_order);
  g_launches += 1;
}

void launch_finalize_host32(const KArgs &a, double *hderiv, int rank_order, cudaStream_t s) {
  k_finalize_host32<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, hderiv, rank_order);
  g_launches += 1;
}

void launch_finalize32(const KArgs &a, int rank_order, cudaStream_t s) {
  k_finalize32<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, rank_order);
  g_launches += 1;
}

} // namespace coordgpu
