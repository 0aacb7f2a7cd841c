// k_mixed_tric.cu -- the mixed path's FP32 pair kernels for frames with a
// generic (triclinic) periodic box: Geo32<true> takes the pair displacement
// through the reduced cell and its octant shifts (Pbc.cpp:383-415), and the
// band around d_max^2 that the FP64 fix-up decides is widened to the error
// bound of that geometry (a.tric_band).  A translation unit of its own, so it
// compiles beside the orthorhombic kernels.
#include "launch.h"
#include "eval.cuh"

namespace coordgpu {

namespace {

dim3 grid1(int n, int block, int frames) { return dim3((n + block - 1) / block > 0 ? (n + block - 1) / block : 1, frames); }

SwitchF32 widened(const SwitchF32 &s32, float rel) {
  SwitchF32 w = s32;
  if (w.dmax2_lo < w.dmax2_hi) {
    w.dmax2_lo = (float)(s32.dmax_2 * (1.0 - (double)rel));
    w.dmax2_hi = (float)(s32.dmax_2 * (1.0 + (double)rel));
  }
  return w;
}

// fixedRational<6> as its own kernel, everything else on the generic
// evaluator (NH = 0)
int nh_tric(const SwitchParams &sw) { return mixed_nh(sw) == 3 ? 3 : 0; }

}  // namespace

#define TRIC_DISPATCH(NHV, M, CALL)                              \
  do {                                                           \
    const int nh_ = (NHV), m_ = (M);                             \
    if (m_ == EVAL_S) {                                          \
      if (nh_ == 3) CALL(3, EVAL_S); else CALL(0, EVAL_S);       \
    } else if (m_ == EVAL_PARAM) {                               \
      if (nh_ == 3) CALL(3, EVAL_PARAM); else CALL(0, EVAL_PARAM); \
    } else {                                                     \
      if (nh_ == 3) CALL(3, EVAL_DERIV); else CALL(0, EVAL_DERIV); \
    }                                                            \
  } while (0)
#define TRIC_DISPATCH_NL(NHV, M, CALL)                                 \
  do {                                                                 \
    const int nhn_ = (NHV), mn_ = (M);                                 \
    if (mn_ == EVAL_PERATOM) {                                         \
      if (nhn_ == 3) CALL(3, EVAL_PERATOM); else CALL(0, EVAL_PERATOM); \
    } else if (mn_ == EVAL_VJP) {                                      \
      if (nhn_ == 3) CALL(3, EVAL_VJP); else CALL(0, EVAL_VJP);        \
    } else {                                                           \
      TRIC_DISPATCH(nhn_, mn_, CALL);                                  \
    }                                                                  \
  } while (0)

void launch_eval_nl32_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int nblocks,
                           cudaStream_t s) {
  const SwitchF32 w = widened(s32, a.tric_band);
  // (at most a.max_blocks: the records of a frame's blocks)
  const int per_frame =
      std::max(1, std::min(std::min((nblocks + a.nframes - 1) / a.nframes, (a.nslices + 7) / 8), a.max_blocks));
  const dim3 g(per_frame, a.nframes);
#define CALL(N, M) k_eval_nl32<N, M, 4, true><<<g, 256, 0, s>>>(a, sw, w)
  TRIC_DISPATCH_NL(nh_tric(sw), mode, CALL);
#undef CALL
  g_launches += 1;
}

void launch_band_fix_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, cudaStream_t s) {
  const SwitchF32 w = widened(s32, a.tric_band);
  const int chunks = (a.nslices + 31) / 32;
  const dim3 g(std::max(1, std::min((chunks + 7) / 8, 8)), a.nframes);  // 8 blocks per frame: one wave
#define CALL(N, M) k_band_fix<N, M, true><<<g, 256, 0, s>>>(a, sw, w)
  TRIC_DISPATCH_NL(nh_tric(sw), mode, CALL);
#undef CALL
  g_launches += 1;
}

void launch_allpairs32_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int tile,
                            int nblocks, cudaStream_t s) {
  const SwitchF32 w = widened(s32, a.tric_band);
  const bool tri = a.mode == MODE_SINGLE;
  const int ni = tri ? a.ns : a.nA, nj = tri ? a.ns : a.ns - a.nA;
  const int nTi = (ni + tile - 1) / tile, nTj = (nj + tile - 1) / tile;
  const long long ntp = tri ? (long long)nTi * (nTi + 1) / 2 : (long long)nTi * nTj;
  const int nb = (int)std::max(1ll, std::min<long long>(ntp, nblocks));
  dim3 g(nb, 1, a.nframes);
  if (tile == 64) {
#define CALL(N, M) k_allpairs32<64, N, M, true><<<g, 64, 0, s>>>(a, sw, w, nTi, nTj, (int)ntp)
    TRIC_DISPATCH(nh_tric(sw), mode, CALL);
#undef CALL
  } else {
#define CALL(N, M) k_allpairs32<128, N, M, true><<<g, 128, 0, s>>>(a, sw, w, nTi, nTj, (int)ntp)
    TRIC_DISPATCH(nh_tric(sw), mode, CALL);
#undef CALL
  }
  g_launches += 1;
}

void launch_pairs32_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int use_flags,
                         cudaStream_t s) {
  const SwitchF32 w = widened(s32, a.tric_band);
#define CALL(N, M) k_pairs32<N, M, true><<<grid1(a.nA, 256, a.nframes), 256, 0, s>>>(a, sw, w, use_flags)
  TRIC_DISPATCH(nh_tric(sw), mode, CALL);
#undef CALL
  g_launches += 1;
}

}  // namespace coordgpu
