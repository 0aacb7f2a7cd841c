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

#define NH_DISPATCH(NHV, CALL) \
  switch (NHV) {               \
  case 1: CALL(1); break;      \
  case 2: CALL(2); break;      \
  case 3: CALL(3); break;      \
  case 4: CALL(4); break;      \
  case 5: CALL(5); break;      \
  case 6: CALL(6); break;      \
  default: CALL(0); break;     \
  }

void launch_eval_nl32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int block, cudaStream_t s) {
  (void)block;
#define CALL(N) k_eval_nl32<N><<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, sw, s32)
  NH_DISPATCH(mixed_nh(sw), CALL)
#undef CALL
  g_launches += 1;
}

void launch_allpairs32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int tile, int nblocks,
                       cudaStream_t s) {
  const bool tri = a.mode == MODE_SINGLE;
  const int ni = tri ? a.ns : a.nA, nj = tri ? a.ns : a.ns - a.nA;
  const int nTi = (ni + tile - 1) / tile, nTj = (nj + tile - 1) / tile;
  const long long ntp = tri ? (long long)nTi * (nTi + 1) / 2 : (long long)nTi * nTj;
  const int nb = (int)std::max(1ll, std::min<long long>(ntp, nblocks));
  dim3 g(nb, 1, a.nframes);
#define CALLT(T, N) k_allpairs32<T, N><<<g, T, 0, s>>>(a, sw, s32, nTi, nTj, (int)ntp)
  if (tile == 64) {
#define CALL(N) CALLT(64, N)
    NH_DISPATCH(mixed_nh(sw), CALL)
#undef CALL
  } else if (tile == 256) {
#define CALL(N) CALLT(256, N)
    NH_DISPATCH(mixed_nh(sw), CALL)
#undef CALL
  } else {
#define CALL(N) CALLT(128, N)
    NH_DISPATCH(mixed_nh(sw), CALL)
#undef CALL
  }
#undef CALLT
  g_launches += 1;
}

void launch_pairs32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int use_flags, cudaStream_t s) {
#define CALL(N) k_pairs32<N><<<grid1(a.nA, 256, a.nframes), 256, 0, s>>>(a, sw, s32, use_flags)
  NH_DISPATCH(mixed_nh(sw), CALL)
#undef CALL
  g_launches += 1;
}

void launch_finalize32(const KArgs &a, int rank_order, cudaStream_t s) {
  k_finalize32<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, rank_order);
  g_launches += 1;
}

} // namespace coordgpu
