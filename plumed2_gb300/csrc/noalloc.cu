// noalloc.cu -- coord_forward_noalloc: the FP64 every-pair forward with its
// scratch in one fixed, statically allocated device array.
//
// Who needs it: MD engines that hand PLUMED device buffers out of their own
// pre-reserved memory pool and do not allow anything else to allocate on the
// device during a run (a cudaMalloc there can fail against the engine's
// budget, and it synchronises the whole device), and callers that cannot
// allocate at the point of the call at all.  They pass inputs and outputs; the
// working memory (the block partial sums of s and the virial, the completion
// ticket, the frame constants, the absolute indices and the derivative
// accumulators) comes from g_noalloc_scratch below, which every GPU that loads
// this library holds until the process exits.
//
// Limits and rules of use:
//  - at most kNoAllocMaxSlots (GROUPA + GROUPB) slots; larger groups are
//    rejected with COORD_ERR_ARG and a message;
//  - FP64, no NLIST, no PAIR (the every-pair kernel of k_fp64.cu);
//  - the array is shared by every call on a device and keeps the previous
//    call's contents, so each call first clears what must start at zero;
//    calls whose kernels overlap on the GPU (two streams, two threads) race
//    on it and must be serialised by the caller;
//  - the first call on each device resolves the array's device address with
//    cudaGetSymbolAddress (the host-side name is only a stand-in for it), so
//    make that first call before any stream capture begins.
// Compiled with -fmad=false like k_fp64.cu: the per-pair arithmetic is the
// same as the existing FP64 path.
#include "coordgpu.h"
#include "launch.h"
#include "eval.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace coordgpu {

// context accessors (coord_api.cu)
int ctx_noalloc_view(const coord_ctx *c, const SwitchParams **sw, const coord_params **p);
void ctx_set_error(coord_ctx *c, const char *msg);

namespace {

constexpr int kNoAllocMaxSlots = COORD_NOALLOC_MAX_SLOTS;
constexpr int kNoAllocTile = 64;
constexpr int kNoAllocMaxBlocks = 2048;

struct NoAllocScratch {
  FrameConst fc;
  unsigned ticket[4];
  double partials[kNoAllocMaxBlocks * kPartials];
  long long abs_of_slot[kNoAllocMaxSlots];
  double acc64[kNoAllocMaxSlots * 3];
};

// The scratch: about 1.2 MB per device (frame constants 4 KB, partial sums
// 192 KB, absolute indices 256 KB, derivative accumulators 768 KB).
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
NoAllocScratch *g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (resolved once).
int noalloc_scratch(int dev, NoAllocScratch **out) {
  if (dev < 0 || dev >= kMaxDevices) return COORD_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return COORD_ERR_CUDA;
    g_noalloc_ptr[dev] = static_cast<NoAllocScratch *>(ptr);
  }
  *out = g_noalloc_ptr[dev];
  return COORD_OK;
}

} // namespace
} // namespace coordgpu

using namespace coordgpu;

extern "C" int coord_forward_noalloc(coord_ctx *ctx, const int64_t *group_a, int64_t n_a, const int64_t *group_b,
                                     int64_t n_b, const double *pos, const double box[9], double *s, double *deriv,
                                     double *virial, void *stream) {
  const SwitchParams *sw = nullptr;
  const coord_params *p = nullptr;
  if (!ctx || ctx_noalloc_view(ctx, &sw, &p)) return COORD_ERR_ARG;
  if (n_a < 0 || n_b < 0 || (n_a && !group_a) || (n_b && !group_b) || !box || !s) return COORD_ERR_ARG;
  const int64_t ns = n_a + n_b;
  if (ns > kNoAllocMaxSlots) {
    char msg[160];
    std::snprintf(msg, sizeof msg,
                  "coord_forward_noalloc: %lld slots exceed its fixed scratch of %d slots (COORD_NOALLOC_MAX_SLOTS)",
                  (long long)ns, kNoAllocMaxSlots);
    ctx_set_error(ctx, msg);
    return COORD_ERR_ARG;
  }
  if (p->nlist != COORD_NL_NONE || p->pair || p->precision != COORD_PREC_FP64) {
    ctx_set_error(ctx, "coord_forward_noalloc: FP64 without NLIST or PAIR only");
    return COORD_ERR_UNSUPPORTED;
  }
  if (ns > 0 && (!pos || !deriv)) return COORD_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return COORD_ERR_CUDA;
  NoAllocScratch *scr = nullptr;
  if (int rc = noalloc_scratch(dev, &scr)) {
    ctx_set_error(ctx, "coord_forward_noalloc: cudaGetSymbolAddress of the scratch array failed");
    return rc;
  }

  // frame constants and absolute indices (host values copied in)
  FrameConst fc;
  std::memset(&fc, 0, sizeof fc);
  pbc_setup(box, &fc.pbc);
  cudaError_t e = cudaMemcpyAsync(&scr->fc, &fc, sizeof fc, cudaMemcpyHostToDevice, st);
  if (!e && n_a) e = cudaMemcpyAsync(scr->abs_of_slot, group_a, sizeof(int64_t) * n_a, cudaMemcpyHostToDevice, st);
  if (!e && n_b)
    e = cudaMemcpyAsync(scr->abs_of_slot + n_a, group_b, sizeof(int64_t) * n_b, cudaMemcpyHostToDevice, st);
  // what must start at zero: the completion ticket and the accumulators
  if (!e) e = cudaMemsetAsync(scr->ticket, 0, sizeof scr->ticket, st);
  if (!e && ns) e = cudaMemsetAsync(scr->acc64, 0, sizeof(double) * 3 * ns, st);
  if (e) return COORD_ERR_CUDA;
  if (ns < 2 && n_b == 0) {
    // no pair: s = 0, zero derivatives and virial
    e = cudaMemsetAsync(s, 0, sizeof(double), st);
    if (!e && virial) e = cudaMemsetAsync(virial, 0, 9 * sizeof(double), st);
    if (!e && ns) e = cudaMemsetAsync(deriv, 0, 3 * sizeof(double) * ns, st);
    return e ? COORD_ERR_CUDA : COORD_OK;
  }

  KArgs a{};
  a.nframes = 1;
  a.ns = (int)ns;
  a.nA = (int)(n_b ? n_a : ns);
  a.mode = n_b ? MODE_TWO : MODE_SINGLE;
  a.do_pbc = !p->nopbc;
  a.fc = &scr->fc;
  a.abs_of_slot = reinterpret_cast<const int64_t *>(scr->abs_of_slot);
  a.pos = pos;
  a.acc64 = scr->acc64;
  a.partials = scr->partials;
  a.max_blocks = kNoAllocMaxBlocks;
  a.tickets = scr->ticket;
  a.out_s = s;
  a.out_deriv = deriv;
  a.out_virial = virial;

  const bool tri = a.mode == MODE_SINGLE;
  const int ni = tri ? a.ns : a.nA, nj = tri ? a.ns : a.ns - a.nA;
  const int nTi = (ni + kNoAllocTile - 1) / kNoAllocTile, nTj = (nj + kNoAllocTile - 1) / kNoAllocTile;
  const long long ntp = tri ? (long long)nTi * (nTi + 1) / 2 : (long long)nTi * nTj;
  const int nb = (int)std::max(1ll, std::min<long long>(ntp, kNoAllocMaxBlocks));
  k_allpairs64<kNoAllocTile, EVAL_DERIV><<<dim3(nb, 1, 1), kNoAllocTile, 0, st>>>(a, *sw, nTi, nTj, (int)ntp);
  k_finalize64<<<dim3((a.ns + 255) / 256, 1), 256, 0, st>>>(a, 0);
  g_launches += 2;
  return cudaGetLastError() == cudaSuccess ? COORD_OK : COORD_ERR_CUDA;
}
