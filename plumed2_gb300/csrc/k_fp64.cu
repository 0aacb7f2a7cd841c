// k_fp64.cu -- neighbour-list build and FP64 pair kernels.
// Compiled with -fmad=false: every FP64 expression keeps the reference's
// rounding (no fused multiply-add), which the exact cutoff test and the
// bit-level parity of per-pair values rely on.
#include "launch.h"
#include "eval.cuh"

namespace coordgpu {

std::atomic<long long> g_launches{0};

static inline dim3 grid1(int n, int block, int frames) { return dim3((n + block - 1) / block > 0 ? (n + block - 1) / block : 1, frames); }

void launch_bounds(const KArgs &a, unsigned long long *mm, double cutoff, int linkcells, cudaStream_t s) {
  const int blocks = std::max(1, std::min(1024, (a.ns + 255) / 256));
  k_bounds<<<dim3(blocks, a.nframes), 256, 0, s>>>(a, mm);
  k_bounds_finish<<<(a.nframes + 63) / 64, 64, 0, s>>>(a, mm, cutoff, linkcells);
  g_launches += 2;
}

void launch_nl_build(const KArgs &a, bool classic, cudaStream_t s) {
  cudaMemsetAsync(a.cell_count, 0, sizeof(int) * (size_t)a.ncell_cap * a.nframes, s);
  k_bin<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a);
  k_scan_cells<<<a.nframes, 1024, 0, s>>>(a);
  k_scatter<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a);
  k_cell_sort<<<dim3(std::max(1, std::min((a.cells_launch + 7) / 8, 65535)), a.nframes), 256, 0, s>>>(a);
  k_gather<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, 1, 1, 1, 1);
  const dim3 sgrid((a.nslices + kSearchWarps - 1) / kSearchWarps, a.nframes);
  if (classic)
    k_nl_search<<<sgrid, kSearchWarps * 32, 0, s>>>(a);
  else
    k_nl_search_cells<<<sgrid, kSearchWarps * 32, 0, s>>>(a);
  g_launches += 6;
}

namespace {
__global__ void k_stream_copy2(const double2 *__restrict__ src, double2 *__restrict__ dst, size_t n2,
                               const double *__restrict__ s1, double *__restrict__ d1, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) d1[n - 1] = s1[n - 1];
}
__global__ void k_stream_copy(const double *__restrict__ src, double *__restrict__ dst, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
}  // namespace

void launch_copy(const double *src, double *dst, size_t n, cudaStream_t s) {
  if (n == 0) return;
  if ((((uintptr_t)src | (uintptr_t)dst) & 15u) == 0) {
    // 16-byte vectors: half the transactions across a CPU-GPU link
    const size_t n2 = n / 2;
    const size_t blocks = std::max<size_t>(1, std::min<size_t>((n2 + 255) / 256, 2048));
    k_stream_copy2<<<(unsigned)blocks, 256, 0, s>>>((const double2 *)src, (double2 *)dst, n2, src, dst, n);
    g_launches += 1;
    return;
  }
  const size_t blocks = std::min<size_t>((n + 255) / 256, 2048);
  k_stream_copy<<<(unsigned)blocks, 256, 0, s>>>(src, dst, n);
  g_launches += 1;
}

void launch_apply_forces(const KArgs &a, bool mixed, int rank_order, const double *ff, long long n_atoms,
                         double *atom_forces, const double *vir, double *box_forces, cudaStream_t s) {
  if (atom_forces && a.ns > 0) {
    if (mixed)
      k_apply_forces<float4><<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, rank_order, ff, n_atoms, atom_forces);
    else
      k_apply_forces<double><<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, rank_order, ff, n_atoms, atom_forces);
    g_launches += 1;
  }
  if (box_forces) {
    k_apply_box_forces<<<(a.nframes * 9 + 127) / 128, 128, 0, s>>>(a.nframes, ff, vir, box_forces);
    g_launches += 1;
  }
}

void launch_nl_partition(const KArgs &a, cudaStream_t s) {
  k_nl_partition<4><<<dim3((a.nslices + 7) / 8 > 0 ? (a.nslices + 7) / 8 : 1, a.nframes), 256, 0, s>>>(a);
  g_launches += 1;
}

void launch_pair_flags(const KArgs &a, cudaStream_t s) {
  k_pair_flags<<<grid1(a.nA, 256, a.nframes), 256, 0, s>>>(a);
  g_launches += 1;
}

void launch_gather(const KArgs &a, int rank_order, int want64, int wantq, cudaStream_t s) {
  k_gather<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, rank_order, want64, wantq, 0);
  g_launches += 1;
}

#define MODE_DISPATCH(M, CALL) \
  switch (M) {                   \
  case EVAL_S: CALL(EVAL_S); break; \
  case EVAL_PARAM: CALL(EVAL_PARAM); break; \
  default: CALL(EVAL_DERIV); break; \
  }

void launch_eval_nl64(const KArgs &a, const SwitchParams &sw, int mode, const SwitchF32 *prefilter, int min_blocks,
                      cudaStream_t s) {
  if (prefilter) {
    // one warp per slice: (nslices + 7) / 8 blocks per frame, as many as
    // grid1(ns, 256) gives below
    const dim3 g((a.nslices + 7) / 8 > 0 ? (a.nslices + 7) / 8 : 1, a.nframes);
    // fixedRational<6> (the default NN=6, MM=12 switch) compiled with N fixed
    if (sw.type == SW_RATFIX && sw.nn == 6) {
#define CALLQ(M) k_eval_nl64q<M, 4, 3><<<g, 256, 0, s>>>(a, sw, *prefilter)
      if (mode == EVAL_PERATOM)
        CALLQ(EVAL_PERATOM);
      else if (mode == EVAL_VJP)
        CALLQ(EVAL_VJP);
      else
        MODE_DISPATCH(mode, CALLQ)
#undef CALLQ
    } else {
#define CALLQ(M) k_eval_nl64q<M, 4, 0><<<g, 256, 0, s>>>(a, sw, *prefilter)
      if (mode == EVAL_PERATOM)
        CALLQ(EVAL_PERATOM);
      else if (mode == EVAL_VJP)
        CALLQ(EVAL_VJP);
      else
        MODE_DISPATCH(mode, CALLQ)
#undef CALLQ
    }
    g_launches += 1;
    return;
  }
  // one thread per row: blocks of 256 rows, fewer (down to one warp) while
  // the launch would have under min_blocks blocks -- on the FP64 pipe (two
  // lanes per clock per SM) a small system otherwise runs on a few SMs; a
  // frame's blocks stay within its max_blocks records
  int bd = 256;
  while (bd > 32 && (long long)((a.ns + bd - 1) / bd) * a.nframes < min_blocks &&
         (a.ns + bd / 2 - 1) / (bd / 2) <= a.max_blocks)
    bd /= 2;
#define CALL(M) k_eval_nl64<M><<<grid1(a.ns, bd, a.nframes), bd, 0, s>>>(a, sw)
  if (mode == EVAL_PERATOM)
    CALL(EVAL_PERATOM);
  else if (mode == EVAL_VJP)
    CALL(EVAL_VJP);
  else
    MODE_DISPATCH(mode, CALL)
#undef CALL
  g_launches += 1;
}

void launch_allpairs64(const KArgs &a, const SwitchParams &sw, int mode, int tile, int nblocks, cudaStream_t s) {
  const bool tri = a.mode == MODE_SINGLE;
  const int ni = tri ? a.ns : a.nA, nj = tri ? a.ns : a.ns - a.nA;
  const int nTi = (ni + tile - 1) / tile, nTj = (nj + tile - 1) / tile;
  const long long ntp = tri ? (long long)nTi * (nTi + 1) / 2 : (long long)nTi * nTj;
  const int nb = (int)std::max(1ll, std::min<long long>(ntp, nblocks));
  dim3 g(nb, 1, a.nframes);
  if (tile == 32) {
#define CALL(M) k_allpairs64<32, M><<<g, 32, 0, s>>>(a, sw, nTi, nTj, (int)ntp)
    MODE_DISPATCH(mode, CALL)
#undef CALL
  } else if (tile == 128) {
#define CALL(M) k_allpairs64<128, M><<<g, 128, 0, s>>>(a, sw, nTi, nTj, (int)ntp)
    MODE_DISPATCH(mode, CALL)
#undef CALL
  } else {
#define CALL(M) k_allpairs64<64, M><<<g, 64, 0, s>>>(a, sw, nTi, nTj, (int)ntp)
    MODE_DISPATCH(mode, CALL)
#undef CALL
  }
  g_launches += 1;
}

void launch_pairs64(const KArgs &a, const SwitchParams &sw, int mode, int use_flags, cudaStream_t s) {
#define CALL(M) k_pairs64<M><<<grid1(a.nA, 256, a.nframes), 256, 0, s>>>(a, sw, use_flags)
  MODE_DISPATCH(mode, CALL)
#undef CALL
  g_launches += 1;
}

void launch_grad_post(const KArgs &a, const double *vir, const double *dpar, double *grad_box, double *grad_param,
                      cudaStream_t s) {
  k_grad_post<<<(a.nframes + 63) / 64, 64, 0, s>>>(a, vir, dpar, grad_box, grad_param);
  g_launches += 1;
}

void launch_finalize64(const KArgs &a, int rank_order, cudaStream_t s) {
  k_finalize64<<<grid1(a.ns, 256, a.nframes), 256, 0, s>>>(a, rank_order);
  g_launches += 1;
}

} // namespace coordgpu
