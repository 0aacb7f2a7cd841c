// launch.h -- host launchers of the kernels (defined in k_fp64.cu / k_mixed.cu).
#pragma once
#include "kargs.h"
#include "coordgpu.h"
#include <atomic>

namespace coordgpu {

// library-wide kernel launch counter (coord_launch_count)
extern std::atomic<long long> g_launches;

// k_fp64.cu (compiled with -fmad=false)
void launch_bounds(const KArgs &a, unsigned long long *mm, double cutoff, int linkcells, cudaStream_t s);
// classic: NLIST with a fixed-point frame in every frame (k_nl_search);
// otherwise NLISTCELLS or a generic box (k_nl_search_cells)
// dst[i] = src[i] for i < n, coalesced; either side may be any address the
// device can access (a pageable host array when the device uses the host
// page tables)
void launch_copy(const double *src, double *dst, size_t n, cudaStream_t s);
// force application from a saved forward (k_apply_forces, k_apply_box_forces)
void launch_apply_forces(const KArgs &a, bool mixed, int rank_order, const double *ff, long long n_atoms,
                         double *atom_forces, const double *vir, double *box_forces, cudaStream_t s);
// host-array calls: fixed-point positions from the caller's array straight
// to rank order; derivatives from the accumulators straight to the caller's
// array (mixed path)
void launch_prep_host(const KArgs &a, const double *hpos, int rank_order, cudaStream_t s);
void launch_finalize_host32(const KArgs &a, double *hderiv, int rank_order, cudaStream_t s);
void launch_nl_build(const KArgs &a, bool classic, cudaStream_t s);
// near part first in every row of a rebuilt list (k_nl_partition)
void launch_nl_partition(const KArgs &a, cudaStream_t s);
void launch_pair_flags(const KArgs &a, cudaStream_t s);
void launch_gather(const KArgs &a, int rank_order, int want64, int wantq, cudaStream_t s);
// prefilter: the FP32 parameters of the switch, for the fixed-point screen of
// k_eval_nl64q (orthorhombic frames of COORDINATION), or null
void launch_eval_nl64(const KArgs &a, const SwitchParams &sw, int mode, const SwitchF32 *prefilter, int min_blocks,
                      cudaStream_t s);
void launch_allpairs64(const KArgs &a, const SwitchParams &sw, int mode, int tile, int nblocks, cudaStream_t s);
void launch_pairs64(const KArgs &a, const SwitchParams &sw, int mode, int use_flags, cudaStream_t s);
void launch_finalize64(const KArgs &a, int rank_order, cudaStream_t s);
void launch_grad_post(const KArgs &a, const double *vir, const double *dpar, double *grad_box, double *grad_param,
                      cudaStream_t s);

// k_mixed.cu
// FP64 decision of d_max for the pairs the mixed NL pass left in the band
// around d_max^2 (after launch_eval_nl32, before the finalize kernel)
void launch_band_fix(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, cudaStream_t s);
void launch_eval_nl32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int nblocks,
                      int unroll, cudaStream_t s);
void launch_allpairs32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int tile, int nblocks,
                       cudaStream_t s);
void launch_pairs32(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int use_flags,
                    cudaStream_t s);
void launch_finalize32(const KArgs &a, int rank_order, cudaStream_t s);

// k_mixed_tric.cu: the same pair kernels for generic (triclinic) boxes
// (a.tric_band > 0), called by the launchers above; fixedRational<6> and the
// generic evaluator, one unroll, the D_MAX band widened to a.tric_band
void launch_eval_nl32_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int nblocks,
                           cudaStream_t s);
void launch_band_fix_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, cudaStream_t s);
void launch_allpairs32_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int tile,
                            int nblocks, cudaStream_t s);
void launch_pairs32_tric(const KArgs &a, const SwitchParams &sw, const SwitchF32 &s32, int mode, int use_flags,
                         cudaStream_t s);

// number of 32-lane switch specialisations compiled for the mixed path
int mixed_nh(const SwitchParams &sw);  // N/2 of fixedRational<N>, or 0 for the generic evaluator

// what multi.cu needs to know about a context (coord_api.cu)
struct MultiView {
  const coord_params *p;
  const SwitchParams *sw;
  const SwitchF32 *s32;
  int mode;
  int64_t nA, ns;
  const int64_t *abs;  // host copy of the groups
};
int ctx_multi_view(coord_ctx *c, MultiView *v);

// peaks.cu
int measure_peaks(int device, double *fp32, double *fp64, double *hbm);

} // namespace coordgpu
