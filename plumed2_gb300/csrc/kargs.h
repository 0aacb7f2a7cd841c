// kargs.h -- kernel argument records shared by the launchers and the host runtime.
#pragma once
#include "coord_internal.h"
#include <cstdint>
#include <cuda_runtime.h>

namespace coordgpu {

constexpr int kPartials = 12;  // s, virial[9], ds/dR0, ds/dD0
constexpr int kBandQueueCap = 512;  // band pairs per frame the fix-up sorts in shared memory
constexpr uint32_t kOrientBit = 0x80000000u;
constexpr uint32_t kRankMask = 0x7fffffffu;

struct KArgs {
  int nframes;
  int ns;         // slots per frame
  int nA;         // slots in GROUPA (== ns for a single list)
  int mode;       // PairMode
  int do_pbc;     // !NOPBC
  int nl_kind;    // COORD_NL_* (1 classic, 2 cells)
  int cap;        // neighbour-list row capacity (entries per row)
  // > 0: the frames have generic (triclinic) boxes on the mixed path; the
  // relative half-width of the FP32 band around d_max^2 (Geo32<true>)
  float tric_band;
  int ncell_cap;  // cells per frame (allocation)
  int self_cap;   // self-pair list capacity per frame
  int nslices;    // ceil(ns/32)
  int flags;      // COORD_FLAG_* of the call
  int has_dup;    // some absolute index appears in two slots (self pairs possible)
  int keep_acc;   // finalize leaves the derivative accumulators in place (saved forward)
  int frame0;     // first frame of a launch over a range of the frames (host-array pipeline)
  FrameConst *fc;               // [nframes]
  const int64_t *abs_of_slot;   // [ns]
  const double *pos;            // [nframes][ns][3]   input, slot order
  int *cell_of_slot;            // [nframes][ns]
  int *cell_count;              // [nframes][ncell_cap]
  int *cell_start;              // [nframes][ncell_cap+1]
  int *cell_fill;               // [nframes][ncell_cap]
  int *slot_of_rank;            // [nframes][ns]
  int *rank_of_slot;            // [nframes][ns] inverse of slot_of_rank (neighbour-list build)
  int *cell_of_rank;            // [nframes][ns] cell of each rank (neighbour-list build)
  int *scatter_tmp;             // [nframes][ns]
  double4 *x64;                 // [nframes][ns] sorted (or slot-order) FP64 positions
  uint4 *q;                     // [nframes][ns] fixed-point positions
  int4 *qhi;                    // [nframes][ns] their high words (the box image of each coordinate), or null
  uint32_t *ell;                // [nframes][nslices*cap*32]
  int *row_len;                 // [nframes][ns]
  int *slice_w;                 // [nframes][nslices]
  // near/far rows (k_nl_partition): entries [0, row_near) of a row were
  // within d_max + skin of the row atom at the rebuild, the rest beyond it
  int *row_near;                // [nframes][ns] or null
  int *slice_wn;                // [nframes][nslices] the slice's longest near part
  uint32_t *ell_far;            // like ell: the partition's scratch for far entries
  uint4 *q_build;               // [nframes][ns] fixed-point positions at the rebuild (rank order)
  unsigned *disp2;              // [2][disp2_frames] the largest squared displacement since the rebuild
                                // (FP32 bits, max over atoms) of this step, and of every step since the
                                // rebuild; measured by the gather; or null
  int disp2_frames;             // the call's frame count (a launch over a chunk of frames keeps it)
  float near_r2;                // the partition's threshold: (d_max + skin)^2 (1 + 1e-5)
  float disp_ok2;               // near parts suffice while disp2 <= (skin/2)^2 (1 - 1e-5); < 0: off
  unsigned long long *nl_count; // [nframes][4]: pairs, self pairs, max row length, geometry error
  uint32_t *self_pairs;         // [nframes][self_cap][2]
  unsigned char *pair_flag;     // [nframes][nA] PAIR-mode neighbour flags
  double *acc64;                // [nframes][ns][3] derivative accumulators (FP64 path)
  float4 *acc32;                // [nframes][ns]    derivative accumulators (mixed path)
  double *partials;             // [nframes][max_blocks][kPartials]
  int max_blocks;
  int cells_launch;             // blocks of the per-cell sort (cells per frame, when known)
  unsigned *tickets;            // [nframes]
  // mixed NL pass: slices holding a pair whose FP32 r^2 lies in the band
  // around d_max^2, for the FP64 fix-up pass (k_band_fix)
  unsigned char *band_flag;     // [nframes][nslices]
  double *band_rec;             // [nframes][nslices][kPartials] per flagged slice
  unsigned *band_tickets;       // [nframes]
  // the band's pairs themselves, queued per frame by the pair kernel:
  // {frame, row rank, list entry, 0}; band_qn[f] counts frame f's (beyond
  // band_qcap only the flags above hold them), band_qn[disp2_frames] is set
  // when some frame's queue overflowed, band_qn[disp2_frames + 1] is the
  // fix-up's completion ticket
  uint4 *band_q;                // [disp2_frames][band_qcap]
  unsigned *band_qn;            // [disp2_frames + 2]
  double *band_qrec;            // [disp2_frames][band_qcap][kPartials]
  int band_qcap;
  double *out_s;                // [nframes]
  double *out_deriv;            // [nframes][ns][3] slot order
  double *out_virial;           // [nframes][9]
  double *out_dparam;           // [nframes][2]
  const double *g;              // [nframes] upstream dV/ds (backward)
  // per-atom coordination (EVAL_PERATOM / EVAL_VJP)
  double *out_peratom;          // [nframes][ns] slot order: sum of sigma over the slot's pairs
  double *accw64;               // [nframes][ns] FP64 path: those sums in rank order
  const double *gslot;          // [nframes][ns] slot order: upstream dV/dcn per slot (EVAL_VJP)
  // the CV's pairing() (COORD_CV_*): the switching function for COORDINATION,
  // or a sibling of CoordinationBase with its per-slot data
  int cv;
  const double *charge;         // [ns] DHENERGY: charge of each slot
  const int *ptype;             // [ns] GHBFIX: type id of each slot
  const double *eta;            // [n_types^2] GHBFIX scaling matrix
  int n_types;
  double dh_k, dh_const, dh_eps;                                    // DHEnergy.cpp:112-113
  double gh_dmax_sq, gh_d0, gh_c_dmax2, gh_A, gh_B, gh_C, gh_D;     // GHBFIX.cpp:111-126
};

// FP32 parameters of a fixedRational<2*NH> switch (mixed path), plus the
// constants of the R_0/D_0 gradients (SwitchParams::c_r0).
struct SwitchF32 {
  float dmax2, invr0_2, stretch, shift, c;  // c = -NH * 2*invr0^2 * stretch
  float d0, invr0, c_r0, c_d0;
  // band around d_max^2 inside which the FP32 r^2 cannot decide the
  // reference's inclusive test r^2 <= d_max^2: such pairs are decided in FP64
  float dmax2_lo, dmax2_hi;
  double dmax_2;  // the reference's d_max^2 (FP64)
};

// What a pair kernel accumulates.
enum EvalMode : int {
  EVAL_S = 0,        // s only
  EVAL_DERIV = 1,    // s, ds/dx, virial
  EVAL_PARAM = 2,    // s, ds/dx, virial, ds/dR_0, ds/dD_0
  EVAL_PERATOM = 3,  // EVAL_DERIV plus the per-atom sums of sigma (coordination numbers)
  EVAL_VJP = 4       // per-atom backward: each pair's derivative weighted by g_i + g_j
};

} // namespace coordgpu
