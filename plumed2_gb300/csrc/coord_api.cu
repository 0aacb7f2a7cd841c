// coord_api.cu -- the C ABI (include/coordgpu.h): contexts, buffers, the
// per-step launch sequence.  Host code; kernels live in k_fp64.cu/k_mixed.cu.
#include "coordgpu.h"
#include "launch.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace coordgpu;

namespace {

template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t want) {
    if (want <= n && p) return cudaSuccess;
    // kernels queued on any stream may still use the old buffer
    if (p) {
      cudaDeviceSynchronize();
      cudaFree(p);
    }
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(want, 1) * sizeof(T));
    if (e == cudaSuccess) {
      n = std::max<size_t>(want, 1);
      // zero-filled before any kernel of the context's (non-blocking) stream can see it
      e = cudaMemset(p, 0, n * sizeof(T));
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

template <typename T> struct HostBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t want) {
    if (want <= n && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMallocHost(&p, std::max<size_t>(want, 1) * sizeof(T));
    if (e == cudaSuccess) n = std::max<size_t>(want, 1);
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
  }
};

} // namespace

struct coord_ctx {
  coord_params p{};
  std::string switch_def;
  SwitchParams sw{};
  // a CUSTOM switch's compiled expression, and its device copy
  ExprProgram expr{};
  DevBuf<ExprProgram> d_expr;
  SwitchF32 s32{};
  int mode = MODE_SINGLE;
  int64_t nA = 0, nB = 0, ns = 0;
  std::vector<int64_t> abs_host;  // GROUPA then GROUPB absolute indices
  bool has_dup = false;           // an absolute index in two slots
  int host_direct = -1;           // kernels access pageable host arrays in place (-1: not probed)
  int host_path = -1;             // how the last host-array call moved its arrays (coord_host_path)
  bool groups_set = false;
  // the CV's pairing (COORD_CV_*); the sibling CVs' constants and per-atom
  // data by absolute index, copied per slot to the device when needed
  int cv = COORD_CV_COORDINATION;
  double dh_k = 0.0, dh_const = 0.0, dh_eps = 1.0;
  double gh_dmax_sq = 0.0, gh_d0 = 0.0, gh_c_dmax2 = 0.0, gh_A = 0.0, gh_B = 0.0, gh_C = 0.0, gh_D = 0.0;
  std::vector<double> charges_abs, eta_host;
  std::vector<int32_t> types_abs;
  int n_types = 0;
  bool sib_dirty = true;
  bool peratom_used = false;  // the per-atom calls have run (FP64: accw64 is kept)
  DevBuf<double> d_charge, d_eta;
  DevBuf<int> d_ptype;
  std::string err;
  cudaStream_t stream = nullptr;
  // host-array calls over several frames with page-locked arrays: the copy
  // streams (H2D, D2H) and the events of the chunked pipeline
  // (launch_evaluation_chunked)
  cudaStream_t stream2 = nullptr, stream3 = nullptr;
  cudaEvent_t ev_split[9] = {};
  int nsm = 0;
  // neighbour-list state
  bool firsttime = true;
  int built_frames = 0;
  // near/far rows of the current lists (k_nl_partition): the skin they were
  // split with, and the boxes of the rebuild (the fixed-point frame the
  // displacements are measured in)
  bool skin_valid = false;
  double skin = 0.0;
  std::vector<double> skin_boxes;
  HostBuf<unsigned> h_disp2;
  // the D_MAX band of the last frames uploaded when they have generic boxes
  // on the mixed path (tric_band_of), else 0
  double tric_band = 0.0;
  int cap = 0, self_cap = 64, ncell_cap = 0, max_blocks = 0;
  int nframes_alloc = 0;
  // device buffers
  DevBuf<int64_t> abs_of_slot;
  DevBuf<FrameConst> fc;
  DevBuf<int4> qhi;
  DevBuf<int> cell_of_slot, cell_count, cell_start, cell_fill, slot_of_rank, rank_of_slot, scatter_tmp, row_len, slice_w,
      cell_of_rank;
  DevBuf<double4> x64;
  DevBuf<uint4> q;
  DevBuf<uint32_t> ell, self_pairs;
  DevBuf<unsigned long long> nl_count, mm;
  DevBuf<unsigned char> pair_flag;
  DevBuf<double> acc64, partials, accw64;
  DevBuf<float4> acc32;
  DevBuf<unsigned> tickets, band_tickets, disp2;
  DevBuf<int> row_near, slice_wn;
  DevBuf<uint4> q_build;
  DevBuf<uint32_t> ell_far;
  DevBuf<unsigned char> band_flag;
  DevBuf<double> band_rec;
  DevBuf<uint4> band_q;
  DevBuf<unsigned> band_qn;
  DevBuf<double> band_qrec;
  // host-API staging
  DevBuf<double> d_pos, d_s, d_deriv, d_virial, d_dparam, d_bvir, d_bpar;
  // saved forward (COORD_FLAG_SAVE)
  // saved forward: the derivative accumulators stay in place (acc_kept), the
  // virial and parameter derivatives are copied aside
  DevBuf<double> sv_vir, sv_par;
  bool saved_valid = false, saved_param = false, acc_kept = false;
  int saved_frames = 0;
  HostBuf<double> h_pos, h_out;
  HostBuf<FrameConst> h_fc;
  HostBuf<unsigned long long> h_nl;
  std::vector<FrameConst> fc_uploaded;
  std::vector<double> boxes_seen;
  // tuning
  int tile64 = 64, tile32 = 128, ap_blocks = 0, nl_blocks = 0, nl_unroll = 4;
  // mixed NL pass, tuned per evaluation mode (EVAL_S / EVAL_DERIV / EVAL_PARAM)
  int nlm_blocks[5] = {0, 0, 0, 0, 0}, nlm_unroll[5] = {4, 4, 4, 4, 4};
  bool nlm_tuned[5] = {false, false, false, false, false};
  int cells_launch = 0;  // cells per frame known on the host (0: use ncell_cap)
  bool tuned = false;
  // timing: one event pair per pair-kernel launch while enabled
  bool timing = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
  size_t ev_used = 0;

  int fail(int code, const std::string &m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char *where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return COORD_ERR_CUDA;
  }
};

namespace {

bool box_is_zero(const double *b) {
  for (int i = 0; i < 9; i++)
    if (b[i] != 0.0) return false;
  return true;
}

int nl_kind_of(const coord_ctx *c) { return c->p.nlist; }

// Per-frame constants from the box (host part; no-pbc frames are finished on
// the device by k_bounds_finish).
int frame_setup(coord_ctx *c, const double *box, FrameConst *fc, bool *need_bounds) {
  std::memset(fc, 0, sizeof *fc);
  pbc_setup(box, &fc->pbc);
  const bool do_pbc = !c->p.nopbc;
  const bool usepbc = do_pbc && fc->pbc.type != PBC_UNSET;
  const int kind = nl_kind_of(c);
  const double cut = c->p.nl_cutoff;
  GridParams &g = fc->grid;
  g.nc[0] = g.nc[1] = g.nc[2] = 1;
  g.ncells = 1;
  for (int k = 0; k < 3; k++) g.inv_width[k] = 1.0;
  *need_bounds = false;
  if (kind == COORD_NL_CLASSIC) {
    if (usepbc && fc->pbc.type == PBC_ORTHO) {
      g.wrap = 1;
      for (int k = 0; k < 3; k++) {
        int n = (int)std::floor(fc->pbc.box[4 * k] / (cut * (1.0 + 1e-9)));
        if (n < 3) n = 1;
        g.nc[k] = std::min(n, 1024);
      }
      // bound the grid (cells may be larger than the cutoff, never smaller)
      const long long maxcells = std::max<long long>(8 * std::max<int64_t>(c->ns, 1), 1 << 16);
      while ((long long)g.nc[0] * g.nc[1] * g.nc[2] > maxcells) {
        const int k = (g.nc[0] >= g.nc[1] && g.nc[0] >= g.nc[2]) ? 0 : (g.nc[1] >= g.nc[2] ? 1 : 2);
        g.nc[k] = std::max(1, g.nc[k] / 2);
      }
    } else if (usepbc) {
      g.wrap = 0;  // generic box: one cell, every candidate tested exactly
    } else {
      *need_bounds = true;
    }
  } else if (kind == COORD_NL_CELLS) {
    if (box_is_zero(box)) {
      *need_bounds = true;
    } else {
      // LinkCells::createCells (LinkCells.cpp:99-122): reciprocal = invBox^T
      for (int k = 0; k < 3; k++) {
        const double *ib = fc->pbc.invbox;
        const double m = std::sqrt(ib[0 * 3 + k] * ib[0 * 3 + k] + ib[1 * 3 + k] * ib[1 * 3 + k] +
                                   ib[2 * 3 + k] * ib[2 * 3 + k]);
        int n = (int)std::floor(1.0 / m / cut);
        if (n == 0) n = 1;
        g.nc[k] = n;
      }
    }
  }
  g.ncells = g.nc[0] * g.nc[1] * g.nc[2];
  fc->cut2 = cut * cut;
  struct FinishFixed {  // the one-FMA constants once inv_l and grid.lo are final
    FrameConst *fc;
    ~FinishFixed() { fixed_frame_finish(*fc); }
  } finish_fixed{fc};
  // fixed-point frame
  if (usepbc && fc->pbc.type == PBC_ORTHO) {
    fc->fixed_ok = 1;
    const double minl = std::min(fc->pbc.box[0], std::min(fc->pbc.box[4], fc->pbc.box[8]));
    fc->shift_ok = (c->sw.dmax_2 < 1e300 && std::sqrt(c->sw.dmax_2) * 1.001 < 0.45 * minl) ? 1 : 0;
    double span = 0;
    for (int k = 0; k < 3; k++) {
      fc->inv_l[k] = fc->pbc.invbox[4 * k];
      fc->scale[k] = (float)(fc->pbc.box[4 * k] / 4294967296.0);
      span = std::max(span, fc->pbc.box[4 * k]);
    }
    const double band = 1e-4 * fc->cut2 + 8.0 * cut * span / 4294967296.0 + 1e-12;
    fc->cut2_lo = (float)(fc->cut2 - band);
    fc->cut2_hi = (float)(fc->cut2 + band);
  } else if (!usepbc) {
    fc->fixed_ok = 1;
    *need_bounds = *need_bounds || (c->p.precision == COORD_PREC_MIXED) || kind == COORD_NL_CLASSIC;
    fc->cut2_lo = -1.0f;  // finished on the device (span known there)
    fc->cut2_hi = -1.0f;
  } else {
    fc->fixed_ok = 0;  // generic box: the exact search, no fixed-point prefilter
    if (c->p.precision == COORD_PREC_MIXED) {
      fc->tric = 1;
      for (int k = 0; k < 9; k++) {
        fc->fx_m[k] = fc->pbc.invreduced[k] * 4294967296.0;
        fc->red32[k] = (float)(fc->pbc.reduced[k] / 4294967296.0);
      }
    }
  }
  return COORD_OK;
}

// Relative half-width of the band around d_max^2 inside which the FP32 r^2
// of a generic-box frame cannot decide the reference's test (Geo32<true>).
// With s = d invReduced and A_i = sum_j |s_j| |R_ji| <= kappa |d|
// (kappa = max_i sum_j |R_ji| |column j of invReduced|): the wrapped
// integer differences as floats and the three FMAs per component are each
// within 2^-24 of A_i, and one fixed-point unit of either position adds
// 2^-32 sum_j |R_ji|; r^2 = |d|^2 then errs by at most
// (10 sqrt(3) kappa + 3) 2^-24 r^2 plus twice the unit term over d_max.
// Doubled, and never below the orthorhombic band (2e-6).
double tric_band_of(const PbcParams &pbc, double dmax) {
  double kappa = 0.0, unit = 0.0;
  for (int i = 0; i < 3; i++) {
    double ki = 0.0, ui = 0.0;
    for (int j = 0; j < 3; j++) {
      const double cj = std::sqrt(pbc.invreduced[0 * 3 + j] * pbc.invreduced[0 * 3 + j] +
                                  pbc.invreduced[1 * 3 + j] * pbc.invreduced[1 * 3 + j] +
                                  pbc.invreduced[2 * 3 + j] * pbc.invreduced[2 * 3 + j]);
      ki += std::fabs(pbc.reduced[j * 3 + i]) * cj;
      ui += std::fabs(pbc.reduced[j * 3 + i]);
    }
    kappa = std::max(kappa, ki);
    unit = std::max(unit, ui);
  }
  const double rel = (10.0 * std::sqrt(3.0) * kappa + 3.0) / 16777216.0 +
                     (std::isfinite(dmax) && dmax > 0 ? 2.0 * std::sqrt(3.0) * unit / 4294967296.0 / dmax : 0.0);
  return std::max(2e-6, 2.0 * rel);
}

int ensure_buffers(coord_ctx *c, int n_frames) {
  cudaError_t e;
  const size_t F = (size_t)n_frames, ns = (size_t)std::max<int64_t>(c->ns, 1);
  const int nslices = (int)((c->ns + 31) / 32);
#define ENS(buf, n)                                    \
  if ((e = (buf).ensure(n)) != cudaSuccess) {          \
    return c->cuda_fail(e, "allocation of " #buf);     \
  }
  ENS(c->fc, F);
  ENS(c->slot_of_rank, F * ns);
  ENS(c->rank_of_slot, F * ns);
  ENS(c->cell_of_rank, F * ns);
  ENS(c->cell_of_slot, F * ns);
  ENS(c->scatter_tmp, F * ns);
  ENS(c->row_len, F * ns);
  ENS(c->slice_w, F * std::max(nslices, 1));
  ENS(c->x64, F * ns);
  ENS(c->q, F * ns);
  if (c->p.precision == COORD_PREC_FP64 && c->p.nlist != COORD_NL_NONE) ENS(c->qhi, F * ns);
  ENS(c->acc64, F * ns * 3);
  if (c->p.precision == COORD_PREC_FP64 && c->peratom_used) ENS(c->accw64, F * ns);
  ENS(c->acc32, F * ns);
  ENS(c->nl_count, F * 4);
  ENS(c->mm, F * 6);
  ENS(c->tickets, F);
  ENS(c->band_tickets, F);
  ENS(c->band_flag, F * (size_t)((nslices + 31) & ~31) + 32);
  ENS(c->band_rec, F * std::max(nslices, 1) * kPartials);
  ENS(c->band_q, F * kBandQueueCap);
  ENS(c->band_qn, F + 2);
  ENS(c->band_qrec, F * kBandQueueCap * kPartials);
  ENS(c->cell_count, F * (size_t)c->ncell_cap);
  ENS(c->cell_fill, F * (size_t)c->ncell_cap);
  ENS(c->cell_start, F * ((size_t)c->ncell_cap + 1));
  ENS(c->self_pairs, F * (size_t)c->self_cap * 2);
  ENS(c->pair_flag, F * (size_t)std::max<int64_t>(c->nA, 1));
  ENS(c->partials, F * (size_t)c->max_blocks * kPartials);
  if (c->p.nlist != COORD_NL_NONE && c->mode != MODE_PAIR) {
    ENS(c->ell, F * (size_t)nslices * (size_t)c->cap * 32);
    ENS(c->row_near, F * ns);
    ENS(c->slice_wn, F * std::max(nslices, 1));
    ENS(c->q_build, F * ns);
    ENS(c->disp2, 2 * F);
  }
#undef ENS
  if ((e = c->h_fc.ensure(F)) != cudaSuccess) return c->cuda_fail(e, "pinned allocation");
  if ((e = c->h_nl.ensure(F * 4)) != cudaSuccess) return c->cuda_fail(e, "pinned allocation");
  if ((e = c->h_disp2.ensure(F)) != cudaSuccess) return c->cuda_fail(e, "pinned allocation");
  c->nframes_alloc = std::max(c->nframes_alloc, n_frames);
  return COORD_OK;
}

KArgs make_args(coord_ctx *c, int n_frames, const double *d_pos, unsigned flags, double *s, double *deriv,
                double *virial, double *dparam) {
  KArgs a{};
  a.nframes = n_frames;
  a.disp2_frames = n_frames;
  a.ns = (int)c->ns;
  a.nA = (int)(c->mode == MODE_SINGLE ? c->ns : c->nA);
  a.mode = c->mode;
  a.do_pbc = !c->p.nopbc;
  a.nl_kind = c->p.nlist;
  a.cap = c->cap;
  a.ncell_cap = c->ncell_cap;
  a.self_cap = c->self_cap;
  a.nslices = (int)((c->ns + 31) / 32);
  a.flags = (int)flags;
  a.has_dup = c->has_dup ? 1 : 0;
  a.fc = c->fc.p;
  a.tric_band = (float)c->tric_band;
  a.abs_of_slot = c->abs_of_slot.p;
  a.pos = d_pos;
  a.accw64 = c->accw64.p;
  a.cv = c->cv;
  a.charge = c->d_charge.p;
  a.ptype = c->d_ptype.p;
  a.eta = c->d_eta.p;
  a.n_types = c->n_types;
  a.dh_k = c->dh_k;
  a.dh_const = c->dh_const;
  a.dh_eps = c->dh_eps;
  a.gh_dmax_sq = c->gh_dmax_sq;
  a.gh_d0 = c->gh_d0;
  a.gh_c_dmax2 = c->gh_c_dmax2;
  a.gh_A = c->gh_A;
  a.gh_B = c->gh_B;
  a.gh_C = c->gh_C;
  a.gh_D = c->gh_D;
  a.cell_of_slot = c->cell_of_slot.p;
  a.cell_count = c->cell_count.p;
  a.cell_start = c->cell_start.p;
  a.cell_fill = c->cell_fill.p;
  a.slot_of_rank = c->slot_of_rank.p;
  a.rank_of_slot = c->rank_of_slot.p;
  a.cell_of_rank = c->cell_of_rank.p;
  a.scatter_tmp = c->scatter_tmp.p;
  a.x64 = c->x64.p;
  a.q = c->q.p;
  a.qhi = c->qhi.p;
  a.ell = c->ell.p;
  a.row_len = c->row_len.p;
  a.slice_w = c->slice_w.p;
  // near/far rows: off unless forward_impl turns them on for this call
  a.row_near = nullptr;
  a.slice_wn = c->slice_wn.p;
  a.q_build = c->q_build.p;
  a.disp2 = nullptr;
  a.near_r2 = -1.f;
  a.disp_ok2 = -1.f;
  a.nl_count = c->nl_count.p;
  a.self_pairs = c->self_pairs.p;
  a.pair_flag = c->pair_flag.p;
  a.acc64 = c->acc64.p;
  a.acc32 = c->acc32.p;
  a.partials = c->partials.p;
  a.max_blocks = c->max_blocks;
  a.cells_launch = c->cells_launch > 0 ? c->cells_launch : c->ncell_cap;
  a.tickets = c->tickets.p;
  a.band_flag = c->band_flag.p;
  a.band_rec = c->band_rec.p;
  a.band_tickets = c->band_tickets.p;
  a.band_q = c->band_q.p;
  a.band_qn = c->band_qn.p;
  a.band_qrec = c->band_qrec.p;
  a.band_qcap = kBandQueueCap;
  a.out_s = s;
  a.out_deriv = deriv;
  a.out_virial = virial;
  a.out_dparam = dparam;
  return a;
}

// Initial row capacity of the neighbour list: half the expected neighbours
// plus margin (grown on overflow).
int estimate_cap(coord_ctx *c, const double *box) {
  PbcParams p;
  pbc_setup(box, &p);
  const double cut = c->p.nl_cutoff;
  double vol = 0.0;
  if (!c->p.nopbc && p.type != PBC_UNSET) {
    const double *b = p.box;
    vol = std::fabs(b[0] * b[4] * b[8] + b[1] * b[5] * b[6] + b[2] * b[3] * b[7] - b[0] * b[5] * b[7] -
                    b[1] * b[3] * b[8] - b[2] * b[4] * b[6]);
  }
  double expect;
  if (vol > 0) {
    const double rho = (double)c->ns / vol;
    if (c->p.nlist == COORD_NL_CELLS) {
      int nc[3];
      for (int k = 0; k < 3; k++) {
        const double m = std::sqrt(p.invbox[k] * p.invbox[k] + p.invbox[3 + k] * p.invbox[3 + k] +
                                   p.invbox[6 + k] * p.invbox[6 + k]);
        nc[k] = std::max(1, (int)std::floor(1.0 / m / cut));
      }
      expect = 27.0 * (double)c->ns / ((double)nc[0] * nc[1] * nc[2]);
    } else {
      expect = rho * 4.18879020478639 * cut * cut * cut;
    }
    expect = std::min(expect, (double)c->ns);
    int cap = (int)std::ceil(0.5 * expect * 1.35 + 24);
    return (cap + 7) & ~7;
  }
  return (int)std::min<int64_t>(std::max<int64_t>(c->ns, 1), 64);
}

int set_tuning_defaults(coord_ctx *c) {
  if (c->ap_blocks == 0) c->ap_blocks = std::max(1, c->nsm) * 8;
  if (c->nl_blocks == 0) c->nl_blocks = std::max(1, c->nsm) * 4;  // 4 resident 256-thread blocks per SM
  return 0;
}

int upload_frames(coord_ctx *c, int n_frames, const double *boxes, bool *need_bounds_any) {
  *need_bounds_any = false;
  double tric_band = 0.0;
  struct SetBand {  // on every return: the band of the frames set up so far
    coord_ctx *c;
    double &b;
    ~SetBand() { c->tric_band = b; }
  } set_band{c, tric_band};
  bool changed = (int)c->fc_uploaded.size() != n_frames;
  c->fc_uploaded.resize(n_frames);
  for (int f = 0; f < n_frames; f++) {
    FrameConst fcs;
    bool nb = false;
    frame_setup(c, boxes + 9 * (size_t)f, &fcs, &nb);
    *need_bounds_any = *need_bounds_any || nb;
    if (std::memcmp(&fcs, &c->fc_uploaded[f], sizeof fcs) != 0) changed = true;
    c->fc_uploaded[f] = fcs;
    if (fcs.tric) tric_band = std::max(tric_band, tric_band_of(fcs.pbc, std::sqrt(c->sw.dmax_2)));
    if (fcs.grid.ncells > c->ncell_cap) return COORD_ERR_STATE;  // caller grows ncell_cap
  }
  if (changed || *need_bounds_any) {
    std::memcpy(c->h_fc.p, c->fc_uploaded.data(), sizeof(FrameConst) * n_frames);
    cudaError_t e =
        cudaMemcpyAsync(c->fc.p, c->h_fc.p, sizeof(FrameConst) * n_frames, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "frame upload");
  }
  return COORD_OK;
}

// A saved forward left ds/dx in the accumulators; any other pass needs them
// zero first.
int clear_kept_acc(coord_ctx *c) {
  if (!c->acc_kept) return COORD_OK;
  cudaError_t e = cudaSuccess;
  if (c->acc32.p) e = cudaMemsetAsync(c->acc32.p, 0, c->acc32.n * sizeof(float4), c->stream);
  if (!e && c->acc64.p) e = cudaMemsetAsync(c->acc64.p, 0, c->acc64.n * sizeof(double), c->stream);
  if (e) return c->cuda_fail(e, "clearing saved derivatives");
  c->acc_kept = false;
  c->saved_valid = false;
  return COORD_OK;
}

// Host arrays of a coord_forward call on a device that accesses them in
// place: the positions are turned into the pair kernel's fixed-point,
// rank-ordered copy in one pass over the caller's array, and the derivatives
// go from the accumulators to the caller's array in one pass.
struct HostIO {
  const double *pos;  // caller's positions (slot order)
  double *deriv;      // caller's derivatives (slot order) or nullptr
  bool fused;         // prep/finalize straight from/to the caller's arrays
  bool pinned;        // both arrays are page-locked: copy-engine transfers can overlap the kernels
};

// Host-array call over several frames with page-locked arrays, on the mixed
// neighbour-list path: the frames in up to four chunks, whose transfers run
// on the copy engines beside the kernels of other chunks,
//   stream 2 (H2D):  pos(0) pos(1) pos(2) ...
//   stream 1:              pair(0)+finalize(0) pair(1)+finalize(1) ...
//   stream 3 (D2H):                            deriv(0)            deriv(1) ...
// (the persistent pair kernel fills every SM, so transfers by kernels could
// not overlap it).  Returns false (nothing launched) without the streams.
bool launch_evaluation_chunked(coord_ctx *c, const KArgs &a, int mode, const HostIO *io) {
  if (!c->stream2 && cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess) {
    c->stream2 = nullptr;
    return false;
  }
  if (!c->stream3 && cudaStreamCreateWithFlags(&c->stream3, cudaStreamNonBlocking) != cudaSuccess) {
    c->stream3 = nullptr;
    return false;
  }
  for (cudaEvent_t &ev : c->ev_split)
    if (!ev && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return false;
  const int F = a.nframes, K = std::min(F, 4);
  const size_t per = (size_t)a.ns * 3;
  cudaStream_t s1 = c->stream, s2 = c->stream2, s3 = c->stream3;
  const int m = std::min(std::max(mode, 0), 4);
  const int nb = c->nlm_blocks[m] > 0 ? c->nlm_blocks[m] : c->nl_blocks;
  double *dpos = const_cast<double *>(c->d_pos.p);
  cudaEvent_t *evH = c->ev_split, *evC = c->ev_split + 4;
  cudaEventRecord(evC[0], s1);  // the other streams follow what stream 1 holds so far
  cudaStreamWaitEvent(s2, evC[0], 0);
  cudaStreamWaitEvent(s3, evC[0], 0);
  for (int k = 0; k < K; k++) {
    const int f0 = a.frame0 + F * k / K, f1 = a.frame0 + F * (k + 1) / K;
    cudaMemcpyAsync(dpos + f0 * per, io->pos + f0 * per, (f1 - f0) * per * sizeof(double), cudaMemcpyHostToDevice,
                    s2);
    cudaEventRecord(evH[k], s2);
  }
  for (int k = 0; k < K; k++) {
    const int f0 = a.frame0 + F * k / K, f1 = a.frame0 + F * (k + 1) / K;
    KArgs ak = a;
    ak.frame0 = f0;
    ak.nframes = f1 - f0;
    ak.pos = dpos;
    cudaStreamWaitEvent(s1, evH[k], 0);
    launch_prep_host(ak, dpos, 1, s1);
    launch_eval_nl32(ak, c->sw, c->s32, mode, nb, c->nlm_unroll[m], s1);
    launch_band_fix(ak, c->sw, c->s32, mode, s1);
    if (io->deriv) {
      launch_finalize32(ak, 1, s1);
      cudaEventRecord(evC[k], s1);
      cudaStreamWaitEvent(s3, evC[k], 0);
      cudaMemcpyAsync(io->deriv + f0 * per, ak.out_deriv + f0 * per, (f1 - f0) * per * sizeof(double),
                      cudaMemcpyDeviceToHost, s3);
    }
  }
  cudaEventRecord(c->ev_split[8], s3);
  cudaStreamWaitEvent(s1, c->ev_split[8], 0);  // stream 1 ends after the last copy
  return true;
}

// Whether the FP64 neighbour-list pass may screen its entries with the
// fixed-point FP32 distance (k_eval_nl64q): COORDINATION (its switch is zero
// beyond a finite d_max) on frames with an orthorhombic periodic box, where
// the fixed-point positions exist.
bool fp64_prefilter(const coord_ctx *c) {
  if (c->cv != COORD_CV_COORDINATION || c->p.nopbc || !std::isfinite(c->s32.dmax2_hi) || c->fc_uploaded.empty())
    return false;
  for (const FrameConst &fq : c->fc_uploaded)
    if (fq.pbc.type != PBC_ORTHO || !fq.fixed_ok) return false;
  return true;
}

// Whether a rebuilt list is split into near and far parts (k_nl_partition):
// COORDINATION lists (every switching function is zero beyond a finite d_max
// below the cutoff) in orthorhombic periodic frames, on the paths that keep
// fixed-point positions (mixed, or the screened FP64 pass).
bool skin_eligible(const coord_ctx *c) {
  if (c->p.nlist == COORD_NL_NONE || c->mode == MODE_PAIR || c->cv != COORD_CV_COORDINATION || c->p.nopbc)
    return false;
  if (!(c->sw.dmax_2 < 1e300) || !(std::sqrt(c->sw.dmax_2) < c->p.nl_cutoff) || c->fc_uploaded.empty()) return false;
  for (const FrameConst &fq : c->fc_uploaded)
    if (fq.pbc.type != PBC_ORTHO || !fq.fixed_ok) return false;
  return c->p.precision == COORD_PREC_MIXED || fp64_prefilter(c);
}

// The every-pair kernels' tile: the context's, halved (down to `smallest`)
// while a frame would have fewer tile pairs than two per SM -- a small
// system (1,000 atoms: 136 tile pairs of 64) otherwise leaves most SMs idle.
int fill_tile(const coord_ctx *c, const KArgs &a, int tile, int smallest) {
  const bool tri = a.mode == MODE_SINGLE;
  const long long ni = tri ? a.ns : a.nA, nj = tri ? a.ns : a.ns - a.nA;
  while (tile > smallest) {
    const long long ti = (ni + tile - 1) / tile, tj = (nj + tile - 1) / tile;
    const long long ntp = tri ? ti * (ti + 1) / 2 : ti * tj;
    if (ntp * a.nframes >= 2LL * std::max(c->nsm, 1)) break;
    tile /= 2;
  }
  return tile;
}

// The pair pass and its finalize kernel (derivatives to slot order, scaled
// by a.g when set).
// gathered: the list build of this call already left the positions in rank
// order (k_gather in launch_nl_build).
void launch_evaluation(coord_ctx *c, const KArgs &a, int mode, const HostIO *io = nullptr, bool gathered = false) {
  const bool nl = c->p.nlist != COORD_NL_NONE;
  const bool mixed = c->p.precision == COORD_PREC_MIXED;
  const int rank_order = (nl && c->mode != MODE_PAIR) ? 1 : 0;
  const bool prefilter64 = !mixed && nl && c->mode != MODE_PAIR && fp64_prefilter(c);
  if (io && io->fused && io->pinned && nl && mixed && c->mode != MODE_PAIR && a.nframes >= 2 && !c->timing &&
      (!io->deriv || a.out_deriv) && launch_evaluation_chunked(c, a, mode, io)) {
    c->host_path = COORD_HOST_PATH_CHUNKED;
    return;
  }
  // positions for the pair kernel: fixed-point (mixed) or FP64 in rank order
  if (io && io->fused) {
    launch_prep_host(a, io->pos, rank_order, c->stream);
  } else if (c->mode == MODE_PAIR || !nl) {
    if (mixed) launch_gather(a, 0, 0, 1, c->stream);
  } else if (!gathered) {
    launch_gather(a, 1, mixed ? 0 : 1, (mixed || prefilter64) ? 1 : 0, c->stream);
  }
  // the pair kernel alone, between the timing events
  cudaEvent_t tev1 = nullptr;
  if (c->timing) {
    if (c->ev_used == c->ev_pool.size()) {
      cudaEvent_t x, y;
      cudaEventCreate(&x);
      cudaEventCreate(&y);
      c->ev_pool.push_back({x, y});
    }
    cudaEventRecord(c->ev_pool[c->ev_used].first, c->stream);
    tev1 = c->ev_pool[c->ev_used].second;
    c->ev_used++;
  }
  if (c->mode == MODE_PAIR) {
    if (mixed)
      launch_pairs32(a, c->sw, c->s32, mode, nl ? 1 : 0, c->stream);
    else
      launch_pairs64(a, c->sw, mode, nl ? 1 : 0, c->stream);
  } else if (!nl) {
    if (mixed)
      launch_allpairs32(a, c->sw, c->s32, mode, fill_tile(c, a, c->tile32, 64), c->ap_blocks, c->stream);
    else
      launch_allpairs64(a, c->sw, mode, fill_tile(c, a, c->tile64, 32), c->ap_blocks, c->stream);
  } else {
    if (mixed) {
      const int m = std::min(std::max(mode, 0), 4);
      const int nb = c->nlm_blocks[m] > 0 ? c->nlm_blocks[m] : c->nl_blocks;
      launch_eval_nl32(a, c->sw, c->s32, mode, nb, c->nlm_unroll[m], c->stream);
      if (tev1) cudaEventRecord(tev1, c->stream);
      tev1 = nullptr;
      launch_band_fix(a, c->sw, c->s32, mode, c->stream);
    } else {
      launch_eval_nl64(a, c->sw, mode, prefilter64 ? &c->s32 : nullptr, 2 * std::max(c->nsm, 1), c->stream);
    }
  }
  if (tev1) cudaEventRecord(tev1, c->stream);
  if (io && io->fused && io->deriv) {
    launch_finalize_host32(a, io->deriv, rank_order, c->stream);
    return;
  }
  if (a.keep_acc && !a.out_deriv) return;  // saved forward, no copy of ds/dx wanted
  if (mixed)
    launch_finalize32(a, rank_order, c->stream);
  else
    launch_finalize64(a, rank_order, c->stream);
}

// The project's autotuner for the mixed neighbour-list pass: persistent grids
// of 2 to 32 256-thread blocks per SM, or one slice per warp -- grids larger
// than what is resident run in waves that the hardware dispatches in frame
// order, so only a few frames' positions and accumulators compete for L2 --
// x gathers in flight per lane (unroll 2, 4, 8); each candidate is timed
// once with CUDA events on the context's stream and the fastest kept, per
// mode.  Every candidate run
// is a complete pass (its finalize kernel rewrites the outputs), so the
// results of the call are unaffected.
void autotune_nl(coord_ctx *c, const KArgs &a, int mode) {
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  // blocks per SM: up to 8 all resident at once; 16 and 32 run in waves, so
  // a few frames at a time hold L2; 0: one slice per warp
  const int bps[7] = {2, 4, 6, 8, 16, 32, 0}, unr[3] = {2, 4, 8};
  const int m = std::min(std::max(mode, 0), 4);
  float best = 1e30f;
  int bb = c->nl_blocks, bu = c->nl_unroll;
  const bool timing = c->timing;
  c->timing = false;
  // COORD_AUTOTUNE_LOG=<file>: every candidate's time appended to the file
  const char *log_path = std::getenv("COORD_AUTOTUNE_LOG");
  FILE *log = (log_path && log_path[0]) ? std::fopen(log_path, "a") : nullptr;
  for (int b : bps)
    for (int u : unr) {
      const int slices_blocks = (int)(((c->ns + 31) / 32 + 7) / 8);  // blocks of one frame at one slice per warp
      c->nlm_blocks[m] = b > 0 ? b * std::max(c->nsm, 1) : a.nframes * slices_blocks;
      c->nlm_unroll[m] = u;
      c->max_blocks = std::max(c->max_blocks, std::min(slices_blocks, (c->nlm_blocks[m] + a.nframes - 1) / a.nframes));
      if (ensure_buffers(c, a.nframes)) continue;
      KArgs aa = a;
      aa.partials = c->partials.p;
      aa.max_blocks = c->max_blocks;
      aa.keep_acc = 0;  // every candidate clears its accumulators
      cudaEventRecord(t0, c->stream);
      launch_evaluation(c, aa, mode);
      cudaEventRecord(t1, c->stream);
      cudaEventSynchronize(t1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, t1);
      if (log) std::fprintf(log, "mode=%d blocks=%d unroll=%d frames=%d slots=%lld ms=%.4f\n", mode,
                            c->nlm_blocks[m], u, a.nframes, (long long)c->ns, ms);
      if (ms < best) {
        best = ms;
        bb = c->nlm_blocks[m];
        bu = u;
      }
    }
  if (log) std::fclose(log);
  c->nlm_blocks[m] = bb;
  c->nlm_unroll[m] = bu;
  c->nlm_tuned[m] = true;
  c->nl_blocks = bb;
  c->nl_unroll = bu;
  c->timing = timing;
  c->tuned = true;
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
}

// The sibling CVs' per-slot data on the device (after coord_set_groups or a
// change of the data).  Every slot's atom must be covered by the data.
int sibling_upload(coord_ctx *c) {
  if (c->cv == COORD_CV_COORDINATION || !c->sib_dirty) return COORD_OK;
  const size_t ns = (size_t)std::max<int64_t>(c->ns, 1);
  cudaError_t e = cudaSuccess;
  if (c->cv == COORD_CV_DHENERGY) {
    if (c->charges_abs.empty()) return c->fail(COORD_ERR_STATE, "DHENERGY needs the atoms' charges (coord_set_charges)");
    std::vector<double> q(ns, 0.0);
    for (int64_t k = 0; k < c->ns; k++) {
      const int64_t at = c->abs_host[k];
      if (at < 0 || at >= (int64_t)c->charges_abs.size())
        return c->fail(COORD_ERR_ARG, "the charges cover " + std::to_string(c->charges_abs.size()) +
                                          " atoms, but atom number " + std::to_string(at + 1) + " is requested");
      q[k] = c->charges_abs[at];
    }
    if ((e = c->d_charge.ensure(ns)) != cudaSuccess) return c->cuda_fail(e, "allocation");
    if ((e = cudaMemcpy(c->d_charge.p, q.data(), ns * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
      return c->cuda_fail(e, "charge upload");
  } else {
    if (c->types_abs.empty()) return c->fail(COORD_ERR_STATE, "GHBFIX needs the types table (coord_set_ghbfix)");
    std::vector<int> t(ns, 0);
    for (int64_t k = 0; k < c->ns; k++) {
      const int64_t at = c->abs_host[k];
      // GHBFIX.cpp:180-186
      if (at < 0 || at >= (int64_t)c->types_abs.size())
        return c->fail(COORD_ERR_ARG, "your types table only covers " + std::to_string(c->types_abs.size()) +
                                          " atoms, but you are trying to access atom number " + std::to_string(at + 1));
      t[k] = c->types_abs[at];
    }
    const size_t ne = c->eta_host.size();
    if ((e = c->d_ptype.ensure(ns)) != cudaSuccess || (e = c->d_eta.ensure(ne)) != cudaSuccess)
      return c->cuda_fail(e, "allocation");
    if ((e = cudaMemcpy(c->d_ptype.p, t.data(), ns * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(c->d_eta.p, c->eta_host.data(), ne * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
      return c->cuda_fail(e, "types upload");
  }
  c->sib_dirty = false;
  return COORD_OK;
}

int forward_impl(coord_ctx *c, int n_frames, const double *d_pos, const double *boxes, int64_t step, unsigned flags,
                 double *s, double *deriv, double *virial, double *dparam, cudaStream_t stream,
                 HostIO *hio = nullptr, double *peratom = nullptr) {
  if (!c->groups_set) return c->fail(COORD_ERR_STATE, "coord_set_groups has not been called");
  if (n_frames < 1) return c->fail(COORD_ERR_ARG, "n_frames must be >= 1");
  if (c->cv != COORD_CV_COORDINATION && (flags & COORD_FLAG_DR0))
    return c->fail(COORD_ERR_UNSUPPORTED, "R_0/D_0 derivatives belong to COORDINATION's switching function");
  if (int rc = sibling_upload(c)) return rc;
  if (c->ns == 0) {
    // empty groups: s = 0, no derivatives
    if (s) cudaMemsetAsync(s, 0, sizeof(double) * n_frames, stream);
    if (virial) cudaMemsetAsync(virial, 0, sizeof(double) * 9 * n_frames, stream);
    return COORD_OK;
  }
  cudaStream_t saved = c->stream;
  if (stream) c->stream = stream;
  struct Restore {
    coord_ctx *c;
    cudaStream_t s;
    ~Restore() { c->stream = s; }
  } restore{c, saved};

  const bool nl = c->p.nlist != COORD_NL_NONE;
  const bool mixed = c->p.precision == COORD_PREC_MIXED;
  const int nl_stride = c->p.nl_stride;
  // NeighborList::prepare (NeighborList.cpp:433-456)
  bool rebuild = false;
  if (nl) {
    if (nl_stride == 1 || c->firsttime || (step % nl_stride) == 0 || (flags & COORD_FLAG_REBUILD) ||
        c->built_frames != n_frames)
      rebuild = true;
  }
  // LinkCells::setupCells(pbc) (LinkCells.cpp:75-83): a cell list is built on
  // the given box whenever it is not all zero (NOPBC included), and that box
  // must have a volume above DBL_EPSILON; checked at each rebuild
  if (rebuild && c->p.nlist == COORD_NL_CELLS) {
    for (int f = 0; f < n_frames; f++) {
      const double *b = boxes + 9 * (size_t)f;
      if (box_is_zero(b)) continue;
      const double det = b[0] * (b[4] * b[8] - b[5] * b[7]) - b[1] * (b[3] * b[8] - b[5] * b[6]) +
                         b[2] * (b[3] * b[7] - b[4] * b[6]);
      if (!(det > DBL_EPSILON)) {
        char msg[128];
        std::snprintf(msg, sizeof msg, "Cell lists cannot be built when passing a box with null volume. Volume is %g",
                      det);
        return c->fail(COORD_ERR_BOX, msg);
      }
    }
  }
  // sizes
  if (c->cap == 0 && nl) c->cap = estimate_cap(c, boxes);
  {
    int need_cells = (int)std::max<int64_t>(c->ns, 64), host_cells = 0;
    bool device_cells = false;
    for (int f = 0; f < n_frames; f++) {
      FrameConst tmp;
      bool nb;
      frame_setup(c, boxes + 9 * (size_t)f, &tmp, &nb);
      need_cells = std::max(need_cells, tmp.grid.ncells);
      host_cells = std::max(host_cells, tmp.grid.ncells);
      device_cells = device_cells || nb;
    }
    if (need_cells > c->ncell_cap) c->ncell_cap = need_cells;
    c->cells_launch = device_cells ? 0 : host_cells;
  }
  set_tuning_defaults(c);
  c->max_blocks = std::max<int>(c->max_blocks, std::max<int>((int)((c->ns + 255) / 256), c->ap_blocks));
  c->max_blocks = std::max<int>(c->max_blocks, c->nl_blocks);
  c->max_blocks = std::max<int>(c->max_blocks, (int)((std::max<int64_t>(c->nA, 1) + 255) / 256));
  int rc = ensure_buffers(c, n_frames);
  if (rc) return rc;
  bool need_bounds = false;
  rc = upload_frames(c, n_frames, boxes, &need_bounds);
  if (rc) return rc;

  const bool save = (flags & COORD_FLAG_SAVE) && !(flags & COORD_FLAG_NO_DERIV);
  c->saved_valid = false;
  if ((rc = clear_kept_acc(c))) return rc;
  if (save) {
    cudaError_t es;
    if ((es = c->sv_vir.ensure((size_t)n_frames * 9)) || (es = c->sv_par.ensure((size_t)n_frames * 2)))
      return c->cuda_fail(es, "allocation of the saved forward");
  }
  if (hio) {
    // fused host transfers on steps that need no device copy of the positions
    // (no rebuild, no bounding frame): mixed pair kernels only
    hio->fused = mixed && !rebuild && !need_bounds && c->mode != MODE_PAIR && !save;
    if (!hio->fused) launch_copy(hio->pos, const_cast<double *>(d_pos), (size_t)n_frames * c->ns * 3, c->stream);
  }
  double *const k_deriv = (flags & COORD_FLAG_NO_DERIV) ? nullptr : deriv;
  double *const k_virial = (flags & COORD_FLAG_NO_DERIV) ? nullptr : (save ? c->sv_vir.p : virial);
  double *const k_dparam = save ? c->sv_par.p : dparam;
  KArgs a = make_args(c, n_frames, d_pos, flags, s, k_deriv, k_virial, k_dparam);
  a.keep_acc = save ? 1 : 0;
  a.out_peratom = peratom;
  // fused host steps leave the device copy stale: the pair kernels' rare
  // exact d_max tests read the caller's array itself
  if (hio && hio->fused) a.pos = hio->pos;
  // near/far rows: the displacements since the last rebuild are measured
  // (by this step's gather) only against a rebuild in the same boxes
  const bool skin_on = nl && skin_eligible(c);
  const bool same_boxes = c->skin_valid && c->skin_boxes.size() == 9 * (size_t)n_frames &&
                          std::memcmp(c->skin_boxes.data(), boxes, 9 * sizeof(double) * n_frames) == 0;
  if (skin_on && same_boxes) {
    a.disp2 = c->disp2.p;
    cudaMemsetAsync(c->disp2.p, 0, sizeof(unsigned) * n_frames, c->stream);
    if (!rebuild) {
      a.row_near = c->row_near.p;
      a.disp_ok2 = (float)(0.25 * c->skin * c->skin * (1.0 - 1e-5));
    }
  }
  cudaError_t e;
  if (rebuild) cudaMemsetAsync(c->nl_count.p, 0, sizeof(unsigned long long) * 4 * n_frames, c->stream);
  if (need_bounds && (mixed || rebuild)) {
    // min/max sentinels: lo = all ones, hi = 0
    std::vector<unsigned long long> init(6 * (size_t)n_frames);
    for (int f = 0; f < n_frames; f++)
      for (int k = 0; k < 6; k++) init[6 * f + k] = k < 3 ? ~0ull : 0ull;
    if ((e = cudaMemcpyAsync(c->mm.p, init.data(), sizeof(unsigned long long) * init.size(), cudaMemcpyHostToDevice,
                             c->stream)) != cudaSuccess)
      return c->cuda_fail(e, "bounds init");
    launch_bounds(a, c->mm.p, nl ? c->p.nl_cutoff : 1.0, c->p.nlist == COORD_NL_CELLS && rebuild ? 1 : 0, c->stream);
    // the band of the FP32 prefilter depends on the frame span: finish it here
  }

  if (rebuild) {
    if (c->mode == MODE_PAIR) {
      cudaMemsetAsync(c->nl_count.p, 0, sizeof(unsigned long long) * 4 * n_frames, c->stream);
      launch_pair_flags(a, c->stream);
    } else {
      bool classic = c->p.nlist == COORD_NL_CLASSIC;
      for (const FrameConst &fq : c->fc_uploaded) classic = classic && fq.fixed_ok;
      for (int attempt = 0; attempt < 8; attempt++) {
        if (attempt > 0)
          cudaMemsetAsync(c->nl_count.p, 0, sizeof(unsigned long long) * 4 * n_frames, c->stream);
        launch_nl_build(a, classic, c->stream);
        if ((e = cudaMemcpyAsync(c->h_nl.p, c->nl_count.p, sizeof(unsigned long long) * 4 * n_frames,
                                 cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess)
          return c->cuda_fail(e, "neighbour-list count");
        // the largest displacement of the interval that this rebuild ends
        if (a.disp2 && (e = cudaMemcpyAsync(c->h_disp2.p, a.disp2 + n_frames, sizeof(unsigned) * n_frames,
                                            cudaMemcpyDeviceToHost, c->stream)) != cudaSuccess)
          return c->cuda_fail(e, "displacement read-back");
        if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return c->cuda_fail(e, "neighbour-list build");
        unsigned long long need = 0, selfn = 0;
        for (int f = 0; f < n_frames; f++) {
          need = std::max(need, c->h_nl.p[4 * f + 2]);
          selfn = std::max(selfn, c->h_nl.p[4 * f + 1]);
          if (c->h_nl.p[4 * f + 3])
            return c->fail(COORD_ERR_UNSUPPORTED, "NLISTCELLS without a box: the bounding box needs more link "
                                                  "cells than this context allocated");
        }
        bool again = false;
        if (need > (unsigned long long)c->cap) {
          c->cap = (int)((need * 5 / 4 + 8) & ~7ull);
          again = true;
        }
        if (selfn > (unsigned long long)c->self_cap) {
          c->self_cap = (int)(selfn + 64);
          again = true;
        }
        if (!again) break;
        if ((rc = ensure_buffers(c, n_frames))) return rc;
        a = make_args(c, n_frames, d_pos, flags, s, k_deriv, k_virial, k_dparam);
        a.keep_acc = save ? 1 : 0;
        a.out_peratom = peratom;
        if (attempt == 7) return c->fail(COORD_ERR_NOMEM, "neighbour list did not fit after 8 attempts");
      }
    }
    c->firsttime = false;
    c->built_frames = n_frames;
    if (skin_on) {
      // the skin of the new lists: half the gap between d_max and the cutoff
      // after a rebuild in new boxes, otherwise 2.5 x the largest
      // displacement of the interval just ended (the maximum over its steps'
      // gathers), at least a quarter and at most all of the gap; only the
      // time taken depends on it, never the results
      const double dmax = std::sqrt(c->sw.dmax_2), gap = c->p.nl_cutoff - dmax;
      double skin = 0.5 * gap;
      if (a.disp2) {
        float dmax2 = 0.f;
        for (int f = 0; f < n_frames; f++) {
          float v;
          std::memcpy(&v, &c->h_disp2.p[f], sizeof v);
          dmax2 = std::max(dmax2, v);
        }
        skin = std::min(gap, std::max(0.25 * gap, 2.5 * std::sqrt((double)dmax2)));
      }
      if ((e = c->ell_far.ensure((size_t)n_frames * a.nslices * (size_t)c->cap * 32)) != cudaSuccess)
        return c->cuda_fail(e, "allocation of the partition's scratch");
      a.ell_far = c->ell_far.p;
      a.row_near = c->row_near.p;
      a.disp2 = c->disp2.p;
      a.near_r2 = (float)((dmax + skin) * (dmax + skin) * (1.0 + 1e-5));
      launch_nl_partition(a, c->stream);
      a.disp_ok2 = (float)(0.25 * skin * skin * (1.0 - 1e-5));
      c->skin = skin;
      c->skin_valid = true;
      c->skin_boxes.assign(boxes, boxes + 9 * (size_t)n_frames);
    } else {
      c->skin_valid = false;
    }
  }

  const int mode = peratom ? EVAL_PERATOM
                           : ((flags & COORD_FLAG_NO_DERIV) ? EVAL_S : ((flags & COORD_FLAG_DR0) ? EVAL_PARAM : EVAL_DERIV));
  if (mode == EVAL_PARAM && !c->sw.grad_ok)
    return c->fail(COORD_ERR_UNSUPPORTED, "R_0/D_0 gradients are not defined for CUBIC and Q switching functions");
  if (!c->nlm_tuned[std::min(std::max(mode, 0), 4)] && mixed && nl && c->mode != MODE_PAIR) {
    autotune_nl(c, a, mode);
    a.partials = c->partials.p;
    a.max_blocks = c->max_blocks;
  }
  // a rebuild of this call has just gathered the positions into rank order
  launch_evaluation(c, a, mode, hio, rebuild && c->mode != MODE_PAIR && !(hio && hio->fused));
  if (hio && !hio->fused && hio->deriv && k_deriv)
    launch_copy(k_deriv, hio->deriv, (size_t)n_frames * c->ns * 3, c->stream);
  if (save) {
    // ds/dx stays in the accumulators until the backward; the caller gets
    // its copies of the virial and parameter derivatives
    c->acc_kept = true;
    if (virial) cudaMemcpyAsync(virial, c->sv_vir.p, (size_t)n_frames * 9 * sizeof(double), cudaMemcpyDefault,
                                c->stream);
    c->saved_param = (flags & COORD_FLAG_DR0) != 0;
    if (dparam && c->saved_param)
      cudaMemcpyAsync(dparam, c->sv_par.p, (size_t)n_frames * 2 * sizeof(double), cudaMemcpyDefault, c->stream);
    c->saved_valid = true;
    c->saved_frames = n_frames;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return c->cuda_fail(e, "kernel launch");
  return COORD_OK;
}

} // namespace

namespace coordgpu {
int ctx_noalloc_view(const coord_ctx *c, const SwitchParams **sw, const coord_params **p) {
  if (!c || c->cv != COORD_CV_COORDINATION) return COORD_ERR_ARG;
  *sw = &c->sw;
  *p = &c->p;
  return COORD_OK;
}
void ctx_set_error(coord_ctx *c, const char *msg) {
  if (c) c->err = msg;
}
int ctx_multi_view(coord_ctx *c, MultiView *v) {
  if (!c || !v) return COORD_ERR_ARG;
  if (!c->groups_set) return COORD_ERR_STATE;
  v->p = &c->p;
  v->sw = &c->sw;
  v->s32 = &c->s32;
  v->mode = c->mode;
  v->nA = c->nA;
  v->ns = c->ns;
  v->abs = c->abs_host.data();
  return COORD_OK;
}
} // namespace coordgpu

namespace {

int device_init(coord_ctx *c) {
  if (c->stream) {
    cudaSetDevice(c->p.device);
    return COORD_OK;
  }
  cudaError_t e = cudaSetDevice(c->p.device);
  if (e != cudaSuccess) return c->cuda_fail(e, "cudaSetDevice");
  cudaDeviceProp prop;
  if ((e = cudaGetDeviceProperties(&prop, c->p.device)) != cudaSuccess) return c->cuda_fail(e, "device properties");
  c->nsm = prop.multiProcessorCount;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return c->cuda_fail(e, "stream");
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  if (c->sw.type == SW_CUSTOM) {
    if ((e = c->d_expr.ensure(1)) != cudaSuccess) return c->cuda_fail(e, "allocation of the expression");
    if ((e = cudaMemcpy(c->d_expr.p, &c->expr, sizeof c->expr, cudaMemcpyHostToDevice)) != cudaSuccess)
      return c->cuda_fail(e, "expression upload");
    c->sw.expr_dev = c->d_expr.p;
  }
  return COORD_OK;
}

} // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

void coord_params_default(coord_params *p) {
  std::memset(p, 0, sizeof *p);
  p->nn = 6;
  p->mm = 0;
  p->d0 = 0.0;
  p->precision = COORD_PREC_FP64;
}

const char *coord_status_string(int status) {
  switch (status) {
  case COORD_OK: return "ok";
  case COORD_ERR_ARG: return "invalid argument";
  case COORD_ERR_CUDA: return "CUDA error";
  case COORD_ERR_BOX: return "invalid box";
  case COORD_ERR_UNSUPPORTED: return "unsupported input";
  case COORD_ERR_NOMEM: return "out of device memory";
  case COORD_ERR_TIMEOUT: return "device wait timed out";
  case COORD_ERR_STATE: return "call out of order";
  default: return "unknown status";
  }
}

const char *coord_last_error(const coord_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int coord_create(const coord_params *p, coord_ctx **out) {
  if (!p || !out) return COORD_ERR_ARG;
  *out = nullptr;
  coord_ctx *c = new coord_ctx();
  c->p = *p;
  auto bad = [&](int code, const std::string &m) {
    // keep the context so the caller can read the message, as Action::error would report it
    c->err = m;
    *out = c;
    return code;
  };
  // CoordinationBase::CoordinationBase (CoordinationBase.cpp:66-84)
  if (p->nlist != COORD_NL_NONE && p->nlist != COORD_NL_CLASSIC && p->nlist != COORD_NL_CELLS)
    return bad(COORD_ERR_ARG, "unknown neighbour-list kind");
  if (p->nlist == COORD_NL_CELLS && p->pair)
    return bad(COORD_ERR_ARG, "Pair is not compatible with the CELLS implementation of the NL");
  if (p->nlist != COORD_NL_NONE) {
    if (p->nl_cutoff <= 0.0) return bad(COORD_ERR_ARG, "NL_CUTOFF should be explicitly specified and positive");
    if (p->nl_stride <= 0) return bad(COORD_ERR_ARG, "NL_STRIDE should be explicitly specified and positive");
  }
  if (p->precision != COORD_PREC_FP64 && p->precision != COORD_PREC_MIXED)
    return bad(COORD_ERR_ARG, "unknown precision");
  // Coordination::Coordination (Coordination.cpp:128-157)
  if (p->switch_def && p->switch_def[0]) {
    c->switch_def = p->switch_def;
    char err[512];
    err[0] = 0;
    const int rc = switch_from_string(p->switch_def, &c->sw, err, sizeof err, &c->expr);
    if (rc == 2) return bad(COORD_ERR_UNSUPPORTED, std::string("problem reading SWITCH keyword : ") + err);
    if (rc) return bad(COORD_ERR_ARG, std::string("problem reading SWITCH keyword : ") + err);
  } else {
    if (p->r0 <= 0.0) return bad(COORD_ERR_ARG, "R_0 should be explicitly specified and positive");
    switch_from_rational(p->nn, p->mm, p->r0, p->d0, &c->sw);
  }
  c->p.switch_def = nullptr;
  // FP32 parameters of the mixed path
  {
    const SwitchParams &s = c->sw;
    c->s32.dmax2 = (s.dmax_2 >= 3.0e38) ? INFINITY : (float)s.dmax_2;
    // FP32 r^2 from fixed-point deltas is within ~4e-7 relative of the FP64
    // value (conversion, scale and three roundings) plus quantisation; 2e-6
    // leaves a margin of five
    c->s32.dmax2_lo = (s.dmax_2 >= 3.0e38) ? INFINITY : (float)(s.dmax_2 * (1.0 - 2e-6));
    c->s32.dmax2_hi = (s.dmax_2 >= 3.0e38) ? INFINITY : (float)(s.dmax_2 * (1.0 + 2e-6));
    c->s32.dmax_2 = s.dmax_2;
    c->s32.invr0_2 = (float)s.invr0_2;
    c->s32.stretch = (float)s.stretch;
    c->s32.shift = (float)s.shift;
    const int nh = s.type == SW_RATFIX ? s.nn / 2 : 0;
    c->s32.c = (float)(-(double)nh * 2.0 * s.invr0_2 * s.stretch);
    c->s32.d0 = (float)s.d0;
    c->s32.invr0 = (float)s.invr0;
    c->s32.c_r0 = (float)s.c_r0;
    c->s32.c_d0 = (float)s.c_d0;
  }
  // CUDA is initialised on first use (coord_set_groups), so keyword checks and
  // switch set-up work on machines without a GPU.
  *out = c;
  return COORD_OK;
}

int coord_destroy(coord_ctx *c) {
  if (!c) return COORD_OK;
  if (c->stream) {
    cudaSetDevice(c->p.device);
    cudaStreamSynchronize(c->stream);
  }
  c->abs_of_slot.release();
  c->fc.release();
  c->cell_of_slot.release();
  c->cell_count.release();
  c->cell_start.release();
  c->cell_fill.release();
  c->slot_of_rank.release();
  c->rank_of_slot.release();
  c->cell_of_rank.release();
  c->scatter_tmp.release();
  c->row_len.release();
  c->slice_w.release();
  c->x64.release();
  c->q.release();
  c->qhi.release();
  c->row_near.release();
  c->slice_wn.release();
  c->q_build.release();
  c->disp2.release();
  c->ell_far.release();
  c->ell.release();
  c->self_pairs.release();
  c->nl_count.release();
  c->mm.release();
  c->pair_flag.release();
  c->acc64.release();
  c->accw64.release();
  c->partials.release();
  c->acc32.release();
  c->tickets.release();
  c->band_tickets.release();
  c->band_flag.release();
  c->band_rec.release();
  c->band_q.release();
  c->band_qn.release();
  c->band_qrec.release();
  c->d_pos.release();
  c->d_expr.release();
  c->d_s.release();
  c->d_deriv.release();
  c->d_virial.release();
  c->d_dparam.release();
  c->d_bvir.release();
  c->d_bpar.release();
  c->sv_vir.release();
  c->sv_par.release();
  c->d_charge.release();
  c->d_eta.release();
  c->d_ptype.release();
  c->h_pos.release();
  c->h_out.release();
  c->h_fc.release();
  c->h_nl.release();
  c->h_disp2.release();
  for (auto &pr : c->ev_pool) {
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  if (c->stream3) cudaStreamDestroy(c->stream3);
  for (cudaEvent_t &ev : c->ev_split)
    if (ev) cudaEventDestroy(ev);
  delete c;
  return COORD_OK;
}

int coord_set_groups(coord_ctx *c, const int64_t *a, int64_t na, const int64_t *b, int64_t nb) {
  if (!c) return COORD_ERR_ARG;
  if (na < 0 || nb < 0 || (na > 0 && !a) || (nb > 0 && !b)) return c->fail(COORD_ERR_ARG, "bad group arrays");
  if (na + nb > (int64_t)kRankMask) return c->fail(COORD_ERR_UNSUPPORTED, "more than 2^31-1 slots");
  if (c->p.pair) {
    if (na != nb)
      return c->fail(COORD_ERR_ARG, "when using PAIR option, the two groups should have the same number of elements");
    c->mode = MODE_PAIR;
  } else {
    c->mode = nb > 0 ? MODE_TWO : MODE_SINGLE;
  }
  c->nA = na;
  c->nB = nb;
  c->ns = na + nb;
  std::vector<int64_t> abs(std::max<int64_t>(c->ns, 1));
  for (int64_t i = 0; i < na; i++) abs[i] = a[i];
  for (int64_t i = 0; i < nb; i++) abs[na + i] = b[i];
  c->abs_host.assign(abs.begin(), abs.begin() + c->ns);
  {
    std::vector<int64_t> sorted(c->abs_host);
    std::sort(sorted.begin(), sorted.end());
    c->has_dup = std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end();
  }
  if (int rc = device_init(c)) return rc;
  cudaError_t e = c->abs_of_slot.ensure(abs.size());
  if (e != cudaSuccess) return c->cuda_fail(e, "allocation");
  if ((e = cudaMemcpy(c->abs_of_slot.p, abs.data(), sizeof(int64_t) * abs.size(), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return c->cuda_fail(e, "group upload");
  c->groups_set = true;
  c->sib_dirty = true;
  c->firsttime = true;
  c->skin_valid = false;
  c->cap = 0;
  c->fc_uploaded.clear();
  return COORD_OK;
}

int coord_set_dhenergy(coord_ctx *c, double ionic_strength, double temp, double epsilon, double unit_energy,
                       double unit_length, double unit_charge) {
  if (!c) return COORD_ERR_ARG;
  if (c->p.precision != COORD_PREC_FP64) return c->fail(COORD_ERR_UNSUPPORTED, "DHENERGY: FP64 precision only");
  if (!(unit_energy > 0.0) || !(unit_length > 0.0) || !(unit_charge > 0.0))
    return c->fail(COORD_ERR_ARG, "DHENERGY cannot be used for calculations performed with natural units");
  // DHEnergy::DHEnergy (DHEnergy.cpp:112-113), same operation order
  c->dh_const = 138.935458111 / unit_energy / unit_length * unit_charge * unit_charge;
  c->dh_k = std::sqrt(ionic_strength / (epsilon * temp)) * 502.903741125 * unit_length;
  c->dh_eps = epsilon;
  c->cv = COORD_CV_DHENERGY;
  c->sib_dirty = true;
  return COORD_OK;
}

int coord_set_charges(coord_ctx *c, const double *charges, int64_t n_atoms) {
  if (!c) return COORD_ERR_ARG;
  if (n_atoms < 1 || !charges) return c->fail(COORD_ERR_ARG, "empty charge array");
  c->charges_abs.assign(charges, charges + n_atoms);
  c->sib_dirty = true;
  return COORD_OK;
}

int coord_set_ghbfix(coord_ctx *c, double d0, double dmax, double cc, const int32_t *types, int64_t n_atoms,
                     const double *eta, int n_types) {
  if (!c) return COORD_ERR_ARG;
  if (c->p.precision != COORD_PREC_FP64) return c->fail(COORD_ERR_UNSUPPORTED, "GHBFIX: FP64 precision only");
  if (n_atoms < 1 || !types || n_types < 1 || !eta) return c->fail(COORD_ERR_ARG, "empty GHBFIX tables");
  for (int64_t k = 0; k < n_atoms; k++)
    if (types[k] < 0 || types[k] >= n_types) return c->fail(COORD_ERR_ARG, "type id outside the eta table");
  // GHBFIX::GHBFIX (GHBFIX.cpp:111-126), same operation order
  const double dmax2 = dmax - d0;
  c->gh_dmax_sq = dmax * dmax;
  c->gh_d0 = d0;
  c->gh_c_dmax2 = cc * dmax2;
  c->gh_A = (-cc * dmax2 * dmax2) / ((1 - cc) * dmax2 * dmax2);
  c->gh_B = (2 * dmax2) / ((1 - cc) * dmax2 * dmax2);
  c->gh_C = -1 / ((1 - cc) * dmax2 * dmax2);
  c->gh_D = 1 / (cc * dmax2 * dmax2);
  c->types_abs.assign(types, types + n_atoms);
  c->eta_host.assign(eta, eta + (size_t)n_types * n_types);
  c->n_types = n_types;
  c->cv = COORD_CV_GHBFIX;
  c->sib_dirty = true;
  return COORD_OK;
}

int coord_switch_eval(const coord_ctx *c, int n, const double *x, int squared, double *f, double *df) {
  if (!c || n < 0 || (n > 0 && (!x || !f || !df))) return COORD_ERR_ARG;
  for (int i = 0; i < n; i++)
    f[i] = squared ? switch_host_calculate_sqr(c->sw, x[i], df + i) : switch_host_calculate(c->sw, x[i], df + i);
  return COORD_OK;
}

int coord_switch_params(const coord_ctx *c, double out[7]) {
  if (!c || !out) return COORD_ERR_ARG;
  const SwitchParams &s = c->sw;
  const double v[7] = {s.d0, s.dmax, s.dmax_2, s.invr0, s.invr0_2, s.stretch, s.shift};
  std::memcpy(out, v, sizeof v);
  return COORD_OK;
}

int coord_get_nslots(const coord_ctx *c, int64_t *nslots) {
  if (!c || !nslots) return COORD_ERR_ARG;
  *nslots = c->ns;
  return COORD_OK;
}

// With no stream given, the work runs on the context's stream but is ordered
// after everything issued so far on the legacy default stream and before
// anything issued there afterwards (events on both sides), as if it had been
// issued on that stream.
struct DefaultStreamFence {
  coord_ctx *c;
  bool on;
  DefaultStreamFence(coord_ctx *cc, void *stream) : c(cc), on(stream == nullptr && cc->stream != nullptr) {
    if (on) {
      cudaEventRecord(c->ev0, cudaStreamLegacy);
      cudaStreamWaitEvent(c->stream, c->ev0, 0);
    }
  }
  ~DefaultStreamFence() {
    if (on) {
      cudaEventRecord(c->ev1, c->stream);
      cudaStreamWaitEvent(cudaStreamLegacy, c->ev1, 0);
    }
  }
};

int coord_forward_device(coord_ctx *c, int n_frames, const double *pos, const double *boxes, int64_t step,
                         unsigned flags, double *s, double *deriv, double *virial, double *dparam, void *stream) {
  if (!c) return COORD_ERR_ARG;
  if (!boxes || (!pos && c->ns > 0)) return c->fail(COORD_ERR_ARG, "null positions or boxes");
  cudaSetDevice(c->p.device);
  DefaultStreamFence fence(c, stream);
  return forward_impl(c, n_frames, pos, boxes, step, flags, s, deriv, virial, dparam, (cudaStream_t)stream);
}

// The per-atom calls work on a COORDINATION context with a neighbour list
// (NLIST or NLISTCELLS; PAIR has no matrix rows).
static int peratom_check(coord_ctx *c) {
  if (!c->groups_set) return c->fail(COORD_ERR_STATE, "coord_set_groups has not been called");
  if (c->cv != COORD_CV_COORDINATION)
    return c->fail(COORD_ERR_UNSUPPORTED, "per-atom coordination needs a COORDINATION context");
  if (c->p.nlist == COORD_NL_NONE || c->mode == MODE_PAIR)
    return c->fail(COORD_ERR_UNSUPPORTED, "per-atom coordination needs NLIST or NLISTCELLS and no PAIR");
  c->peratom_used = true;
  return COORD_OK;
}

int coord_peratom_device(coord_ctx *c, int n_frames, const double *pos, const double *boxes, int64_t step,
                         unsigned flags, double *cn, double *s, void *stream) {
  if (!c) return COORD_ERR_ARG;
  if (!boxes || !cn || (!pos && c->ns > 0)) return c->fail(COORD_ERR_ARG, "null positions, boxes or cn");
  if (flags & ~COORD_FLAG_REBUILD) return c->fail(COORD_ERR_ARG, "per-atom forward: COORD_FLAG_REBUILD only");
  if (int rc = peratom_check(c)) return rc;
  cudaSetDevice(c->p.device);
  DefaultStreamFence fence(c, stream);
  if (c->ns == 0) return COORD_OK;
  cudaError_t e;
  if (!s) {
    if ((e = c->d_s.ensure((size_t)std::max(n_frames, 1))) != cudaSuccess) return c->cuda_fail(e, "allocation");
    s = c->d_s.p;
  }
  return forward_impl(c, n_frames, pos, boxes, step, flags, s, nullptr, nullptr, nullptr, (cudaStream_t)stream,
                      nullptr, cn);
}

int coord_peratom_backward_device(coord_ctx *c, int n_frames, const double *pos, const double *boxes,
                                  const double *g, double *grad_pos, double *grad_box, void *stream) {
  if (!c) return COORD_ERR_ARG;
  if (!boxes || !g || (!pos && c->ns > 0)) return c->fail(COORD_ERR_ARG, "null positions, boxes or g");
  if (n_frames < 1) return c->fail(COORD_ERR_ARG, "n_frames must be >= 1");
  if (int rc = peratom_check(c)) return rc;
  if (c->built_frames != n_frames)
    return c->fail(COORD_ERR_STATE, "backward needs the neighbour lists of a forward call with the same frames");
  cudaSetDevice(c->p.device);
  if (c->ns == 0) {
    if (grad_box) cudaMemsetAsync(grad_box, 0, sizeof(double) * 9 * n_frames, stream ? (cudaStream_t)stream : c->stream);
    return COORD_OK;
  }
  DefaultStreamFence fence(c, stream);
  cudaStream_t saved = c->stream;
  if (stream) c->stream = (cudaStream_t)stream;
  struct Restore {
    coord_ctx *c;
    cudaStream_t s;
    ~Restore() { c->stream = s; }
  } restore{c, saved};
  cudaError_t e;
  if ((e = c->d_bvir.ensure((size_t)9 * n_frames)) != cudaSuccess) return c->cuda_fail(e, "allocation");
  if (int rc = clear_kept_acc(c)) return rc;
  c->saved_valid = false;
  bool need_bounds = false;
  if (int rc = upload_frames(c, n_frames, boxes, &need_bounds)) return rc;
  KArgs a = make_args(c, n_frames, pos, 0, nullptr, grad_pos, c->d_bvir.p, nullptr);
  a.gslot = g;  // dV/dcn per slot: the gather puts it beside each position
  if (need_bounds && c->p.precision == COORD_PREC_MIXED) {
    std::vector<unsigned long long> init(6 * (size_t)n_frames);
    for (int f = 0; f < n_frames; f++)
      for (int k = 0; k < 6; k++) init[6 * f + k] = k < 3 ? ~0ull : 0ull;
    if ((e = cudaMemcpyAsync(c->mm.p, init.data(), sizeof(unsigned long long) * init.size(), cudaMemcpyHostToDevice,
                             c->stream)))
      return c->cuda_fail(e, "bounds init");
    launch_bounds(a, c->mm.p, c->p.nl_cutoff, 0, c->stream);
  }
  if (!c->nlm_tuned[EVAL_VJP] && c->p.precision == COORD_PREC_MIXED) {
    autotune_nl(c, a, EVAL_VJP);
    a.partials = c->partials.p;
    a.max_blocks = c->max_blocks;
  }
  launch_evaluation(c, a, EVAL_VJP);
  if (grad_box) launch_grad_post(a, c->d_bvir.p, nullptr, grad_box, nullptr, c->stream);
  if ((e = cudaGetLastError()) != cudaSuccess) return c->cuda_fail(e, "per-atom backward launch");
  return COORD_OK;
}

int coord_forward(coord_ctx *c, const double *pos, const double box[9], int64_t step, unsigned flags, double *s,
                  double *deriv, double *virial) {
  if (!c) return COORD_ERR_ARG;
  if (!box || !s || (!pos && c->ns > 0)) return c->fail(COORD_ERR_ARG, "null positions, box or s");
  if (!(flags & COORD_FLAG_NO_DERIV) && !deriv && c->ns > 0) return c->fail(COORD_ERR_ARG, "null deriv");
  cudaSetDevice(c->p.device);
  const size_t n3 = (size_t)c->ns * 3;
  const bool want_d = !(flags & COORD_FLAG_NO_DERIV);
  cudaError_t e;
  if (c->ns == 0) {
    *s = 0.0;
    if (want_d && virial) std::memset(virial, 0, 9 * sizeof(double));
    return COORD_OK;
  }
  if (c->host_direct < 0) {
    int pageable = 0, tables = 0;
    coord_host_memory_access(c->p.device, &pageable, &tables);
    const char *staged = std::getenv("COORD_HOST_STAGED");  // "1": always stage through pinned buffers
    c->host_direct = (pageable && tables && !(staged && staged[0] == '1')) ? 1 : 0;
  }
  if (c->host_direct && !(flags & COORD_FLAG_SAVE)) {
    // The device reads and writes the caller's pageable arrays through the
    // host page tables (cache-coherent CPU-GPU link).  Streaming copies move
    // the arrays (coalesced, whole lines across the link); the derivatives
    // are scattered to slot order in HBM first, never across the link.  s and
    // the virial are written by the pair pass straight into the caller's
    // variables.
    if ((e = c->d_pos.ensure(n3)) || (e = c->d_deriv.ensure(n3))) return c->cuda_fail(e, "staging allocation");
    HostIO hio{pos, want_d ? deriv : nullptr, false, false};
    c->host_path = COORD_HOST_PATH_DIRECT;
    int rc = forward_impl(c, 1, c->d_pos.p, box, step, flags, s, want_d ? c->d_deriv.p : nullptr,
                          want_d ? virial : nullptr, nullptr, nullptr, &hio);
    if (rc) return rc;
    if ((e = cudaStreamSynchronize(c->stream))) return c->cuda_fail(e, "forward");
    return COORD_OK;
  }
  if ((e = c->d_pos.ensure(n3)) || (e = c->d_deriv.ensure(n3)) || (e = c->d_s.ensure(1)) ||
      (e = c->d_virial.ensure(9)) || (e = c->h_pos.ensure(n3)) || (e = c->h_out.ensure(n3 + 10)))
    return c->cuda_fail(e, "staging allocation");
  c->host_path = COORD_HOST_PATH_STAGED;
  if (n3) {
    std::memcpy(c->h_pos.p, pos, n3 * sizeof(double));
    if ((e = cudaMemcpyAsync(c->d_pos.p, c->h_pos.p, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream)))
      return c->cuda_fail(e, "H2D positions");
  }
  int rc = forward_impl(c, 1, c->d_pos.p, box, step, flags, c->d_s.p, c->d_deriv.p, c->d_virial.p, nullptr, nullptr);
  if (rc) return rc;
  cudaMemcpyAsync(c->h_out.p, c->d_s.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (want_d) {
    cudaMemcpyAsync(c->h_out.p + 1, c->d_virial.p, 9 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (n3) cudaMemcpyAsync(c->h_out.p + 10, c->d_deriv.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  }
  if ((e = cudaStreamSynchronize(c->stream))) return c->cuda_fail(e, "forward");
  *s = c->h_out.p[0];
  if (want_d) {
    if (virial) std::memcpy(virial, c->h_out.p + 1, 9 * sizeof(double));
    if (n3) std::memcpy(deriv, c->h_out.p + 10, n3 * sizeof(double));
  }
  return COORD_OK;
}

int coord_forward_batch(coord_ctx *c, int n_frames, const double *pos, const double *boxes, int64_t step,
                        unsigned flags, double *s, double *deriv, double *virial) {
  if (!c) return COORD_ERR_ARG;
  if (n_frames < 1) return c->fail(COORD_ERR_ARG, "n_frames must be >= 1");
  if (n_frames == 1) return coord_forward(c, pos, boxes, step, flags, s, deriv, virial);
  if (!boxes || !s || (!pos && c->ns > 0)) return c->fail(COORD_ERR_ARG, "null positions, boxes or s");
  const bool want_d = !(flags & COORD_FLAG_NO_DERIV);
  if (want_d && !deriv && c->ns > 0) return c->fail(COORD_ERR_ARG, "null deriv");
  if (flags & COORD_FLAG_SAVE) return c->fail(COORD_ERR_ARG, "COORD_FLAG_SAVE needs the device call");
  cudaSetDevice(c->p.device);
  const size_t n3 = (size_t)c->ns * 3 * n_frames;
  cudaError_t e;
  if (c->ns == 0) {
    for (int f = 0; f < n_frames; f++) s[f] = 0.0;
    if (want_d && virial) std::memset(virial, 0, 9 * sizeof(double) * n_frames);
    return COORD_OK;
  }
  if (c->host_direct < 0) {
    int pageable = 0, tables = 0;
    coord_host_memory_access(c->p.device, &pageable, &tables);
    const char *staged = std::getenv("COORD_HOST_STAGED");
    c->host_direct = (pageable && tables && !(staged && staged[0] == '1')) ? 1 : 0;
  }
  if ((e = c->d_pos.ensure(n3)) || (e = c->d_deriv.ensure(n3))) return c->cuda_fail(e, "staging allocation");
  if (c->host_direct) {
    // as coord_forward: the kernels read and write the caller's arrays in
    // place; page-locked arrays move on the copy engines, chunk by chunk
    auto locked = [](const void *p) {
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      return at.type == cudaMemoryTypeHost;
    };
    HostIO hio{pos, want_d ? deriv : nullptr, false, locked(pos) && (!want_d || locked(deriv))};
    c->host_path = COORD_HOST_PATH_DIRECT;  // COORD_HOST_PATH_CHUNKED when the chunked pass runs
    int rc = forward_impl(c, n_frames, c->d_pos.p, boxes, step, flags, s, want_d ? c->d_deriv.p : nullptr,
                          want_d ? virial : nullptr, nullptr, nullptr, &hio);
    if (rc) return rc;
    if ((e = cudaStreamSynchronize(c->stream))) return c->cuda_fail(e, "forward");
    return COORD_OK;
  }
  const size_t nf = (size_t)n_frames;
  if ((e = c->d_s.ensure(nf)) || (e = c->d_virial.ensure(9 * nf)) || (e = c->h_pos.ensure(n3)) ||
      (e = c->h_out.ensure(n3 + 10 * nf)))
    return c->cuda_fail(e, "staging allocation");
  c->host_path = COORD_HOST_PATH_STAGED;
  std::memcpy(c->h_pos.p, pos, n3 * sizeof(double));
  if ((e = cudaMemcpyAsync(c->d_pos.p, c->h_pos.p, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream)))
    return c->cuda_fail(e, "H2D positions");
  int rc = forward_impl(c, n_frames, c->d_pos.p, boxes, step, flags, c->d_s.p, want_d ? c->d_deriv.p : nullptr,
                        want_d ? c->d_virial.p : nullptr, nullptr, nullptr);
  if (rc) return rc;
  double *hs = c->h_out.p, *hv = hs + nf, *hd = hv + 9 * nf;
  cudaMemcpyAsync(hs, c->d_s.p, nf * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (want_d) {
    cudaMemcpyAsync(hv, c->d_virial.p, 9 * nf * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(hd, c->d_deriv.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  }
  if ((e = cudaStreamSynchronize(c->stream))) return c->cuda_fail(e, "forward");
  std::memcpy(s, hs, nf * sizeof(double));
  if (want_d) {
    if (virial) std::memcpy(virial, hv, 9 * nf * sizeof(double));
    std::memcpy(deriv, hd, n3 * sizeof(double));
  }
  return COORD_OK;
}

int coord_backward_device(coord_ctx *c, int n_frames, const double *pos, const double *boxes, const double *g,
                          double *grad_pos, double *grad_box, double *grad_param, void *stream) {
  if (!c) return COORD_ERR_ARG;
  if (!c->groups_set) return c->fail(COORD_ERR_STATE, "coord_set_groups has not been called");
  if (!boxes || !g || (!pos && c->ns > 0)) return c->fail(COORD_ERR_ARG, "null positions, boxes or g");
  if (n_frames < 1) return c->fail(COORD_ERR_ARG, "n_frames must be >= 1");
  if (grad_param && !c->sw.grad_ok)
    return c->fail(COORD_ERR_UNSUPPORTED, "R_0/D_0 gradients are not defined for CUBIC and Q switching functions");
  if (grad_param && c->cv != COORD_CV_COORDINATION)
    return c->fail(COORD_ERR_UNSUPPORTED, "R_0/D_0 derivatives belong to COORDINATION's switching function");
  if (int rc = sibling_upload(c)) return rc;
  cudaSetDevice(c->p.device);
  if (c->ns == 0) {
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    if (grad_box) cudaMemsetAsync(grad_box, 0, sizeof(double) * 9 * n_frames, st);
    if (grad_param) cudaMemsetAsync(grad_param, 0, sizeof(double) * 2 * n_frames, st);
    return COORD_OK;
  }
  const bool nl = c->p.nlist != COORD_NL_NONE;
  if (nl && c->built_frames != n_frames)
    return c->fail(COORD_ERR_STATE, "backward needs the neighbour lists of a forward call with the same frames");
  DefaultStreamFence fence(c, stream);
  cudaStream_t saved = c->stream;
  if (stream) c->stream = (cudaStream_t)stream;
  struct Restore {
    coord_ctx *c;
    cudaStream_t s;
    ~Restore() { c->stream = s; }
  } restore{c, saved};
  cudaError_t e;
  if ((e = c->d_bvir.ensure((size_t)9 * n_frames)) || (e = c->d_bpar.ensure((size_t)2 * n_frames)))
    return c->cuda_fail(e, "allocation");
  if (c->saved_valid && c->saved_frames == n_frames && (!grad_param || c->saved_param)) {
    // the forward kept ds/dx, the virial and ds/d(R_0, D_0): scale them
    KArgs a = make_args(c, n_frames, pos, 0, nullptr, grad_pos, nullptr, nullptr);
    a.g = g;
    // g * ds/dx from the kept accumulators, which are cleared on the way
    const bool nl_order = c->p.nlist != COORD_NL_NONE && c->mode != MODE_PAIR;
    if (c->p.precision == COORD_PREC_MIXED)
      launch_finalize32(a, nl_order ? 1 : 0, c->stream);
    else
      launch_finalize64(a, nl_order ? 1 : 0, c->stream);
    c->acc_kept = false;
    c->saved_valid = false;
    if (grad_box || grad_param) launch_grad_post(a, c->sv_vir.p, c->sv_par.p, grad_box, grad_param, c->stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return c->cuda_fail(e, "backward launch");
    return COORD_OK;
  }
  int rc = clear_kept_acc(c);
  if (rc) return rc;
  bool need_bounds = false;
  rc = upload_frames(c, n_frames, boxes, &need_bounds);
  if (rc) return rc;
  KArgs a = make_args(c, n_frames, pos, COORD_FLAG_DR0, nullptr, grad_pos, c->d_bvir.p, c->d_bpar.p);
  a.g = g;
  if (need_bounds && c->p.precision == COORD_PREC_MIXED) {
    std::vector<unsigned long long> init(6 * (size_t)n_frames);
    for (int f = 0; f < n_frames; f++)
      for (int k = 0; k < 6; k++) init[6 * f + k] = k < 3 ? ~0ull : 0ull;
    if ((e = cudaMemcpyAsync(c->mm.p, init.data(), sizeof(unsigned long long) * init.size(), cudaMemcpyHostToDevice,
                             c->stream)))
      return c->cuda_fail(e, "bounds init");
    launch_bounds(a, c->mm.p, nl ? c->p.nl_cutoff : 1.0, 0, c->stream);
  }
  launch_evaluation(c, a, c->sw.grad_ok ? EVAL_PARAM : EVAL_DERIV);
  if (grad_box || grad_param) launch_grad_post(a, c->d_bvir.p, c->d_bpar.p, grad_box, grad_param, c->stream);
  if ((e = cudaGetLastError()) != cudaSuccess) return c->cuda_fail(e, "backward launch");
  return COORD_OK;
}

int coord_nl_size(coord_ctx *c, int frame, int64_t *n) {
  if (!c || !n) return COORD_ERR_ARG;
  if (c->p.nlist == COORD_NL_NONE) {
    const int64_t ns = c->ns;
    *n = c->mode == MODE_SINGLE ? ns * (ns - 1) / 2 : (c->mode == MODE_TWO ? c->nA * c->nB : c->nA);
    return COORD_OK;
  }
  if (frame < 0 || frame >= c->built_frames) return c->fail(COORD_ERR_STATE, "no neighbour list for that frame");
  unsigned long long h[4];
  cudaSetDevice(c->p.device);
  cudaError_t e = cudaMemcpyAsync(h, c->nl_count.p + 4 * (size_t)frame, sizeof h, cudaMemcpyDeviceToHost, c->stream);
  if (!e) e = cudaStreamSynchronize(c->stream);
  if (e) return c->cuda_fail(e, "nl size");
  *n = (int64_t)(h[0] + h[1]);
  return COORD_OK;
}

int coord_nl_near_size(coord_ctx *c, int frame, int64_t *n, double *skin) {
  if (!c || !n) return COORD_ERR_ARG;
  if (c->p.nlist == COORD_NL_NONE || c->mode == MODE_PAIR)
    return c->fail(COORD_ERR_STATE, "no sliced neighbour list in this context");
  if (frame < 0 || frame >= c->built_frames) return c->fail(COORD_ERR_STATE, "no neighbour list for that frame");
  cudaSetDevice(c->p.device);
  std::vector<int> len((size_t)c->ns);
  const int *src = (c->skin_valid ? c->row_near.p : c->row_len.p) + (size_t)frame * c->ns;
  cudaError_t e = cudaMemcpyAsync(len.data(), src, sizeof(int) * len.size(), cudaMemcpyDeviceToHost, c->stream);
  if (!e) e = cudaStreamSynchronize(c->stream);
  if (e) return c->cuda_fail(e, "near size");
  int64_t t = 0;
  for (int v : len) t += v;
  *n = t;
  if (skin) *skin = c->skin_valid ? c->skin : 0.0;
  return COORD_OK;
}

int coord_get_pairs(coord_ctx *c, int frame, uint32_t *pairs, int64_t cap, int64_t *n) {
  if (!c || !n) return COORD_ERR_ARG;
  if (c->p.nlist == COORD_NL_NONE) return c->fail(COORD_ERR_STATE, "no neighbour list (NLIST not active)");
  if (frame < 0 || frame >= c->built_frames) return c->fail(COORD_ERR_STATE, "no neighbour list for that frame");
  cudaSetDevice(c->p.device);
  cudaStreamSynchronize(c->stream);
  std::vector<std::pair<uint32_t, uint32_t>> out;
  const size_t ns = (size_t)c->ns, fo = (size_t)frame * ns;
  if (c->mode == MODE_PAIR) {
    std::vector<unsigned char> fl(c->nA);
    cudaMemcpy(fl.data(), c->pair_flag.p + (size_t)frame * c->nA, c->nA, cudaMemcpyDeviceToHost);
    for (int64_t i = 0; i < c->nA; i++)
      if (fl[i]) out.push_back({(uint32_t)i, (uint32_t)(i + c->nA)});
  } else {
    const int nslices = (int)((ns + 31) / 32);
    std::vector<int> slot(ns), len(ns);
    std::vector<uint32_t> ell((size_t)nslices * c->cap * 32);
    unsigned long long cnt[4];
    cudaMemcpy(slot.data(), c->slot_of_rank.p + fo, ns * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(len.data(), c->row_len.p + fo, ns * sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(ell.data(), c->ell.p + (size_t)frame * nslices * c->cap * 32, ell.size() * sizeof(uint32_t),
               cudaMemcpyDeviceToHost);
    cudaMemcpy(cnt, c->nl_count.p + 4 * (size_t)frame, sizeof cnt, cudaMemcpyDeviceToHost);
    for (size_t r = 0; r < ns; r++)
      for (int k = 0; k < len[r]; k++) {
        const uint32_t e = ell[((r >> 5) * c->cap + k) * 32 + (r & 31)];
        const uint32_t p = e & kRankMask;
        const bool rfirst = (e & kOrientBit) != 0;
        const uint32_t a = (uint32_t)slot[r], b = (uint32_t)slot[p];
        out.push_back(rfirst ? std::make_pair(a, b) : std::make_pair(b, a));
      }
    const size_t nself = std::min<unsigned long long>(cnt[1], (unsigned long long)c->self_cap);
    std::vector<uint32_t> sp(2 * std::max<size_t>(nself, 1));
    if (nself)
      cudaMemcpy(sp.data(), c->self_pairs.p + (size_t)frame * c->self_cap * 2, nself * 2 * sizeof(uint32_t),
                 cudaMemcpyDeviceToHost);
    for (size_t k = 0; k < nself; k++) out.push_back({sp[2 * k], sp[2 * k + 1]});
  }
  cudaError_t e = cudaGetLastError();
  if (e) return c->cuda_fail(e, "get pairs");
  std::sort(out.begin(), out.end());
  *n = (int64_t)out.size();
  for (int64_t i = 0; i < *n && i < cap; i++) {
    pairs[2 * i] = out[i].first;
    pairs[2 * i + 1] = out[i].second;
  }
  return COORD_OK;
}

int coord_autotune(coord_ctx *c, char *desc, size_t desclen) {
  if (!c) return COORD_ERR_ARG;
  if (desc && desclen)
    std::snprintf(desc, desclen,
                  "tuned=%d nl_pass(s/deriv/param)=%d/%d/%d blocks, unroll %d/%d/%d allpairs_tile64=%d "
                  "allpairs_tile32=%d blocks=%d",
                  (int)c->tuned, c->nlm_blocks[0], c->nlm_blocks[1], c->nlm_blocks[2], c->nlm_unroll[0],
                  c->nlm_unroll[1], c->nlm_unroll[2], c->tile64, c->tile32, c->ap_blocks);
  return COORD_OK;
}

int coord_measure_peaks(int device, double *fp32, double *fp64, double *hbm) {
  return measure_peaks(device, fp32, fp64, hbm);
}

int64_t coord_launch_count(void) { return g_launches.load(); }

int coord_last_kernel_ms(coord_ctx *c, double *ms, int *count) {
  if (!c || !ms) return COORD_ERR_ARG;
  *ms = 0.0;
  if (count) *count = 0;
  double tot = 0.0;
  for (size_t i = 0; i < c->ev_used; i++) {
    float t = 0.f;
    cudaEventSynchronize(c->ev_pool[i].second);
    if (cudaEventElapsedTime(&t, c->ev_pool[i].first, c->ev_pool[i].second) == cudaSuccess) tot += t;
  }
  if (c->ev_used) *ms = tot / (double)c->ev_used;
  if (count) *count = (int)c->ev_used;
  c->ev_used = 0;
  return COORD_OK;
}

int coord_apply_forces(coord_ctx *c, int n_frames, const double *ff, int64_t n_atoms, double *atom_forces,
                       double *box_forces, void *stream) {
  if (!c) return COORD_ERR_ARG;
  if (!ff || n_frames < 1 || n_atoms < 0) return c->fail(COORD_ERR_ARG, "null force or bad sizes");
  if (!c->saved_valid || !c->acc_kept || c->saved_frames != n_frames)
    return c->fail(COORD_ERR_STATE, "coord_apply_forces needs a forward with COORD_FLAG_SAVE on the same frames");
  for (int64_t v : c->abs_host)
    if (v >= n_atoms) return c->fail(COORD_ERR_ARG, "an atom index of the groups is beyond n_atoms");
  cudaSetDevice(c->p.device);
  DefaultStreamFence fence(c, stream);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  KArgs a = make_args(c, n_frames, nullptr, 0, nullptr, nullptr, nullptr, nullptr);
  const bool nl_order = c->p.nlist != COORD_NL_NONE && c->mode != MODE_PAIR;
  launch_apply_forces(a, c->p.precision == COORD_PREC_MIXED, nl_order ? 1 : 0, ff, (long long)n_atoms, atom_forces,
                      c->sv_vir.p, box_forces, st);
  c->acc_kept = false;
  c->saved_valid = false;
  cudaError_t e;
  if ((e = cudaGetLastError()) != cudaSuccess) return c->cuda_fail(e, "force application");
  return COORD_OK;
}

int coord_host_path(const coord_ctx *c) { return c ? c->host_path : -1; }

int coord_host_memory_access(int device, int *pageable, int *host_page_tables) {
  int a = 0, b = 0;
  if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) a = 0;
  if (cudaDeviceGetAttribute(&b, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess) b = 0;
  if (pageable) *pageable = a;
  if (host_page_tables) *host_page_tables = b;
  return COORD_OK;
}

int coord_kernel_times(coord_ctx *c, float *ms, int cap, int *count) {
  if (!c || !count) return COORD_ERR_ARG;
  *count = (int)c->ev_used;
  for (size_t i = 0; i < c->ev_used && (int)i < cap; i++) {
    float t = 0.f;
    cudaEventSynchronize(c->ev_pool[i].second);
    cudaEventElapsedTime(&t, c->ev_pool[i].first, c->ev_pool[i].second);
    if (ms) ms[i] = t;
  }
  return COORD_OK;
}

int coord_set_timing(coord_ctx *c, int enable) {
  if (!c) return COORD_ERR_ARG;
  c->timing = enable != 0;
  c->ev_used = 0;
  return COORD_OK;
}

// multi-action batches: implemented in multi.cu
} // extern "C"
