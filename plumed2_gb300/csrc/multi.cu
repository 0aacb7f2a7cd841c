// multi.cu -- many COORDINATION actions over one shared system in one launch.
//
// The batch the reference runs as many separate actions (one
// CoordinationBase::calculate each, CoordinationBase.cpp:142-231): here every
// (frame, action, tile pair) is an item of one persistent kernel.  Actions
// with no NLIST, mixed precision and an orthorhombic box are fused; any other
// action runs through its own context on the same stream, one after another.
//
//   k_multi_prep    FP64 system positions -> 32-bit fixed-point fractions
//                   of the box, once per (frame, atom)
//   k_multi_pairs   items = (frame, action, tile pair); TILE slots of the
//                   action's i-tile against TILE slots of its j-tile, the
//                   j-tile staged in shared memory through the action's
//                   slot -> atom table; one FP64 record (s, virial) per item
//   k_multi_finish  per (frame, action): Neumaier-compensated sum of its
//                   items' records in item order
//   k_multi_finalize FP32 derivative accumulators -> FP64 outputs
//
// Tile size and blocks per SM come from a small autotuner that times each
// candidate once on the first call.  With coord_multi_use_graph(m, 1) and
// every action fused, the whole sequence is captured into a CUDA graph on the
// first call and replayed afterwards (the host writes the frame boxes into a
// pinned buffer the graph's copy node reads).
#include "coordgpu.h"
#include "launch.h"
#include "eval.cuh"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace coordgpu {
namespace {

struct ActionDesc {
  int slot_base;  // first fused slot of the action
  int ns, nA, mode;
  int nTi, nTj, ntp;
  int item_base;  // first item of the action within a frame
  int out_action; // index of the action in the user's order
  SwitchF32 s32;
};

struct MultiArgs {
  int nframes, n_atoms, n_desc, n_items, total_slots, n_out;
  const ActionDesc *desc;
  const int *atom_of_slot;      // [total_slots]
  const uint4 *qsys;            // [frames][n_atoms]
  float4 *acc;                  // [frames][total_slots]
  double *partials;             // [frames][n_items][kPartials]
  const FrameConst *fc;         // [frames]
  const double *pos;            // [frames][n_atoms][3]
  const long long *out_of_slot; // [total_slots] derivative offset (doubles) within a frame
  long long per_frame;          // derivative doubles per frame, all actions
  double *out_s, *out_deriv, *out_virial;
};

__global__ void k_multi_prep(MultiArgs m) {
  const int f = blockIdx.y;
  const int at = blockIdx.x * blockDim.x + threadIdx.x;
  if (at >= m.n_atoms) return;
  const double *x = m.pos + ((size_t)f * m.n_atoms + at) * 3;
  const double xx[3] = {x[0], x[1], x[2]};
  ((uint4 *)m.qsys)[(size_t)f * m.n_atoms + at] = fixed_of(m.fc[f], xx);
}

template <int TILE, int NH>
__global__ void __launch_bounds__(TILE) k_multi_pairs(MultiArgs m, SwitchParams sw_generic) {
  __shared__ uint4 qj[TILE];
  __shared__ float accj[TILE][3];
  __shared__ int atj[TILE];
  __shared__ double red[kPartials][TILE / 32];
  const long long total = (long long)m.nframes * m.n_items;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    const int f = (int)(t / m.n_items);
    const int it = (int)(t - (long long)f * m.n_items);
    // the action owning item it (binary search on item_base)
    int lo = 0, hi = m.n_desc - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (m.desc[mid].item_base <= it)
        lo = mid;
      else
        hi = mid - 1;
    }
    const ActionDesc &D = m.desc[lo];
    const bool tri = D.mode == MODE_SINGLE;
    int I, J;
    tile_pair(it - D.item_base, D.nTi, D.nTj, tri, I, J);
    const int iend = tri ? D.ns : D.nA, jbase0 = tri ? 0 : D.nA, jend = D.ns;
    const int i = I * TILE + threadIdx.x;
    const int jb = jbase0 + J * TILE;
    const FrameConst &fc = m.fc[f];
    const float sx = fc.scale[0], sy = fc.scale[1], sz = fc.scale[2];
    const uint4 *qs = m.qsys + (size_t)f * m.n_atoms;
    float4 *acc4 = m.acc + (size_t)f * m.total_slots + D.slot_base;
    __syncthreads();
    {
      const int j = jb + threadIdx.x;
      if (j < jend) {
        const int at = m.atom_of_slot[D.slot_base + j];
        atj[threadIdx.x] = at;
        qj[threadIdx.x] = qs[at];
      }
      accj[threadIdx.x][0] = accj[threadIdx.x][1] = accj[threadIdx.x][2] = 0.f;
    }
    __syncthreads();
    Acc32 acc;
    const SwitchF32 s32 = D.s32;
    if (i < iend) {
      const int ai = m.atom_of_slot[D.slot_base + i];
      const uint4 qi = qs[ai];
      const bool diag = tri && (I == J);
      float ax = 0.f, ay = 0.f, az = 0.f;
      for (int s = 0; s < TILE; s++) {
        const int jl = (threadIdx.x + s) & (TILE - 1);
        const int j = jb + jl;
        if (j >= jend || (diag && jl <= (int)threadIdx.x) || atj[jl] == ai) continue;
        const uint4 qp = qj[jl];
        const float dx = fixed_delta(qi.x, qp.x, sx), dy = fixed_delta(qi.y, qp.y, sy),
                    dz = fixed_delta(qi.z, qp.z, sz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        bool in = r2 <= s32.dmax2_lo;
        if (!in && r2 <= s32.dmax2_hi)  // band: the reference's FP64 test, slot i first
          in = dmax_exact(m.pos + ((size_t)f * m.n_atoms + ai) * 3, m.pos + ((size_t)f * m.n_atoms + atj[jl]) * 3,
                          &fc.pbc, 1, s32.dmax_2);
        if (in) {
          float sig, df;
          sw32<NH>(sw_generic, s32, fminf(r2, s32.dmax2), sig, df);
          acc.add_s(sig);
          const float ddx = df * dx, ddy = df * dy, ddz = df * dz;
          ax -= ddx;
          ay -= ddy;
          az -= ddz;
          atomicAdd(&accj[jl][0], ddx);
          atomicAdd(&accj[jl][1], ddy);
          atomicAdd(&accj[jl][2], ddz);
          acc.add_vir(ddx, ddy, ddz, dx, dy, dz);
        }
      }
      if (ax != 0.f || ay != 0.f || az != 0.f) red_add_v4(acc4 + i, ax, ay, az);
    }
    __syncthreads();
    {
      const int j = jb + threadIdx.x;
      const float *v = accj[threadIdx.x];
      if (j < jend && (v[0] != 0.f || v[1] != 0.f || v[2] != 0.f)) red_add_v4(acc4 + j, v[0], v[1], v[2]);
    }
    // the item's record
    double part[kPartials];
    acc.to_partials(part);
#pragma unroll
    for (int k = 0; k < kPartials; k++) {
      double w = warp_sum(part[k]);
      if (lane == 0) red[k][warp] = w;
    }
    __syncthreads();
    if (threadIdx.x < kPartials) {
      double sum = 0.0;
      for (int w = 0; w < TILE / 32; w++) sum += red[threadIdx.x][w];
      m.partials[((size_t)f * m.n_items + it) * kPartials + threadIdx.x] = sum;
    }
  }
}

// one warp per (frame, fused action)
__global__ void k_multi_finish(MultiArgs m) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= m.nframes * m.n_desc) return;
  const int f = gw / m.n_desc, k = gw - f * m.n_desc;
  const ActionDesc &D = m.desc[k];
  const double *base = m.partials + ((size_t)f * m.n_items + D.item_base) * kPartials;
  for (int c = 0; c < 10; c++) {
    double s = 0.0, comp = 0.0;
    for (int b = lane; b < D.ntp; b += 32) {
      const double x = base[(size_t)b * kPartials + c];
      const double t = s + x;
      comp += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
      s = t;
    }
    s += comp;
    s = warp_sum(s);  // fixed shuffle tree: deterministic
    if (lane == 0) {
      const size_t o = (size_t)f * m.n_out + D.out_action;
      if (c == 0) {
        m.out_s[o] = s;
      } else if (m.out_virial) {
        m.out_virial[o * 9 + (c - 1)] = s;
      }
    }
  }
}

__global__ void k_multi_finalize(MultiArgs m) {
  const int f = blockIdx.y;
  const int sl = blockIdx.x * blockDim.x + threadIdx.x;
  if (sl >= m.total_slots) return;
  float4 *a = m.acc + (size_t)f * m.total_slots + sl;
  const float4 v = *a;
  if (m.out_deriv) {
    double *o = m.out_deriv + (size_t)f * m.per_frame + m.out_of_slot[sl];
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
  }
  *a = make_float4(0.f, 0.f, 0.f, 0.f);
}

// gather an action's slot positions from the system (the non-fused path)
__global__ void k_multi_gather(const double *pos, int n_atoms, int nframes, const int64_t *atoms, int ns, double *dst) {
  const int f = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns || f >= nframes) return;
  const double *x = pos + ((size_t)f * n_atoms + atoms[s]) * 3;
  double *d = dst + ((size_t)f * ns + s) * 3;
  d[0] = x[0];
  d[1] = x[1];
  d[2] = x[2];
}

// scatter one action's batched results into the interleaved user layout
__global__ void k_multi_scatter(int nframes, int ns, int n_out, int k, long long off, long long per_frame,
                                const double *s_in, const double *d_in, const double *v_in, double *s_out,
                                double *d_out, double *v_out) {
  const int f = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nframes) return;
  if (t < 3 * ns && d_out) d_out[(size_t)f * per_frame + off + t] = d_in[(size_t)f * 3 * ns + t];
  if (t == 0) s_out[(size_t)f * n_out + k] = s_in[f];
  if (t < 9 && v_out) v_out[((size_t)f * n_out + k) * 9 + t] = v_in[(size_t)f * 9 + t];
}

template <typename T> struct Buf {
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

struct Group {  // fused actions sharing one switch specialisation
  int nh = 0;
  std::vector<int> actions;  // user indices
  SwitchParams sw{};         // for the generic evaluator (nh == 0: one launch per action)
  Buf<ActionDesc> desc;
  Buf<int> atom_of_slot;
  Buf<long long> out_of_slot;
  Buf<float4> acc;
  Buf<double> partials;
  int total_slots = 0, n_items = 0, tile_built = 0;
};

} // namespace
} // namespace coordgpu

using namespace coordgpu;

struct coord_multi {
  std::vector<coord_ctx *> ctxs;
  std::vector<MultiView> views;
  int64_t n_atoms = 0;
  std::string err;
  bool graph = false;
  int device = 0, nsm = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr, t0 = nullptr, t1 = nullptr;
  std::vector<long long> deriv_off;  // per action, doubles within a frame
  long long per_frame = 0;
  std::vector<Group> groups;
  std::vector<int> others;  // actions run through their own context
  Buf<FrameConst> fc;
  Buf<uint4> qsys;
  Buf<double> tmp_pos, tmp_s, tmp_d, tmp_v;
  Buf<int64_t> tmp_atoms;
  FrameConst *h_fc = nullptr;
  int h_fc_n = 0;
  int tile = 128, bps = 8;
  bool tuned = false;
  long long calls = 0;
  // graph cache
  cudaGraphExec_t exec = nullptr;
  struct Key {
    int nf;
    const void *pos, *s, *d, *v;
    unsigned flags;
    bool operator==(const Key &o) const {
      return nf == o.nf && pos == o.pos && s == o.s && d == o.d && v == o.v && flags == o.flags;
    }
  } key{};
  int fail(int code, const std::string &m) {
    err = m;
    return code;
  }
};

namespace {

int build_group_tables(coord_multi *m, Group &g, int tile, int n_frames) {
  std::vector<ActionDesc> d;
  std::vector<int> atoms;
  std::vector<long long> outs;
  int items = 0;
  for (int k : g.actions) {
    const MultiView &v = m->views[k];
    ActionDesc a{};
    a.slot_base = (int)atoms.size();
    a.ns = (int)v.ns;
    a.nA = (int)(v.mode == MODE_SINGLE ? v.ns : v.nA);
    a.mode = v.mode;
    const int ni = a.mode == MODE_SINGLE ? a.ns : a.nA, nj = a.mode == MODE_SINGLE ? a.ns : a.ns - a.nA;
    a.nTi = (ni + tile - 1) / tile;
    a.nTj = (nj + tile - 1) / tile;
    a.ntp = a.mode == MODE_SINGLE ? a.nTi * (a.nTi + 1) / 2 : a.nTi * a.nTj;
    a.item_base = items;
    a.out_action = k;
    a.s32 = *v.s32;
    items += a.ntp;
    for (int64_t s = 0; s < v.ns; s++) {
      atoms.push_back((int)v.abs[s]);
      outs.push_back(m->deriv_off[k] + 3 * s);
    }
    d.push_back(a);
  }
  g.total_slots = (int)atoms.size();
  g.n_items = items;
  cudaError_t e;
  if ((e = g.desc.ensure(d.size())) || (e = g.atom_of_slot.ensure(atoms.size())) ||
      (e = g.out_of_slot.ensure(outs.size())) || (e = g.acc.ensure((size_t)n_frames * atoms.size())) ||
      (e = g.partials.ensure((size_t)n_frames * std::max(items, 1) * kPartials)))
    return m->fail(COORD_ERR_CUDA, std::string("batch allocation: ") + cudaGetErrorString(e));
  // pageable copies on the legacy stream: wait for them before any kernel of
  // the batch's non-blocking stream reads the tables
  cudaMemcpy(g.desc.p, d.data(), sizeof(ActionDesc) * d.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(g.atom_of_slot.p, atoms.data(), sizeof(int) * atoms.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(g.out_of_slot.p, outs.data(), sizeof(long long) * outs.size(), cudaMemcpyHostToDevice);
  if ((e = cudaDeviceSynchronize()))
    return m->fail(COORD_ERR_CUDA, std::string("batch tables: ") + cudaGetErrorString(e));
  g.tile_built = tile;
  return COORD_OK;
}

MultiArgs group_args(coord_multi *m, Group &g, int n_frames, const double *pos, double *s, double *deriv,
                     double *virial) {
  MultiArgs a{};
  a.nframes = n_frames;
  a.n_atoms = (int)m->n_atoms;
  a.n_desc = (int)g.actions.size();
  a.n_items = g.n_items;
  a.total_slots = g.total_slots;
  a.n_out = (int)m->ctxs.size();
  a.desc = g.desc.p;
  a.atom_of_slot = g.atom_of_slot.p;
  a.qsys = m->qsys.p;
  a.acc = g.acc.p;
  a.partials = g.partials.p;
  a.fc = m->fc.p;
  a.pos = pos;
  a.out_of_slot = g.out_of_slot.p;
  a.per_frame = m->per_frame;
  a.out_s = s;
  a.out_deriv = deriv;
  a.out_virial = virial;
  return a;
}

void launch_pairs(const MultiArgs &a, const Group &g, int tile, int nblocks, cudaStream_t st) {
  const int nb = (int)std::max(1ll, std::min<long long>((long long)a.nframes * a.n_items, nblocks));
#define PAIRS(T, N) k_multi_pairs<T, N><<<nb, T, 0, st>>>(a, g.sw)
#define BYNH(T)                   \
  switch (g.nh) {                 \
  case 2: PAIRS(T, 2); break;     \
  case 3: PAIRS(T, 3); break;     \
  case 4: PAIRS(T, 4); break;     \
  case 6: PAIRS(T, 6); break;     \
  default: PAIRS(T, 0); break;    \
  }
  if (tile == 64) {
    BYNH(64)
  } else {
    BYNH(128)
  }
#undef BYNH
#undef PAIRS
  g_launches += 1;
}

// Issues the fused sequence (no host synchronisation: capturable).
int issue_fused(coord_multi *m, int n_frames, const double *pos, double *s, double *deriv, double *virial,
                cudaStream_t st) {
  cudaMemcpyAsync(m->fc.p, m->h_fc, sizeof(FrameConst) * n_frames, cudaMemcpyHostToDevice, st);
  {
    MultiArgs a{};
    a.nframes = n_frames;
    a.n_atoms = (int)m->n_atoms;
    a.qsys = m->qsys.p;
    a.fc = m->fc.p;
    a.pos = pos;
    k_multi_prep<<<dim3((unsigned)((m->n_atoms + 255) / 256), n_frames), 256, 0, st>>>(a);
    g_launches += 1;
  }
  for (Group &g : m->groups) {
    MultiArgs a = group_args(m, g, n_frames, pos, s, deriv, virial);
    launch_pairs(a, g, m->tile, m->bps * std::max(m->nsm, 1), st);
    const int warps = n_frames * a.n_desc;
    k_multi_finish<<<(warps * 32 + 255) / 256, 256, 0, st>>>(a);
    k_multi_finalize<<<dim3((a.total_slots + 255) / 256, n_frames), 256, 0, st>>>(a);
    g_launches += 2;
  }
  return COORD_OK;
}

} // namespace

extern "C" {

int coord_multi_create(coord_ctx *const *ctxs, int n_actions, int64_t n_atoms, coord_multi **out) {
  if (!ctxs || n_actions < 1 || !out || n_atoms < 1) return COORD_ERR_ARG;
  *out = nullptr;
  coord_multi *m = new coord_multi();
  *out = m;
  m->ctxs.assign(ctxs, ctxs + n_actions);
  m->n_atoms = n_atoms;
  m->views.resize(n_actions);
  long long off = 0;
  for (int k = 0; k < n_actions; k++) {
    if (!ctxs[k] || ctx_multi_view(ctxs[k], &m->views[k]))
      return m->fail(COORD_ERR_STATE, "every action needs coord_set_groups before joining a batch");
    const MultiView &v = m->views[k];
    for (int64_t s = 0; s < v.ns; s++)
      if (v.abs[s] < 0 || v.abs[s] >= n_atoms) return m->fail(COORD_ERR_ARG, "group index outside the system");
    m->deriv_off.push_back(off);
    off += 3 * v.ns;
    if (k == 0) m->device = v.p->device;
    if (v.p->device != m->device) return m->fail(COORD_ERR_ARG, "all actions of a batch must use one device");
  }
  m->per_frame = off;
  if (m->n_atoms > 0x7fffffff) return m->fail(COORD_ERR_UNSUPPORTED, "more than 2^31-1 atoms");
  // fused groups (mixed, no NLIST, not PAIR, periodic)
  for (int k = 0; k < n_actions; k++) {
    const MultiView &v = m->views[k];
    const bool fuse = v.p->nlist == COORD_NL_NONE && v.p->precision == COORD_PREC_MIXED && v.mode != MODE_PAIR &&
                      !v.p->nopbc && v.ns > 0 && v.sw->type != SW_CUSTOM;
    if (!fuse) {
      m->others.push_back(k);
      continue;
    }
    const int nh = mixed_nh(*v.sw);
    const int nhc = (nh == 2 || nh == 3 || nh == 4 || nh == 6) ? nh : 0;
    Group *g = nullptr;
    for (Group &x : m->groups)
      if (x.nh == nhc && (nhc != 0 || std::memcmp(&x.sw, v.sw, sizeof(SwitchParams)) == 0)) g = &x;
    if (!g) {
      m->groups.emplace_back();
      g = &m->groups.back();
      g->nh = nhc;
      g->sw = *v.sw;
    }
    g->actions.push_back(k);
  }
  cudaError_t e = cudaSetDevice(m->device);
  cudaDeviceProp prop;
  if (!e) e = cudaGetDeviceProperties(&prop, m->device);
  if (!e) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e) return m->fail(COORD_ERR_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e));
  m->nsm = prop.multiProcessorCount;
  cudaEventCreateWithFlags(&m->ev_in, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&m->ev_out, cudaEventDisableTiming);
  cudaEventCreate(&m->t0);
  cudaEventCreate(&m->t1);
  return COORD_OK;
}

int coord_multi_destroy(coord_multi *m) {
  if (!m) return COORD_OK;
  if (m->stream) {
    cudaSetDevice(m->device);
    cudaStreamSynchronize(m->stream);
  }
  if (m->exec) cudaGraphExecDestroy(m->exec);
  for (Group &g : m->groups) {
    g.desc.release();
    g.atom_of_slot.release();
    g.out_of_slot.release();
    g.acc.release();
    g.partials.release();
  }
  m->fc.release();
  m->qsys.release();
  m->tmp_pos.release();
  m->tmp_s.release();
  m->tmp_d.release();
  m->tmp_v.release();
  m->tmp_atoms.release();
  if (m->h_fc) cudaFreeHost(m->h_fc);
  for (cudaEvent_t ev : {m->ev_in, m->ev_out, m->t0, m->t1})
    if (ev) cudaEventDestroy(ev);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return COORD_OK;
}

int coord_multi_deriv_offset(const coord_multi *m, int action, int64_t *offset, int64_t *per_frame) {
  if (!m || action < 0 || action >= (int)m->ctxs.size()) return COORD_ERR_ARG;
  if (offset) *offset = m->deriv_off[action];
  if (per_frame) *per_frame = m->per_frame;
  return COORD_OK;
}

int coord_multi_use_graph(coord_multi *m, int enable) {
  if (!m) return COORD_ERR_ARG;
  m->graph = enable != 0;
  return COORD_OK;
}

const char *coord_multi_last_error(const coord_multi *m) { return m ? m->err.c_str() : "null batch"; }

int coord_multi_forward_device(coord_multi *m, int n_frames, const double *pos, const double *boxes, unsigned flags,
                               double *s, double *deriv, double *virial, void *stream) {
  if (!m) return COORD_ERR_ARG;
  if (n_frames < 1 || !pos || !boxes || !s) return m->fail(COORD_ERR_ARG, "null positions, boxes or s");
  cudaSetDevice(m->device);
  const bool fence = stream == nullptr;
  cudaStream_t st = m->stream;
  if (!fence) st = (cudaStream_t)stream;
  if (fence) {
    cudaEventRecord(m->ev_in, cudaStreamLegacy);
    cudaStreamWaitEvent(st, m->ev_in, 0);
  }
  if (flags & COORD_FLAG_NO_DERIV) {
    deriv = nullptr;
    virial = nullptr;
  }
  cudaError_t e;
  // frame constants (pinned staging, read by the copy node of a captured graph)
  if (n_frames > m->h_fc_n) {
    if (m->h_fc) cudaFreeHost(m->h_fc);
    if ((e = cudaMallocHost(&m->h_fc, sizeof(FrameConst) * n_frames)))
      return m->fail(COORD_ERR_CUDA, "pinned allocation");
    m->h_fc_n = n_frames;
    if (m->exec) {
      cudaGraphExecDestroy(m->exec);
      m->exec = nullptr;
    }
  }
  for (int f = 0; f < n_frames; f++) {
    FrameConst &fc = m->h_fc[f];
    std::memset(&fc, 0, sizeof fc);
    pbc_setup(boxes + 9 * (size_t)f, &fc.pbc);
    if (!m->groups.empty() && fc.pbc.type != PBC_ORTHO)
      return m->fail(COORD_ERR_UNSUPPORTED, "fused batch actions need an orthorhombic box");
    fc.fixed_ok = 1;
    for (int k = 0; k < 3; k++) {
      fc.inv_l[k] = fc.pbc.invbox[4 * k];
      fc.scale[k] = (float)(fc.pbc.box[4 * k] / 4294967296.0);
    }
    fixed_frame_finish(fc);
  }
  if (!m->groups.empty()) {
    if ((e = m->fc.ensure(n_frames)) || (e = m->qsys.ensure((size_t)n_frames * m->n_atoms)))
      return m->fail(COORD_ERR_CUDA, std::string("batch allocation: ") + cudaGetErrorString(e));
    // autotune once: tile size x blocks per SM, each candidate timed once
    if (!m->tuned) {
      const int tiles[2] = {64, 128}, bpss[3] = {4, 8, 16};
      float best = 1e30f;
      int bt = 128, bb = 8;
      for (int ti : tiles)
        for (int bp : bpss) {
          for (Group &g : m->groups)
            if (int rc = build_group_tables(m, g, ti, n_frames)) return rc;
          m->tile = ti;
          m->bps = bp;
          cudaEventRecord(m->t0, st);
          issue_fused(m, n_frames, pos, s, deriv, virial, st);
          cudaEventRecord(m->t1, st);
          cudaEventSynchronize(m->t1);
          float ms = 0.f;
          cudaEventElapsedTime(&ms, m->t0, m->t1);
          if (ms < best) {
            best = ms;
            bt = ti;
            bb = bp;
          }
        }
      m->tile = bt;
      m->bps = bb;
      m->tuned = true;
    }
    for (Group &g : m->groups)
      if (g.tile_built != m->tile || g.acc.n < (size_t)n_frames * g.total_slots ||
          g.partials.n < (size_t)n_frames * std::max(g.n_items, 1) * kPartials)
        if (int rc = build_group_tables(m, g, m->tile, n_frames)) return rc;
    const bool use_graph = m->graph && m->others.empty() && stream != cudaStreamLegacy;
    coord_multi::Key key{n_frames, pos, s, deriv, virial, flags};
    if (use_graph) {
      if (!m->exec || !(key == m->key)) {
        if (m->exec) {
          cudaGraphExecDestroy(m->exec);
          m->exec = nullptr;
        }
        cudaGraph_t gph;
        if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)))
          return m->fail(COORD_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        issue_fused(m, n_frames, pos, s, deriv, virial, st);
        if ((e = cudaStreamEndCapture(st, &gph)))
          return m->fail(COORD_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&m->exec, gph, 0);
        cudaGraphDestroy(gph);
        if (e) return m->fail(COORD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        m->key = key;
      }
      if ((e = cudaGraphLaunch(m->exec, st))) return m->fail(COORD_ERR_CUDA, cudaGetErrorString(e));
    } else {
      issue_fused(m, n_frames, pos, s, deriv, virial, st);
    }
  }
  // the other actions through their own contexts; staging sized once for the
  // largest of them, before anything is queued
  if (!m->others.empty()) {
    size_t ns_max = 1;
    for (int k : m->others) ns_max = std::max(ns_max, (size_t)m->views[k].ns);
    if ((e = m->tmp_pos.ensure((size_t)n_frames * ns_max * 3)) || (e = m->tmp_s.ensure(n_frames)) ||
        (e = m->tmp_d.ensure((size_t)n_frames * ns_max * 3)) || (e = m->tmp_v.ensure((size_t)n_frames * 9)) ||
        (e = m->tmp_atoms.ensure(ns_max)))
      return m->fail(COORD_ERR_CUDA, std::string("batch allocation: ") + cudaGetErrorString(e));
  }
  for (int k : m->others) {
    const MultiView &v = m->views[k];
    const size_t ns = (size_t)v.ns;
    if (ns) {
      cudaMemcpyAsync(m->tmp_atoms.p, v.abs, sizeof(int64_t) * ns, cudaMemcpyHostToDevice, st);
      k_multi_gather<<<dim3((unsigned)((ns + 255) / 256), n_frames), 256, 0, st>>>(pos, (int)m->n_atoms, n_frames,
                                                                                 m->tmp_atoms.p, (int)ns, m->tmp_pos.p);
      g_launches += 1;
    }
    int rc = coord_forward_device(m->ctxs[k], n_frames, m->tmp_pos.p, boxes, m->calls, flags, m->tmp_s.p, m->tmp_d.p,
                                  m->tmp_v.p, nullptr, st);
    if (rc) return m->fail(rc, std::string("action ") + std::to_string(k) + ": " + coord_last_error(m->ctxs[k]));
    k_multi_scatter<<<dim3((unsigned)((3 * ns + 255) / 256 + 1), n_frames), 256, 0, st>>>(
        n_frames, (int)ns, (int)m->ctxs.size(), k, m->deriv_off[k], m->per_frame, m->tmp_s.p, m->tmp_d.p, m->tmp_v.p,
        s, deriv, virial);
    g_launches += 1;
  }
  m->calls++;
  if (fence) {
    cudaEventRecord(m->ev_out, st);
    cudaStreamWaitEvent(cudaStreamLegacy, m->ev_out, 0);
  }
  if ((e = cudaGetLastError())) return m->fail(COORD_ERR_CUDA, cudaGetErrorString(e));
  return COORD_OK;
}

} // extern "C"
