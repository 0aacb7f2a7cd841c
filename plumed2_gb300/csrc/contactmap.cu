// contactmap.cu -- CONTACTMAP (colvar/ContactMap.cpp:149-365) on the GPU.
//
// A contact map is a list of explicit contacts i = (first, second), each with
// its own switching function, reference value and weight.  The reference
// requests the first atoms of all contacts, then the second atoms
// (NeighborList in pair mode, tools/NeighborList.cpp:54-57), so contact i
// owns the slots i and n + i.  Per contact (ContactMap.cpp:291-325):
//   d      = pbc.distance(x[i], x[n + i])
//   c_i    = w_i * (sigma_i(|d|) - ref_i)          SwitchingFunction::calculate
//   tmpder = w_i * dfunc * d,  tmpvir = w_i * dfunc * (d x d)
// components: value_i = c_i, slot derivatives -tmpder / +tmpder, box -tmpvir;
// SUM: the sum of c_i; CMDIST: the sum of c_i^2 with tmpder, tmpvir times 2 c_i.
// One thread per contact and frame.  SUM and CMDIST close with the library's
// deterministic grid reduction.  FP64 throughout, built without FMA
// contraction, in the reference's operation order.
#include "kernels.cuh"
#include "launch.h"

#include <string>
#include <vector>

namespace coordgpu {
namespace {

template <int MODE>
__global__ void __launch_bounds__(128) k_cmap(KArgs a, int n, int nsw, const SwitchParams *__restrict__ sw, const double *__restrict__ ref,
           const double *__restrict__ w, const PbcParams *__restrict__ pbc, int do_pbc, const double *__restrict__ pos,
           double *value, double *deriv, double *vir) {
  const int f = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double part[kPartials];
#pragma unroll
  for (int k = 0; k < kPartials; k++) part[k] = 0.0;
  if (i < n) {
    const size_t fo = (size_t)f * 2 * n;
    const double *p0 = pos + (fo + i) * 3, *p1 = pos + (fo + n + i) * 3;
    const double v1[3] = {p0[0], p0[1], p0[2]}, v2[3] = {p1[0], p1[1], p1[2]};
    double d[3];
    if (do_pbc)
      pbc_distance(pbc[f], v1, v2, d);
    else
      for (int k = 0; k < 3; k++) d[k] = v2[k] - v1[k];
    const VD<double> s = sw_calculate<double>(sw[nsw == 1 ? 0 : i], sqrt(mod2(d)));
    const double coord = w[i] * (s.f - ref[i]);
    const double wdf = w[i] * s.d;
    double tmpder[3], tmpvir[9];
    for (int k = 0; k < 3; k++) tmpder[k] = wdf * d[k];
    for (int x = 0; x < 3; x++)
      for (int y = 0; y < 3; y++) tmpvir[3 * x + y] = wdf * (d[x] * d[y]);
    if (MODE == COORD_CMAP_CMDIST) {
      for (int k = 0; k < 3; k++) tmpder[k] *= 2. * coord;
      for (int k = 0; k < 9; k++) tmpvir[k] *= 2. * coord;
    }
    if (deriv)
      for (int k = 0; k < 3; k++) {
        deriv[(fo + i) * 3 + k] = -tmpder[k];
        deriv[(fo + n + i) * 3 + k] = tmpder[k];
      }
    if (MODE == COORD_CMAP_COMPONENTS) {
      value[(size_t)f * n + i] = coord;
      if (vir)
        for (int k = 0; k < 9; k++) vir[((size_t)f * n + i) * 9 + k] = -tmpvir[k];
    } else {
      part[0] = MODE == COORD_CMAP_CMDIST ? coord * coord : coord;
      for (int k = 0; k < 9; k++) part[1 + k] = -tmpvir[k];
    }
  }
  if (MODE != COORD_CMAP_COMPONENTS) block_partials_finish(a, f, part, gridDim.x);
}

} // namespace
} // namespace coordgpu

using namespace coordgpu;

struct coord_cmap {
  int64_t n = 0;
  int mode = COORD_CMAP_COMPONENTS, nopbc = 0, device = 0;
  std::vector<SwitchParams> sw;
  std::vector<double> ref, w;
  SwitchParams *d_sw = nullptr;
  double *d_ref = nullptr, *d_w = nullptr, *d_partials = nullptr;
  PbcParams *d_pbc = nullptr;
  unsigned *d_tickets = nullptr;
  int frames_cap = 0;
  // host-array calls: device staging of one frame
  double *d_stage = nullptr;  // positions in, then value, derivatives, virials
  std::string err;
  int fail(int code, const std::string &m) {
    err = m;
    return code;
  }
};

static constexpr int kCmapBlock = 128;

static void cmap_free(coord_cmap *m) {
  if (m->d_pbc || m->d_partials || m->d_sw) cudaDeviceSynchronize();
  cudaFree(m->d_sw);
  cudaFree(m->d_ref);
  cudaFree(m->d_w);
  cudaFree(m->d_partials);
  cudaFree(m->d_pbc);
  cudaFree(m->d_tickets);
  cudaFree(m->d_stage);
  m->d_stage = nullptr;
  m->d_sw = nullptr;
  m->d_ref = m->d_w = m->d_partials = nullptr;
  m->d_pbc = nullptr;
  m->d_tickets = nullptr;
}

extern "C" {

int coord_cmap_create(int64_t n_contacts, const char *const *switch_defs, int n_switch_defs, const double *reference,
                      const double *weight, int mode, int nopbc, int device, coord_cmap **out) {
  if (!out) return COORD_ERR_ARG;
  *out = nullptr;
  coord_cmap *m = new coord_cmap();
  *out = m;
  if (n_contacts < 1 || n_contacts > (1 << 28)) return m->fail(COORD_ERR_ARG, "CONTACTMAP needs at least one contact");
  if (mode < COORD_CMAP_COMPONENTS || mode > COORD_CMAP_CMDIST) return m->fail(COORD_ERR_ARG, "unknown CONTACTMAP mode");
  if (!switch_defs || (n_switch_defs != 1 && n_switch_defs != n_contacts))
    return m->fail(COORD_ERR_ARG, "give one SWITCH or one per contact");
  m->n = n_contacts;
  m->mode = mode;
  m->nopbc = nopbc;
  m->device = device;
  // ContactMap::ContactMap (ContactMap.cpp:192-226): the switching functions
  m->sw.resize(n_switch_defs);
  for (int k = 0; k < n_switch_defs; k++) {
    char e[512];
    e[0] = 0;
    const int rc = switch_from_string(switch_defs[k] ? switch_defs[k] : "", &m->sw[k], e, sizeof e);
    const std::string which = n_switch_defs == 1 ? std::string("SWITCH") : "SWITCH" + std::to_string(k + 1);
    if (rc == 2) return m->fail(COORD_ERR_UNSUPPORTED, "problem reading " + which + " keyword : " + e);
    if (rc) return m->fail(COORD_ERR_ARG, "problem reading " + which + " keyword : " + e);
  }
  // references default to 0 and weights to 1 (ContactMap.cpp:228-262)
  m->ref.assign(n_contacts, 0.0);
  m->w.assign(n_contacts, 1.0);
  if (reference) m->ref.assign(reference, reference + n_contacts);
  if (weight) m->w.assign(weight, weight + n_contacts);
  cudaError_t e;
  if ((e = cudaSetDevice(device)) != cudaSuccess ||
      (e = cudaMalloc(&m->d_sw, sizeof(SwitchParams) * m->sw.size())) != cudaSuccess ||
      (e = cudaMalloc(&m->d_ref, sizeof(double) * n_contacts)) != cudaSuccess ||
      (e = cudaMalloc(&m->d_w, sizeof(double) * n_contacts)) != cudaSuccess ||
      (e = cudaMemcpy(m->d_sw, m->sw.data(), sizeof(SwitchParams) * m->sw.size(), cudaMemcpyHostToDevice)) !=
          cudaSuccess ||
      (e = cudaMemcpy(m->d_ref, m->ref.data(), sizeof(double) * n_contacts, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(m->d_w, m->w.data(), sizeof(double) * n_contacts, cudaMemcpyHostToDevice)) != cudaSuccess)
    return m->fail(COORD_ERR_CUDA, std::string("CONTACTMAP set-up: ") + cudaGetErrorString(e));
  return COORD_OK;
}

int coord_cmap_destroy(coord_cmap *m) {
  if (!m) return COORD_OK;
  cudaSetDevice(m->device);
  cmap_free(m);
  delete m;
  return COORD_OK;
}

const char *coord_cmap_last_error(const coord_cmap *m) { return m ? m->err.c_str() : "null contact map"; }

int coord_cmap_forward_device(coord_cmap *m, int n_frames, const double *pos, const double *boxes, double *value,
                              double *deriv, double *virial, void *stream) {
  if (!m) return COORD_ERR_ARG;
  if (n_frames < 1 || !pos || !boxes || !value) return m->fail(COORD_ERR_ARG, "null positions, boxes or values");
  if (!m->d_sw) return m->fail(COORD_ERR_STATE, "the contact map was not created");
  cudaSetDevice(m->device);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  const int nblocks = (int)((m->n + kCmapBlock - 1) / kCmapBlock);
  if (n_frames > m->frames_cap) {
    // grown only when a call brings more frames than any before
    cudaDeviceSynchronize();
    cudaFree(m->d_pbc);
    cudaFree(m->d_partials);
    cudaFree(m->d_tickets);
    m->d_pbc = nullptr;
    m->d_partials = nullptr;
    m->d_tickets = nullptr;
    if ((e = cudaMalloc(&m->d_pbc, sizeof(PbcParams) * n_frames)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_partials, sizeof(double) * (size_t)n_frames * nblocks * kPartials)) != cudaSuccess ||
        (e = cudaMalloc(&m->d_tickets, sizeof(unsigned) * n_frames)) != cudaSuccess ||
        (e = cudaMemset(m->d_tickets, 0, sizeof(unsigned) * n_frames)) != cudaSuccess ||
        (e = cudaDeviceSynchronize()) != cudaSuccess) {
      m->frames_cap = 0;
      return m->fail(COORD_ERR_NOMEM, std::string("CONTACTMAP buffers: ") + cudaGetErrorString(e));
    }
    m->frames_cap = n_frames;
  }
  std::vector<PbcParams> pb(n_frames);
  for (int f = 0; f < n_frames; f++) pbc_setup(boxes + 9 * (size_t)f, &pb[f]);
  // the copy is synchronous with respect to the host array, ordered on the stream
  if ((e = cudaMemcpyAsync(m->d_pbc, pb.data(), sizeof(PbcParams) * n_frames, cudaMemcpyHostToDevice, st)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return m->fail(COORD_ERR_CUDA, std::string("CONTACTMAP boxes: ") + cudaGetErrorString(e));
  KArgs a{};
  a.nframes = n_frames;
  a.partials = m->d_partials;
  a.max_blocks = nblocks;
  a.tickets = m->d_tickets;
  a.out_s = m->mode == COORD_CMAP_COMPONENTS ? nullptr : value;
  a.out_virial = m->mode == COORD_CMAP_COMPONENTS ? nullptr : virial;
  const dim3 g(nblocks, n_frames);
  const int n = (int)m->n, nsw = (int)m->sw.size();
  if (m->mode == COORD_CMAP_COMPONENTS)
    k_cmap<COORD_CMAP_COMPONENTS><<<g, kCmapBlock, 0, st>>>(a, n, nsw, m->d_sw, m->d_ref, m->d_w, m->d_pbc,
                                                            !m->nopbc, pos, value, deriv, virial);
  else if (m->mode == COORD_CMAP_SUM)
    k_cmap<COORD_CMAP_SUM><<<g, kCmapBlock, 0, st>>>(a, n, nsw, m->d_sw, m->d_ref, m->d_w, m->d_pbc, !m->nopbc, pos,
                                                     value, deriv, virial);
  else
    k_cmap<COORD_CMAP_CMDIST><<<g, kCmapBlock, 0, st>>>(a, n, nsw, m->d_sw, m->d_ref, m->d_w, m->d_pbc, !m->nopbc,
                                                        pos, value, deriv, virial);
  g_launches += 1;
  if ((e = cudaGetLastError()) != cudaSuccess)
    return m->fail(COORD_ERR_CUDA, std::string("CONTACTMAP launch: ") + cudaGetErrorString(e));
  return COORD_OK;
}

int coord_cmap_forward(coord_cmap *m, const double *pos, const double box[9], double *value, double *deriv,
                       double *virial) {
  if (!m) return COORD_ERR_ARG;
  if (!pos || !box || !value) return m->fail(COORD_ERR_ARG, "null positions, box or values");
  if (!m->d_sw) return m->fail(COORD_ERR_STATE, "the contact map was not created");
  cudaSetDevice(m->device);
  const size_t n = (size_t)m->n, nv = m->mode == COORD_CMAP_COMPONENTS ? n : 1;
  const size_t npos = 6 * n, nder = 6 * n, nvir = 9 * nv, total = npos + nv + nder + nvir;
  cudaError_t e;
  if (!m->d_stage && (e = cudaMalloc(&m->d_stage, sizeof(double) * total)) != cudaSuccess)
    return m->fail(COORD_ERR_NOMEM, std::string("CONTACTMAP staging: ") + cudaGetErrorString(e));
  double *d_pos = m->d_stage, *d_val = d_pos + npos, *d_der = d_val + nv, *d_vir = d_der + nder;
  if ((e = cudaMemcpy(d_pos, pos, sizeof(double) * npos, cudaMemcpyHostToDevice)) != cudaSuccess)
    return m->fail(COORD_ERR_CUDA, std::string("CONTACTMAP positions: ") + cudaGetErrorString(e));
  if (int rc = coord_cmap_forward_device(m, 1, d_pos, box, d_val, d_der, d_vir, nullptr)) return rc;
  if ((e = cudaMemcpy(value, d_val, sizeof(double) * nv, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (deriv && (e = cudaMemcpy(deriv, d_der, sizeof(double) * nder, cudaMemcpyDeviceToHost)) != cudaSuccess) ||
      (virial && (e = cudaMemcpy(virial, d_vir, sizeof(double) * nvir, cudaMemcpyDeviceToHost)) != cudaSuccess))
    return m->fail(COORD_ERR_CUDA, std::string("CONTACTMAP results: ") + cudaGetErrorString(e));
  return COORD_OK;
}

} // extern "C"
