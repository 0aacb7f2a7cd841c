/*
 * coordgpu.h -- C ABI of libcoordgpu.so, a GB300 (sm_103a) implementation of
 * PLUMED's COORDINATION collective variable.
 *
 * The library replaces, behind PLUMED's own action interface, the hot path of
 *   src/colvar/CoordinationBase.cpp:142-231   CoordinationBase::calculate
 *   src/colvar/Coordination.cpp:103-163       Coordination (keywords, pairing)
 *   src/tools/SwitchingFunction.cpp           SwitchingFunction::calculateSqr
 *   src/tools/NeighborList.cpp:168-315        NeighborList::update
 *   src/tools/Pbc.cpp:362-415, Tools.h:547    minimum-image distances
 * A PLUMED plugin (plumed2_gb300/plugin/CoordinationGPU.cpp) registers the
 * COORDINATION directive and forwards each calculate() to coord_forward().
 *
 * Conventions
 *  - coord_create() validates keywords and sets up the switching function
 *    without touching CUDA; the device is initialised by coord_set_groups().
 *  - Every entry point returns an int status (COORD_OK == 0).  A nonzero status
 *    leaves a message retrievable with coord_last_error(ctx).
 *  - Positions are AoS doubles, 3 per slot; slots are GROUPA followed by
 *    GROUPB, in the order given to coord_set_groups (the order in which
 *    CoordinationBase requests its atoms, NeighborList.cpp:62-67).
 *  - Boxes are 3x3 row-major doubles (row i = lattice vector i), as passed to
 *    Pbc::setBox; an all-zero box means no periodicity.
 *  - Derivatives are ds/dx per slot (AoS, 3 per slot); the virial is the 3x3
 *    box derivative -sum dfunc * d (x) d, in the layout of
 *    Colvar::setBoxDerivatives (Colvar.h:74-113).
 *  - No function allocates or frees caller memory; the context owns its
 *    device buffers.  Host-pointer functions copy in/out through pinned
 *    staging on the context's stream; *_device functions take device pointers
 *    and a cudaStream_t passed as void*.  NULL orders the call like work on
 *    the legacy default stream (it runs on the context's own stream, fenced
 *    with events against the default stream on both sides).
 *  - A context is not thread-safe; use one per action instance (the
 *    reference's contract: one Colvar per action, CoordinationBase.h:33).
 */
#ifndef COORDGPU_H
#define COORDGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define COORD_OK 0
#define COORD_ERR_ARG 1         /* invalid argument / keyword error          */
#define COORD_ERR_CUDA 2        /* CUDA runtime error                        */
#define COORD_ERR_BOX 3         /* box not usable (see Pbc::setBox)          */
#define COORD_ERR_UNSUPPORTED 4 /* valid input the library does not handle   */
#define COORD_ERR_NOMEM 5       /* device allocation failed                  */
#define COORD_ERR_TIMEOUT 6     /* a bounded device-side wait expired        */
#define COORD_ERR_STATE 7       /* call out of order (e.g. no groups set)    */

/* ---- parameters: the COORDINATION keyword surface ------------------------ */
/* Mirrors CoordinationBase::registerKeywords (CoordinationBase.cpp:30-40)
 * and Coordination::registerKeywords (Coordination.cpp:115-126). */
#define COORD_NL_NONE 0     /* no NLIST: every pair, every step             */
#define COORD_NL_CLASSIC 1  /* NLIST: pairs with |d|<=NL_CUTOFF, rebuilt every NL_STRIDE */
#define COORD_NL_CELLS 2    /* NLISTCELLS: pairs in neighbouring link cells  */

#define COORD_PREC_FP64 0   /* FP64 throughout: the drop-in path            */
#define COORD_PREC_MIXED 1  /* FP32 pair math, compensated FP64 sums        */

typedef struct {
  const char *switch_def; /* SWITCH={...} body, e.g. "RATIONAL R_0=0.3 D_MAX=1.0";
                             NULL/"" selects the R_0/NN/MM/D_0 keywords below */
  double r0;              /* R_0 (required and >0 when switch_def is empty)  */
  double d0;              /* D_0 (default 0.0)                               */
  int nn;                 /* NN  (default 6)                                 */
  int mm;                 /* MM  (default 0 -> 2*NN)                         */
  int nopbc;              /* NOPBC flag                                      */
  int pair;               /* PAIR flag                                       */
  int nlist;              /* COORD_NL_*                                      */
  double nl_cutoff;       /* NL_CUTOFF (>0 when nlist != NONE)               */
  int nl_stride;          /* NL_STRIDE (>0 when nlist != NONE)               */
  int serial;             /* SERIAL flag (accepted; no effect on the GPU)    */
  int precision;          /* COORD_PREC_*                                    */
  int device;             /* CUDA device ordinal                             */
} coord_params;

typedef struct coord_ctx coord_ctx;

/* Fill p with the reference defaults (NN=6, MM=0, D_0=0, FP64, device 0). */
void coord_params_default(coord_params *p);

/* Create a context: parses SWITCH / R_0,NN,MM,D_0 exactly as
 * Coordination::Coordination (Coordination.cpp:128-157) and checks the
 * NLIST/NL_CUTOFF/NL_STRIDE/PAIR rules of CoordinationBase.cpp:66-84. */
int coord_create(const coord_params *p, coord_ctx **out);
int coord_destroy(coord_ctx *ctx);
const char *coord_last_error(const coord_ctx *ctx);
const char *coord_status_string(int status);

/* Groups as absolute atom indices (AtomNumber::index()).  n_b==0 selects the
 * single-list N(N-1)/2 form; PAIR pairs a[i] with b[i].  Pairs whose two
 * absolute indices are equal are skipped (CoordinationBase.cpp:183). */
int coord_set_groups(coord_ctx *ctx, const int64_t *group_a, int64_t n_a, const int64_t *group_b, int64_t n_b);

/* Number of slots (n_a + n_b). */
int coord_get_nslots(const coord_ctx *ctx, int64_t *nslots);

/* ---- sibling CVs of CoordinationBase ---------------------------------------
 * DHENERGY and GHBFIX run CoordinationBase::calculate's loop (groups, PAIR,
 * NLIST/NLISTCELLS, NOPBC, derivatives and virial) with their own pairing()
 * in place of the switching function.  A context becomes one of them through
 * the calls below, after coord_create (whose switching-function keywords are
 * then unused: give any valid set, e.g. r0 = 1).  FP64 precision only; the
 * R_0/D_0 derivatives (COORD_FLAG_DR0, grad_param) are refused. */
#define COORD_CV_COORDINATION 0
#define COORD_CV_DHENERGY 1 /* colvar/DHEnergy.cpp:62 */
#define COORD_CV_GHBFIX 2   /* colvar/GHBFIX.cpp:63   */

/* DHENERGY keywords I, TEMP, EPSILON (DHEnergy.cpp:80-86) and the action's
 * units (Units::getEnergy/getLength/getCharge; 1,1,1 for kJ/mol, nm, e).
 * k = sqrt(I/(EPSILON*TEMP))*502.903741125*length and the prefactor
 * 138.935458111/energy/length*charge^2 as DHEnergy.cpp:112-113; the pairing
 * of DHEnergy.cpp:128-142.  Replaces DHEnergy::DHEnergy. */
int coord_set_dhenergy(coord_ctx *ctx, double ionic_strength, double temp, double epsilon, double unit_energy,
                       double unit_length, double unit_charge);
/* DHENERGY's per-atom charges (Atoms::getCharge, in the action's charge
 * unit), indexed by absolute atom index like the groups; n_atoms must cover
 * every atom of the groups (checked at the next forward). */
int coord_set_charges(coord_ctx *ctx, const double *charges, int64_t n_atoms);
/* GHBFIX keywords D_0, D_MAX, C (GHBFIX.cpp:111-126) and its tables:
 * types[a] = type id of absolute atom a (the TYPES file, ids in order of
 * first appearance), eta = n_types x n_types scaling matrix (the PARAMS file,
 * eta[n*t1+t2], already in the action's energy unit).  A group atom beyond
 * n_atoms is an error at the next forward, with the message of
 * GHBFIX.cpp:181-186.  Replaces GHBFIX::GHBFIX. */
int coord_set_ghbfix(coord_ctx *ctx, double d0, double dmax, double c, const int32_t *types, int64_t n_atoms,
                     const double *eta, int n_types);

/* The context's switching function evaluated on the host:
 * SwitchingFunction::calculateSqr (squared != 0, x = r^2) or ::calculate
 * (x = r), SwitchingFunction.cpp:1163-1175.  f and df receive n values. */
int coord_switch_eval(const coord_ctx *ctx, int n, const double *x, int squared, double *f, double *df);
/* Its constants d0, dmax, dmax^2, 1/r0, 1/r0^2, stretch, shift
 * (switchContainers::Data, SwitchingFunction.h:57-95). */
int coord_switch_params(const coord_ctx *ctx, double out[7]);

/* ---- forward: CV, derivatives, virial ------------------------------------ */
#define COORD_FLAG_REBUILD 1u   /* force a neighbour-list rebuild this step   */
#define COORD_FLAG_NO_DERIV 2u  /* compute s only (no derivatives, no virial) */
#define COORD_FLAG_DR0 4u       /* also return ds/dR_0 and ds/dD_0            */
#define COORD_FLAG_SAVE 8u      /* keep ds/dx and the virial of this forward
                                   (and ds/d(R_0,D_0) with COORD_FLAG_DR0) in
                                   the context for the next
                                   coord_backward_device (the positions must be
                                   unchanged in between, like saved tensors)  */

/* One step of CoordinationBase::prepare()+calculate() for one frame, host
 * buffers.  The neighbour list is rebuilt when the list is new, when
 * step % NL_STRIDE == 0, or on COORD_FLAG_REBUILD (NeighborList::prepare,
 * NeighborList.cpp:433-456).  pos: nslots*3; deriv: nslots*3 (may be NULL
 * with COORD_FLAG_NO_DERIV); virial: 9 (may be NULL). */
int coord_forward(coord_ctx *ctx, const double *pos, const double box[9], int64_t step, unsigned flags, double *s,
                  double *deriv, double *virial);
/* coord_forward for n_frames frames (walkers or trajectory frames) of one
 * context in one call: pos [frames][slots][3], boxes [frames][9], s
 * [frames], deriv [frames][slots][3] and virial [frames][9] are host arrays.
 * Same host paths as coord_forward; every frame has its own neighbour list.
 * No reference counterpart: a host that drives several walkers in one
 * process can make one call instead of one per walker. */
int coord_forward_batch(coord_ctx *ctx, int n_frames, const double *pos, const double *boxes, int64_t step,
                        unsigned flags, double *s, double *deriv, double *virial);

/* Batched form for walkers / trajectory frames sharing one action definition:
 * n_frames independent frames, each with its own neighbour list.  Device
 * pointers: pos [n_frames][nslots][3], s [n_frames], deriv
 * [n_frames][nslots][3], virial [n_frames][9], dparam [n_frames][2]
 * (ds/dR_0, ds/dD_0; only with COORD_FLAG_DR0, else may be NULL).  boxes are
 * HOST [n_frames][9].  stream: cudaStream_t or NULL. */
int coord_forward_device(coord_ctx *ctx, int n_frames, const double *pos, const double *boxes, int64_t step,
                         unsigned flags, double *s, double *deriv, double *virial, double *dparam, void *stream);

/* ---- backward: gradients of an upstream scalar ---------------------------- */
/* Given g[f] = dV/ds for each frame (device), returns on the device
 * grad_pos [n_frames][nslots][3] = g * ds/dx, grad_box [n_frames][9] =
 * g * ds/dh (h = box, scaled coordinates held fixed; the box-derivative
 * convention of ActionAtomistic.cpp:221-265), grad_param [n_frames][2] =
 * g * (ds/dR_0, ds/dD_0).  Reuses the neighbour list of the last forward;
 * any output pointer may be NULL.  After a forward with COORD_FLAG_SAVE on
 * the same frames it only scales the saved quantities (an O(N) kernel; with
 * grad_param set this needs COORD_FLAG_DR0 on that forward too); otherwise
 * it runs a pair pass over the positions given. */
int coord_backward_device(coord_ctx *ctx, int n_frames, const double *pos, const double *boxes, const double *g,
                          double *grad_pos, double *grad_box, double *grad_param, void *stream);

/* ---- per-atom coordination -------------------------------------------------
 * COORDINATIONNUMBER (symfunc/CoordinationNumbers.cpp:247-309) is a
 * CONTACT_MATRIX (adjmat/ContactMatrix.h:95-120) times a vector of ones:
 * cn_i = sum_j sigma(r_ij) over the pairs of slot i.  Replaces that
 * CONTACT_MATRIX + MATRIX_VECTOR_PRODUCT chain.  A pair with r^2 < DBL_EPSILON
 * or sigma < DBL_EPSILON contributes nothing, as in ContactMatrix.h:99-107.
 * Needs a COORDINATION context with NLIST or NLISTCELLS (the contact matrix's
 * link cells have cutoff d_max; a classic list with NL_CUTOFF = d_max and
 * NL_STRIDE = 1 holds exactly its nonzero pairs) and no PAIR.
 * Single list (SPECIES): every slot's sum over its pairs.  Two lists
 * (SPECIESA, SPECIESB): GROUPA slots get the row sums of the reference's
 * matrix; GROUPB slots get the column sums, which the reference does not
 * output.
 * cn [frames][slots] and s [frames] (NULL allowed: sum of sigma over the
 * pairs) are device pointers; flags: COORD_FLAG_REBUILD only. */
int coord_peratom_device(coord_ctx *ctx, int n_frames, const double *pos, const double *boxes, int64_t step,
                         unsigned flags, double *cn, double *s, void *stream);
/* Vector-Jacobian product of the per-atom forward: g [frames][slots] is
 * dV/dcn; grad_pos [frames][slots][3] receives dV/dx = sum over pairs of
 * (g_i + g_j) dsigma_ij/dx, grad_box [frames][9] dV/dh (NULL allowed), on
 * the neighbour lists of the last forward with the same frames. */
int coord_peratom_backward_device(coord_ctx *ctx, int n_frames, const double *pos, const double *boxes,
                                  const double *g, double *grad_pos, double *grad_box, void *stream);

/* Force application on the device (Colvar::apply, src/core/Colvar.cpp:50-60;
 * ActionWithValue::checkForForces, src/core/ActionWithValue.cpp:337-411;
 * ActionAtomistic::setForcesOnAtoms/setForcesOnCell, ActionAtomistic.cpp:
 * 502-549) after a forward with COORD_FLAG_SAVE on the same frames: for every
 * frame f and slot i, atom_forces[f][abs(i)][0..2] += ff[f] * ds/dx_i, and
 * box_forces[f][0..8] += ff[f] * virial[f] (either output may be NULL).
 * ff[f] is the force on the CV (-dV/ds); atom_forces is the engine's
 * [n_frames][n_atoms][3] device array, indexed by the absolute atom indices
 * of coord_set_groups.  Device arrays; consumes the saved state. */
int coord_apply_forces(coord_ctx *ctx, int n_frames, const double *ff, int64_t n_atoms, double *atom_forces,
                       double *box_forces, void *stream);

/* ---- neighbour list introspection ------------------------------------------ */
/* nl->size() of the last build for frame f (pairs processed per step,
 * CoordinationBase.cpp:163), including pairs skipped as self pairs. */
int coord_nl_size(coord_ctx *ctx, int frame, int64_t *n);
/* No reference counterpart.  Of those pairs, how many lie in the rows' near
 * parts (within D_MAX plus the skin at the last build): the entries a step
 * reads while every atom has moved less than half the skin since the build.
 * Equals coord_nl_size's count less the self pairs when the lists are not
 * split (no finite D_MAX below NL_CUTOFF, no orthorhombic box, or a sibling
 * CV).  skin (may be NULL) receives the skin in length units, 0 when not
 * split. */
int coord_nl_near_size(coord_ctx *ctx, int frame, int64_t *n, double *skin);
/* The pair set of the last build for frame f as (first, second) slot pairs
 * in the reference's orientation (first<second for a single list, first in
 * GROUPA otherwise), sorted; writes min(n, cap) pairs, returns n. */
int coord_get_pairs(coord_ctx *ctx, int frame, uint32_t *pairs, int64_t cap, int64_t *n);

/* ---- many actions in one launch ------------------------------------------- */
/* A batch of contexts whose groups index one shared system of n_atoms atoms
 * (absolute indices = rows of pos).  One forward evaluates every action on
 * every frame in a single persistent launch.  Device pointers: pos
 * [n_frames][n_atoms][3]; s [n_frames][n_actions]; deriv: for each frame, for
 * each action, nslots_k*3 values, concatenated (offsets from
 * coord_multi_deriv_offset); virial [n_frames][n_actions][9]. */
typedef struct coord_multi coord_multi;
int coord_multi_create(coord_ctx *const *ctxs, int n_actions, int64_t n_atoms, coord_multi **out);
int coord_multi_destroy(coord_multi *m);
int coord_multi_deriv_offset(const coord_multi *m, int action, int64_t *offset, int64_t *per_frame);
int coord_multi_forward_device(coord_multi *m, int n_frames, const double *pos, const double *boxes, unsigned flags,
                               double *s, double *deriv, double *virial, void *stream);
/* Record the next coord_multi_forward_device call into a CUDA graph and
 * replay it on later calls with the same shapes (1) or launch directly (0). */
int coord_multi_use_graph(coord_multi *m, int enable);
const char *coord_multi_last_error(const coord_multi *m);

/* ---- CONTACTMAP (colvar/ContactMap.cpp:149-365) ----------------------------
 * Explicit contacts i = (ATOMSi[0], ATOMSi[1]), each with its switching
 * function (one SWITCH for all, or SWITCHi), REFERENCEi (default 0) and
 * WEIGHTi (default 1):  c_i = w_i (sigma_i(|d|) - ref_i), sigma from
 * SwitchingFunction::calculate of the minimum-image distance.
 *   COORD_CMAP_COMPONENTS  value[f][i] = c_i (components contact-i),
 *                          virial[f][i][9] the box derivatives of c_i
 *   COORD_CMAP_SUM         value[f] = sum_i c_i, virial[f][9]
 *   COORD_CMAP_CMDIST      value[f] = sum_i c_i^2, virial[f][9]
 * Positions are [frames][2n][3]: the first atoms of all contacts, then the
 * second atoms (the reference's request order); deriv [frames][2n][3] gets
 * the derivative of the contact's value (components) or of the sum for each
 * slot.  boxes: host [frames][9].  FP64.  Replaces ContactMap::ContactMap
 * and ContactMap::calculate. */
#define COORD_CMAP_COMPONENTS 0
#define COORD_CMAP_SUM 1
#define COORD_CMAP_CMDIST 2
typedef struct coord_cmap coord_cmap;
int coord_cmap_create(int64_t n_contacts, const char *const *switch_defs, int n_switch_defs, const double *reference,
                      const double *weight, int mode, int nopbc, int device, coord_cmap **out);
int coord_cmap_destroy(coord_cmap *m);
const char *coord_cmap_last_error(const coord_cmap *m);
/* value and virial as above; deriv and virial may be NULL.  Calls on one
 * context are ordered on their stream (NULL: the legacy default stream). */
int coord_cmap_forward_device(coord_cmap *m, int n_frames, const double *pos, const double *boxes, double *value,
                              double *deriv, double *virial, void *stream);
/* One frame from host arrays (the plugin's call): pos (2n x 3), box[9];
 * value, deriv (2n x 3) and virial as above, on the host. */
int coord_cmap_forward(coord_cmap *m, const double *pos, const double box[9], double *value, double *deriv,
                       double *virial);

/* ---- forward without device allocation ------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they call in (an MD engine that reserves its whole device pool
 * up front and forbids other allocations during a run): the FP64 every-pair
 * forward (no NLIST, no PAIR) with all working memory in one static device
 * array of COORD_NOALLOC_MAX_SLOTS slots that each GPU keeps until exit.
 * ctx comes from coord_create (which touches no CUDA); do not call
 * coord_set_groups on it.  Groups are host arrays of absolute indices; pos,
 * s, deriv and virial are device pointers on the current device; box is
 * host; stream is a cudaStream_t or NULL.  pos and deriv are indexed by
 * slot, as for coord_forward: (n_a + n_b) rows of 3 doubles, group_a's atoms
 * then group_b's in the order given, an atom listed twice taking two rows.
 * They are not the engine's whole position and force arrays indexed by
 * atom number.  The call allocates nothing and
 * clears the parts of the shared array that must start at zero; calls that
 * overlap on the GPU share the array and race.  Every call copies the frame
 * constants and the groups from host memory the call owns only while it
 * runs, so it cannot be captured into a CUDA graph (call it outside stream
 * capture).  More than COORD_NOALLOC_MAX_SLOTS slots: COORD_ERR_ARG. */
#define COORD_NOALLOC_MAX_SLOTS 32768
int coord_forward_noalloc(coord_ctx *ctx, const int64_t *group_a, int64_t n_a, const int64_t *group_b, int64_t n_b,
                          const double *pos, const double box[9], double *s, double *deriv, double *virial,
                          void *stream);

/* ---- tuning and measurement ------------------------------------------------ */
/* The configuration the autotuner chose for this context, as text.  The
 * autotuner runs on the first forward of a mixed-precision neighbour-list
 * context (blocks per SM x gathers in flight, each timed once); batches
 * (coord_multi_*) tune tile size x blocks per SM on their first call. */
int coord_autotune(coord_ctx *ctx, char *desc, size_t desclen);
/* Microbenchmarks of the device (FP32 FMA, FP64 FMA TFLOP/s, HBM copy GB/s). */
int coord_measure_peaks(int device, double *fp32_tflops, double *fp64_tflops, double *hbm_gbs);
/* ---- biases on the CV, on the device ------------------------------------- */
/* Sum of truncated Gaussian hills of a one-dimensional CV for every frame:
 * the non-multivariate hills of METAD (MetaD::evaluateGaussianAndDerivatives,
 * src/bias/MetaD.cpp:2148-2181,2256-2273; cutoff dp2 < 6.25 and the stretch
 * of src/tools/Tools.h:71-74, on when stretch != 0).  Device arrays: s
 * [n_frames]; centers, sigmas, heights [n_frames][n_hills]; V, dVds
 * [n_frames] (either may be NULL), overwritten or, with accumulate != 0,
 * added to.  Runs on `stream` (NULL: the legacy default stream). */
int coord_bias_hills(int n_frames, const double *s, int n_hills, const double *centers, const double *sigmas,
                     const double *heights, int stretch, int accumulate, double *V, double *dVds, void *stream);
/* RESTRAINT on one argument (Restraint::calculate, src/bias/Restraint.cpp:
 * 125-141): V = kappa/2 (s-at)^2 + slope (s-at), dV/ds = kappa (s-at) + slope
 * for every frame; same array conventions as coord_bias_hills. */
int coord_bias_restraint(int n_frames, const double *s, double at, double kappa, double slope, int accumulate,
                         double *V, double *dVds, void *stream);

/* Whether the device reads and writes pageable host memory coherently
 * (cudaDevAttrPageableMemoryAccess) and does so through the host's page
 * tables without migrating pages (cudaDevAttrPageableMemoryAccessUsesHostPageTables,
 * e.g. a Grace CPU with NVLink-C2C).  When both hold, coord_forward moves
 * positions and results with kernels that access the caller's arrays
 * directly instead of staging them through pinned buffers (unless the
 * environment sets COORD_HOST_STAGED=1 when the context first runs).  No
 * reference counterpart. */
int coord_host_memory_access(int device, int *pageable, int *host_page_tables);

/* How the last host-array call of ctx (coord_forward, coord_forward_batch)
 * moved the caller's arrays: COORD_HOST_PATH_STAGED through the context's
 * pinned buffers, COORD_HOST_PATH_DIRECT by kernels that access the arrays in
 * place, COORD_HOST_PATH_CHUNKED (page-locked arrays of several frames) by the
 * copy engines, chunk by chunk beside the kernels of other chunks; -1 before
 * the first such call or for a null ctx.  A rebuild step moves the arrays
 * directly.  No reference counterpart (diagnostics). */
#define COORD_HOST_PATH_STAGED 0
#define COORD_HOST_PATH_DIRECT 1
#define COORD_HOST_PATH_CHUNKED 2
int coord_host_path(const coord_ctx *ctx);

/* Kernel launches issued by this library since load (for launch accounting). */
int64_t coord_launch_count(void);
/* Average device time (ms) of the pair-evaluation kernel over the launches
 * since timing was enabled or last read, from CUDA events recorded around it
 * on the stream it runs on; count receives the number of launches (may be
 * NULL).  Waits for those events; resets the record. */
int coord_last_kernel_ms(coord_ctx *ctx, double *ms, int *count);
/* Turn per-launch event timing of the pair kernel on/off (default off). */
int coord_set_timing(coord_ctx *ctx, int enable);
/* The individual device times (ms) behind coord_last_kernel_ms, in launch
 * order: writes min(count, cap) values and returns count in *count.  Waits for
 * the events; does not reset the record (coord_last_kernel_ms does).
 * Diagnostic; no reference counterpart. */
int coord_kernel_times(coord_ctx *ctx, float *ms, int cap, int *count);

#ifdef __cplusplus
}
#endif
#endif
