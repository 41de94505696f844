/*
 * tetemoko_gb300.h -- C ABI of the GB300 (sm_103a) per-level Godunov step of
 * tetemoko's 2-D velocity-stress elasticity with fault boundaries.
 *
 * Every entry point is plain C: pointers, sizes and POD structs only.  A Chombo
 * build calls these from thin shims that keep the reference's class names
 * (LinElastLevelGodunov, LinElastPatchGodunov, LEPhysIBC/RSIBC/SWIBC,
 * LinElastPhysics::plasticUpdate).
 *
 * Data layout.  State arrays use Chombo's FArrayBox layout: structure of arrays,
 * i fastest, then j, then component, over the allocated box (valid box grown by
 * the ghost width).  The 22 state components are those of srcLinElast/LEINDEX.H:12-47
 * (side 1: vx vy vz sxx syy szz sxy sxz syz lambda gamma; side 2 at +11).
 * Fault ("boundary") data live on the row of y-lo faces of a patch, indexed by
 * the face's i, with 11 components for rate-and-state (ibcLinElast/RSINDEX.H:12-22)
 * and 9 for slip weakening (ibcLinElast/SWIBCF.ChF:32-72).
 *
 * Units follow the reference decks: km, km/s, g/cm^3, GPa (G), MPa (stress),
 * m/s (particle and slip velocity), m (slip, L, Dc), s.
 *
 * Errors.  Every call returns a tmk_status code and never aborts the process.
 * Device kernels never trap: they record the first problem in a device status
 * word that the host reads after the step (tmk_level_status).
 */
#ifndef TETEMOKO_GB300_H
#define TETEMOKO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TMK_ABI_VERSION 5   /* 2: tmk_scheme gained use_fourth_order_slopes; 3: tmk_tuning gained fault_first;
                               4: tmk_tag_params gained slip_rate_thresh; 5: tmk_tuning gained plastic_fused */

#define TMK_NCOMP      22   /* state components, srcLinElast/LEINDEX.H:12-47 */
#define TMK_NSIDE_COMP 11   /* IX_OFFSET, srcLinElast/LEINDEX.H:23 */
#define TMK_RS_NBDRY   11   /* rate-and-state boundary components, ibcLinElast/RSINDEX.H */
#define TMK_SW_NBDRY    9   /* slip-weakening boundary components, ibcLinElast/SWIBC.cpp:63 */
#define TMK_NGHOST      4   /* m_numGhost for PPM, srcLinElast/LinElastLevelGodunov.cpp:108-115 */
#define TMK_SW_MAX_PATCHES 8

/* ---- status codes (the reference aborts through MayDay::Error / Fortran stop) ---- */
typedef enum {
  TMK_OK                = 0,
  TMK_ERR_BAD_DESC      = 1,  /* inconsistent box / FAB descriptor or parameter */
  TMK_ERR_NAN_STATE     = 2,  /* NaN state variable (ibcLinElast/RSIBCF.ChF:133-145 stops) */
  TMK_ERR_TIMEOUT       = 3,  /* a bounded device wait ran out */
  TMK_ERR_CUDA          = 4,  /* a CUDA runtime call failed */
  TMK_ERR_UNSUPPORTED   = 5,  /* option the reference rejects or this build lacks */
  TMK_ERR_ALLOC         = 6,  /* device allocation failed */
  TMK_ERR_NO_DEVICE     = 7,  /* no CUDA device visible */
  TMK_ERR_TOO_LARGE     = 8   /* patch needs more than the fixed scratch of
                                 tmk_patch_update_state_noalloc */
} tmk_status;

/* boundary types of comp.x_boundary / y_boundary (execLinElast/amrGodunov.cpp:571-590) */
enum { TMK_BC_OUTFLOW = 0, TMK_BC_FREE = 1, TMK_BC_FAULT = 2 };
/* friction law plugged into the y-lo face (LEPhysIBC subclasses) */
enum { TMK_FAULT_NONE = 0, TMK_FAULT_RS = 1, TMK_FAULT_SW = 2 };
/* rate-and-state state evolution: the reference's slip law (ibcLinElast/RSIBCF.ChF:125-132)
 * or the aging law, an extension absent from the reference */
enum { TMK_RS_SLIP_LAW = 0, TMK_RS_AGING_LAW = 1 };
/* slip-weakening side-2 component offset: the reference reads/writes side 2 at
 * component 9 (ibcLinElast/SWIBCF.ChF:139-147,255-263); 11 is IX_OFFSET */
enum { TMK_SW_LAYOUT_REFERENCE9 = 0, TMK_SW_LAYOUT_OFFSET11 = 1 };
/* arithmetic of the volume stencil */
enum { TMK_PREC_FP64 = 0, TMK_PREC_MIXED = 1 };

/* LEPhysIBC::setFortranCommonLE -> LINELASTSETF (srcLinElast/LinElastPhysicsF.ChF:1149-1210) */
typedef struct {
  double cs, cp, G;                       /* G is overridden by rho*cs^2 when rho > 0 */
  double rho;                             /* <= 0: derive from G (execLinElast/amrGodunov.cpp:206-215) */
  double sxx0, syy0, szz0, sxy0, sxz0, syz0;
} tmk_elastic_params;

/* RSIBC constructor -> RSSETF (ibcLinElast/RSIBCF.ChF:8-55, ibcLinElast/RSIBC.cpp:17-51) */
typedef struct {
  double r0, x0, y0, nsig, ntime;         /* Gaussian nucleation: nsig*exp(-(x/r0)^2/2) */
  double a, b, V0, f0, L, fw, Vw, fexp;
  double ramp_x, ramp_w, ramp_a, ramp_Vw;
  double rupture_threshold;
  double psi_init;                        /* RSIBC::initializeBdry psi (ibcLinElast/RSIBC.cpp:158-160) */
  int    state_law;                       /* TMK_RS_SLIP_LAW (reference) or TMK_RS_AGING_LAW */
} tmk_rs_params;

/* SWIBC constructor -> SWSETF (ibcLinElast/SWIBCF.ChF:6-27, ibcLinElast/SWIBC.cpp:16-52) */
typedef struct {
  double fs, fd, dw, smooth;
  int    num_patches;
  double xc[TMK_SW_MAX_PATCHES], xw[TMK_SW_MAX_PATCHES];
  double zc[TMK_SW_MAX_PATCHES], zw[TMK_SW_MAX_PATCHES];
  double tau[TMK_SW_MAX_PATCHES];
  double fric_box_center[2], fric_box_width[2];
  double outside_friction;
  double rupture_threshold;
  int    layout;                          /* TMK_SW_LAYOUT_* */
} tmk_sw_params;

/* setFortranCommonPlastic -> PLASTICSETF (srcLinElast/PlasticPhysicsF.ChF:6-25).
 * b (cohesion term) and h (hardening) are hard-wired to 0 in the reference;
 * non-zero values are an extension. */
typedef struct { double mu, beta, eta, b, h; } tmk_plastic_params;

/* AMRLevelLinElastFactory / LinElastPatchGodunov::define options */
typedef struct {
  int normal_pred_order;                  /* 0 CTU, 1 PLM, 2 PPM (srcLinElast/LinElastPatchGodunov.cpp:272-314) */
  int use_prim_limiting;
  int use_char_limiting;
  int boundary_type[6];                   /* x lo, x hi, y lo, y hi, z lo, z hi */
  int fault_law;                          /* TMK_FAULT_* on the y-lo face when boundary_type[2]==2 */
  int plasticity;                         /* apply PLASTICCORRECTION after the step */
  int precision;                          /* TMK_PREC_* for level objects */
  int volume_kernel;                      /* TMK_VOLUME_* implementation of the volume update */
  int use_fourth_order_slopes;            /* comp.use_fourth_order_slopes: PLM slopes of fourth order */
} tmk_scheme;

/* Implementations of the volume update (same results to rounding):
 * TILE  shared-memory tiles, one side of the fault per CTA (fuses plasticity);
 * MARCH column-marching warps with both sides packed per lane, plasticity as a
 *       pointwise pass after the update;
 * AUTO  MARCH (TILE with the PLM predictor, which the marching kernels do not
 *       implement).  Both store the coarse-fine face fluxes of coupled levels. */
enum { TMK_VOLUME_AUTO = 0, TMK_VOLUME_TILE = 1, TMK_VOLUME_MARCH = 2 };

/* Chombo FArrayBox view: data[((c*(hi1-lo1+1)) + (j-lo1))*(hi0-lo0+1) + (i-lo0)] */
typedef struct {
  double* data;
  int lo[2], hi[2];
  int ncomp;
} tmk_fab;

typedef struct { int lo[2], hi[2]; } tmk_box;   /* cell-centred, inclusive */

/* How a level's step is cut into work (an extension: the reference's patch
 * loop has no such choices).  Defaults: the scheme's volume kernel, one wave
 * per marching group, runs of at least 16 rows, one antiplane slot per
 * fault-kernel CTA, 32 fault faces per fault-kernel CTA, the fault kernel
 * after the in-plane marching kernel, the plastic return as a pass. */
typedef struct {
  int volume_kernel;    /* TMK_VOLUME_MARCH or TMK_VOLUME_TILE (march only if the scheme allows it) */
  int march_waves[2];   /* marching items of the in-plane / antiplane group, in waves of resident CTAs: 1..8 */
  int min_run;          /* fewest rows of a marching item: 4..4096 */
  int fault_displace;   /* antiplane CTA slots left free per fault-kernel CTA: 0..4 */
  int fault_seg;        /* fault faces per fault-kernel CTA: 32 (4 warps) or 16 (2 warps) */
  int fault_first;      /* 1: the fault kernel first, running beside the in-plane marching kernel
                           (2-warp CTAs fit in the registers two in-plane CTAs leave free);
                           0: after it, beside the antiplane kernel */
  int plastic_fused;    /* plastic levels of the marching form: 1: the Drucker-Prager return is
                           applied by the in-plane marching kernel as it stores each cell (the
                           antiplane kernel runs first, the fault kernel on a side stream beside
                           both); 0: a pass over the level after the marching kernels */
} tmk_tuning;

/* Refinement tagging parameters (the comp.* keys of the input deck,
 * execLinElast/amrGodunov.cpp:274-283, 400-440; defaults there in brackets). */
typedef struct {
  int    level;                /* index of the level tagged (AMRLevel::m_level) */
  int    initial;              /* 1: tagCellsInit (fault-law marks only), 0: tagCells */
  double refine_thresh;        /* comp.refine_thresh */
  double plastic_thresh;       /* comp.plastic_thresh [1e-5] */
  int    tag_buffer;           /* comp.tag_buffer_size */
  double x_coarsen[2], y_coarsen[2];    /* comp.x_coarsen, y_coarsen [-1e40 1e40] */
  double slope_coarsen;        /* comp.slope_coarsen [0] */
  double width_coarsen;        /* comp.width_coarsen [1e40] */
  double x_coarsen2[2], y_coarsen2[2];  /* comp.x_coarsen2, y_coarsen2 [-1e40 1e40] */
  int    coarsen2_max_level;   /* comp.coarsen2_max_level [max_level] */
  double slip_rate_thresh;     /* extension (the reference has no slip-rate tag): > 0 also tags
                                  every cell of the fault row j = domain.lo[1] whose face's slip
                                  rate (rate and state: boundary component 2; slip weakening: 4)
                                  is at least this (m/s), inside the coarsen2 window; <= 0: off */
} tmk_tag_params;

typedef struct tmk_context_s tmk_context;
typedef struct tmk_level_s   tmk_level;
typedef struct tmk_level3d_s tmk_level3d;
typedef struct tmk_amr_s     tmk_amr;
typedef struct tmk_stations_s tmk_stations;
typedef struct tmk_graph_s   tmk_graph;

/* ---------------------------------------------------------------------------
 * Parameters (replaces the process-global Fortran COMMON blocks /IBC/, /rs/,
 * /slipweak/, /PLASTIC/: srcLinElast/IBCCommon.fh:4-6, ibcLinElast/RSCommon.fh:4-5,
 * ibcLinElast/SWCommon.fh:4-5, srcLinElast/PlasticCommon.fh:4-5).  Contexts are
 * independent: several scenarios can coexist in one process.
 * ------------------------------------------------------------------------- */
int  tmk_abi_version(void);
tmk_status tmk_context_create(const tmk_elastic_params* elastic,
                              const tmk_scheme* scheme,
                              const tmk_rs_params* rs,          /* NULL unless fault_law==RS */
                              const tmk_sw_params* sw,          /* NULL unless fault_law==SW */
                              const tmk_plastic_params* plastic,/* NULL unless plasticity */
                              tmk_context** out);
void tmk_context_destroy(tmk_context* ctx);
/* Derived constants of LINELASTSETF: rho, lam, K, Zs, Zp (LinElastPhysicsF.ChF:1172-1176) */
tmk_status tmk_context_constants(const tmk_context* ctx, double out[5]);

/* ---------------------------------------------------------------------------
 * Patch step on caller-owned DEVICE FABs (FP64).  Replaces
 * LinElastPatchGodunov::setCurrentTime/setCurrentBox + LEPhysIBC::setBdryData +
 * LinElastPatchGodunov::updateState (srcLinElast/LinElastPatchGodunov.H:63-83,
 * srcLinElast/LinElastPatchGodunov.cpp:101-129).  U must hold 4 filled ghost
 * cells around `valid` (cells outside `domain` are never read).  B is the
 * patch's fault FAB (face row j=domain.lo[1], x ghosts filled) or NULL when the
 * patch does not touch a fault.  F[0], F[1] (optional, may be NULL) receive
 * the face fluxes of LinElastPhysics::computeUpdate for refluxing; each is a
 * 22-component FAB over the x- or y-faces of `valid`.  Asynchronous on
 * `stream` (a cudaStream_t, NULL = legacy default stream).
 * ------------------------------------------------------------------------- */
tmk_status tmk_patch_update_state(tmk_context* ctx,
                                  const tmk_fab* U, const tmk_fab* B,
                                  const tmk_fab* Fx, const tmk_fab* Fy,
                                  const tmk_box* valid, const tmk_box* domain,
                                  double dx, double time, double dt,
                                  double* max_wave_speed, void* stream);

/* Same computation and arguments as tmk_patch_update_state, but the call
 * allocates no device memory at all.  This entry point has no counterpart in
 * the reference.  It exists for callers that cannot allocate during a step:
 * a driver that has handed the GPU's memory to its own pool (a Chombo run
 * sizing its level data to fill HBM, where a cudaMalloc here would fail), or
 * one that cannot afford the device-wide synchronisation cudaMalloc/cudaFree
 * may impose in the middle of a time step.  Its temporaries live in a fixed
 * device array of TMK_NOALLOC_SCRATCH_BYTES that every GPU loading this
 * library holds until the process exits; a patch that needs more is refused
 * with TMK_ERR_TOO_LARGE.  The first call on each device looks up that
 * array's address (make the first call before any stream capture).  All calls
 * on a device share the one array and it keeps the previous call's contents
 * (every value is rewritten before it is read): calls that overlap on the GPU
 * -- on different streams, or from several host threads -- race, so order
 * them on one stream. */
#define TMK_NOALLOC_SCRATCH_BYTES (8u << 20)
tmk_status tmk_patch_update_state_noalloc(tmk_context* ctx,
                                          const tmk_fab* U, const tmk_fab* B,
                                          const tmk_fab* Fx, const tmk_fab* Fy,
                                          const tmk_box* valid, const tmk_box* domain,
                                          double dx, double time, double dt,
                                          double* max_wave_speed, void* stream);

/* LinElastPhysics::plasticUpdate -> PLASTICCORRECTION on device FAB U over box
 * (srcLinElast/LinElastPhysics.cpp:544-554, srcLinElast/PlasticPhysicsF.ChF:30-69). */
tmk_status tmk_plastic_update(tmk_context* ctx, const tmk_fab* U,
                              const tmk_box* box, double dt, void* stream);

/* LinElastPhysics::getMaxWaveSpeed -> MAXWAVESPEEDF (LinElastPhysicsF.ChF:10-21). */
tmk_status tmk_max_wave_speed(const tmk_context* ctx, double* speed);

/* ---------------------------------------------------------------------------
 * 3-D (a CH_SPACEDIM == 3 build of the reference).  The fault is the domain's
 * y-lo plane, spanning x and z.
 * Chombo FArrayBox view: data[((c*nz + (k-lo2))*ny + (j-lo1))*nx + (i-lo0)] */
typedef struct {
  double* data;
  int lo[3], hi[3];
  int ncomp;
} tmk_fab3;

typedef struct { int lo[3], hi[3]; } tmk_box3;   /* cell-centred, inclusive */

/* LinElastPatchGodunov::updateState with CH_SPACEDIM == 3
 * (srcLinElast/LinElastPatchGodunov.cpp:101-129, 174-469: the 3-D corner
 * transport upwind corrections of :329-381 and :422-440) on one patch, FP64,
 * with the fault laws' 3-D forms (ibcLinElast/RSIBCF.ChF, SWIBCF.ChF z terms).
 * U: device FAB of 22 comps containing grow(valid, 3) & domain, updated in
 * place over valid (lambda, gamma and ghosts untouched).  B: when the scheme
 * has a fault law and valid starts on the domain's y-lo plane, the fault's
 * boundary data, a device FAB3 with lo[1] = hi[1] = domain lo[1] covering
 * grow(valid, 1) & domain in x and z (nbdry comps); else ignored.  F0, F1, F2:
 * optional device FAB3s over the faces of valid in x, y, z (22 comps) that
 * receive the fluxes (for the flux registers).  scheme.precision picks the FP64
 * form or the mixed one (FP32 volume arithmetic; U, friction and boundary data
 * stay FP64).  The intermediates live in the context's scratch, so calls on
 * one context are ordered on one stream; the first call of a context with
 * fault faces creates its second stream and events (make it before any
 * stream capture). */
tmk_status tmk_patch_update_state_3d(tmk_context* ctx, const tmk_fab3* U, const tmk_fab3* B,
                                     const tmk_fab3* F0, const tmk_fab3* F1, const tmk_fab3* F2,
                                     const tmk_box3* valid, const tmk_box3* domain,
                                     double dx, double time, double dt,
                                     double* max_wave_speed, void* stream);

/* The patch loop of LinElastLevelGodunov::step (srcLinElast/LinElastLevelGodunov.cpp:284-333)
 * in a CH_SPACEDIM == 3 build, batched: tmk_patch_update_state_3d on the npatch patches
 * of one level, each pass of the step one launch over all of them (Chombo's
 * 3-D boxes are small: per-patch calls are bound by their launches).  U, valid:
 * arrays of npatch; B: array of npatch (the entries of patches off the fault plane
 * are not read) or NULL when no patch starts on it; F0, F1, F2: arrays of npatch
 * or NULL.  The patches' U must not overlap in their valid boxes (the ghost
 * exchange is the caller's, before the call).  Same results as npatch calls of
 * tmk_patch_update_state_3d. */
tmk_status tmk_patches_update_state_3d(tmk_context* ctx, int npatch, const tmk_fab3* U, const tmk_fab3* B,
                                       const tmk_fab3* F0, const tmk_fab3* F1, const tmk_fab3* F2,
                                       const tmk_box3* valid, const tmk_box3* domain,
                                       double dx, double time, double dt,
                                       double* max_wave_speed, void* stream);

/* LinElastPhysics::plasticUpdate -> PLASTICCORRECTION on a 3-D device FAB over box. */
tmk_status tmk_plastic_update_3d(tmk_context* ctx, const tmk_fab3* U, const tmk_box3* box,
                                 double dt, void* stream);

/* Device-resident level of a CH_SPACEDIM == 3 build (LinElastLevelGodunov::
 * define/step/plasticUpdate, srcLinElast/LinElastLevelGodunov.cpp:45-398,
 * 643-667, with 3-D boxes).  The level owns every patch's FP64 state FAB over
 * its valid box grown by TMK_NGHOST (22 components) and, for the patches that
 * start on the domain's y-lo plane when the scheme has a fault law, the fault
 * data FAB over that box's x-z range on the plane (nbdry components; lo[1] =
 * hi[1] = domain lo[1]).  The valid boxes must lie in the domain and must not
 * overlap (TMK_ERR_BAD_DESC). */
tmk_status tmk_level3d_create(tmk_context* ctx, const tmk_box3* domain, double dx, int npatch,
                              const tmk_box3* patches, tmk_level3d** out);
void       tmk_level3d_destroy(tmk_level3d* lvl);
/* Copy one patch's whole FABs in / out (`host` as for tmk_level_set_patch;
 * B is required on set for a fault patch, ignored for the others). */
tmk_status tmk_level3d_set_patch(tmk_level3d* lvl, int patch, const double* U, const double* B,
                                 int host);
tmk_status tmk_level3d_get_patch(tmk_level3d* lvl, int patch, double* U, double* B, int host);
/* The device FABs of one patch (B zeroed off the fault plane), for callers that
 * read or write them in place on the level's stream. */
tmk_status tmk_level3d_patch_fabs(const tmk_level3d* lvl, int patch, tmk_fab3* U, tmk_fab3* B);
/* Same-level ghost exchange (LevelData::exchange): every ghost cell inside the
 * domain that another patch's valid box covers takes that patch's value, all
 * components; likewise the fault data's ghost faces on the plane. */
tmk_status tmk_level3d_exchange(tmk_level3d* lvl, void* stream);
/* One level step: the exchange, the patch loop as tmk_patches_update_state_3d
 * (one launch per pass over every patch) and, when the scheme has plasticity,
 * tmk_plastic_update_3d on every patch; the kernels are queued on `stream`. */
tmk_status tmk_level3d_step(tmk_level3d* lvl, double time, double dt, double* max_wave_speed,
                            void* stream);

/* ---------------------------------------------------------------------------
 * Device-resident level (LinElastLevelGodunov::define/step/plasticUpdate,
 * srcLinElast/LinElastLevelGodunov.cpp:45-398, 643-667).  The level owns the
 * device mirrors of every patch's U (two buffers, swapped each step) and B.
 * Precision follows scheme->precision: FP64 mirrors, or FP32 volume mirrors
 * with FP64 fault data (mixed form).
 * ------------------------------------------------------------------------- */
tmk_status tmk_level_create(tmk_context* ctx, const tmk_box* domain, double dx,
                            int npatch, const tmk_box* patches, tmk_level** out);
void       tmk_level_destroy(tmk_level* lvl);
/* Per-face rate-and-state friction of one fault patch (an extension: the
 * reference varies only a and Vw along strike, by the linear ramp of RSSETF,
 * ibcLinElast/RSIBCF.ChF:8-55).  abL holds 3 planes (a, b, L) over the patch's
 * fault row grown by TMK_NGHOST in x, laid out like B; `host` as for
 * tmk_level_set_patch.  The face's a replaces the scenario's a (the ramp is still
 * added), b and L replace the scenario's.  Every value must be positive.  Levels
 * of an AMR hierarchy each take their own faces' values. */
tmk_status tmk_level_set_fault_friction(tmk_level* lvl, int patch, const double* abL, int host);
/* The per-face friction of a fault patch, if set (*present = 1; else 0 and
 * abL untouched), in the layout tmk_level_set_fault_friction takes. */
tmk_status tmk_level_get_fault_friction(const tmk_level* lvl, int patch, double* abL, int host,
                                        int* present);
/* Ensemble of independent scenarios stepped as one level (an extension: the
 * reference runs one scenario per process with its parameters in COMMON
 * blocks, srcLinElast/LinElastPhysicsF.ChF:1149-1210, ibcLinElast/RSIBCF.ChF:8-55).
 * Scenario k has context ctxs[k] and problem domain domains[k]; patch p covers
 * boxes[p] of scenario patch_scen[p].  All scenarios share dx and every
 * parameter but friction (material, background stress, scheme, boundary types,
 * plasticity): TMK_ERR_UNSUPPORTED otherwise.  Ghost exchange stays within a
 * scenario; each kernel of a step covers every patch of every scenario.  The
 * result handle takes every tmk_level_* call except the coarse-fine ones
 * (TMK_ERR_UNSUPPORTED); the fault status is ctxs[0]'s. */
tmk_status tmk_ensemble_create(int nscen, tmk_context* const* ctxs, const tmk_box* domains,
                               double dx, int npatch, const tmk_box* boxes,
                               const int* patch_scen, tmk_level** out);
/* Copy one patch's state in / out.  `host` selects host (1) or device (0)
 * pointers.  U covers the valid box grown by TMK_NGHOST, 22 components (FP64);
 * B covers the patch's fault row grown by TMK_NGHOST in x (NULL if none). */
tmk_status tmk_level_set_patch(tmk_level* lvl, int patch, const double* U,
                               const double* B, int host);
tmk_status tmk_level_get_patch(tmk_level* lvl, int patch, double* U, double* B,
                               int host);
/* Copy in / out only what a level step reads and rewrites of one patch: the
 * 18 evolving components (9 per side; on a plastic level also lambda and
 * gamma of both sides) over the valid box, and the fault data B.  U and B are
 * laid out as for tmk_level_set_patch (ghost cells and the other components
 * are not written and their values do not matter); `host` as there.  The
 * counterpart of the reference's step on FABs that live in host memory
 * (LinElastLevelGodunov::step, srcLinElast/LinElastLevelGodunov.H:91-105, reads
 * the valid cells of U and writes them back): put before a step, take after
 * it.  The level must have been given a whole state once (tmk_level_set_patch)
 * so that the components these calls leave alone are defined. */
tmk_status tmk_level_put_valid(tmk_level* lvl, int patch, const double* U,
                               const double* B, int host);
tmk_status tmk_level_take_valid(tmk_level* lvl, int patch, double* U, double* B,
                                int host);
/* One level step at `time` by `dt`: same-level ghost exchange of U and B,
 * fault solve, volume update of every patch in one launch, and (if the
 * scheme has plasticity) the plastic correction.  *dt_new = dx / max wave
 * speed (LinElastLevelGodunov.cpp:377-391).  Graph-capturable: no host sync. */
tmk_status tmk_level_step(tmk_level* lvl, double time, double dt, void* stream,
                          double* dt_new);
/* The full LinElastLevelGodunov::step signature for a level that has a coarser
 * level (LinElastLevelGodunov.H:91-105): the coarse level's old and new times
 * give the time-interpolation coefficient of the coarse-fine ghost fill,
 * alpha = (time - t_coarse_old) / (t_coarse_new - t_coarse_old), snapped to 0 or
 * 1 within 0.04 dt / ratio (LinElastLevelGodunov.cpp:225-256); alpha outside
 * [0, 1] is TMK_ERR_BAD_DESC (the reference's MayDay).  The step also keeps
 * the flux registers with the coarser and finer levels.  tmk_level_step is
 * this call for a level without a coarser level. */
tmk_status tmk_level_step_cf(tmk_level* lvl, double time, double dt, double t_coarse_old,
                             double t_coarse_new, void* stream, double* dt_new);
/* Read and clear the device status word: returns the first recorded error and
 * fills info[0]=code, info[1]=flat index of the first bad value,
 * info[2]=Newton iterations that hit the limit (not an error in the reference). */
tmk_status tmk_level_status(tmk_level* lvl, long long info[3]);
/* Number of kernel launches one tmk_level_step issues. */
int        tmk_level_launches_per_step(const tmk_level* lvl);
/* Per-launch timing of tmk_level_step: with enable=1 the next (at most
 * max_steps) steps record CUDA events on their stream around each launch
 * (the work is unchanged); enable=0 stops recording. */
tmk_status tmk_level_profile(tmk_level* lvl, int enable, int max_steps);
/* Average milliseconds per recorded step of: out[0] ghost exchange,
 * out[1] fault kernel, out[2] volume kernel, out[3] whole step. */
tmk_status tmk_level_profile_read(tmk_level* lvl, double out[4], int* nsteps);
/* The level's tuning; setting it rebuilds the work lists (and the coarse-fine
 * capture lists of an attached level).  TMK_ERR_BAD_DESC for values out of
 * range or while a recorded graph launches the level's kernels. */
tmk_status tmk_level_get_tuning(const tmk_level* lvl, tmk_tuning* out);
tmk_status tmk_level_set_tuning(tmk_level* lvl, const tmk_tuning* t);
/* Autotuner: times `steps` level steps (after 2 untimed ones) from the level's
 * present state for each candidate tuning -- volume kernel, marching waves per
 * group, shortest run, fault displacement and fault segment -- keeps the
 * fastest, and puts the state back as it was.  *best (optional) receives the
 * choice and *ms_per_step (optional) its time.  Synchronous on `stream`.  Not
 * for a level attached to another level (TMK_ERR_BAD_DESC): tune the levels
 * of a hierarchy before attaching them. */
tmk_status tmk_level_autotune(tmk_level* lvl, double time, double dt, int steps, void* stream,
                              tmk_tuning* best, double* ms_per_step);

/* Refinement tags of a level (AMRLevelLinElast::tagCells / tagCellsInit,
 * srcLinElast/AMRLevelLinElast.cpp:577-717, 721-771).  tagCells first fills
 * the level's ghost cells from its coarser level's new state (if attached)
 * and by exchange, then per valid cell takes the largest undivided difference
 * of side 1's velocities in x and y (GETFULLGRADF and MAXF,
 * srcLinElast/LinElastPhysicsF.ChF:59-82, 199-259; one-sided on the domain's
 * edges), sets it to 1 on the fault law's nucleation cells (RSIBC/SWIBC::
 * tagCellsInit, ibcLinElast/RSIBC.cpp:341-377, ibcLinElast/SWIBC.cpp:336-394),
 * and tags it where it reaches the coarsening-scaled threshold or either
 * side's plastic strain reaches plastic_thresh, within the coarsen2 window
 * from level coarsen2_max_level on.  tagCellsInit tags the nucleation cells
 * only.  The tags are grown by tag_buffer cells (IntVectSet::grow) and clipped
 * to the domain.  mask: one byte per cell of the level's domain, x fastest,
 * 1 tagged; `host` selects a host (1) or device (0) pointer.  Synchronous.
 * TMK_ERR_UNSUPPORTED for an ensemble level. */
tmk_status tmk_level_tag_cells(tmk_level* lvl, const tmk_tag_params* p, unsigned char* mask, int host,
                               void* stream);

/* Fault and body stations of a level (AMRLevelLinElast::writeStationLevel,
 * srcLinElast/AMRLevelLinElast.cpp:1758-1869, with the cells and weights of
 * :257-335): a fault station at x reads the fault data of faces i and i+1,
 * i = floor((x + center[0])/dx - 0.5), as B(i)(1-w) + B(i+1)w with the
 * reference's w = x + center[0] - (i + 0.5)dx (a distance, not divided by dx);
 * a body station at (x, y) reads the state of the four cells from (i, j) the
 * same way in both directions.  Each of those cells is read from the patch
 * that holds it (the reference reads the station patch's ghost cells).  A
 * record is the time, then nb values per fault station, then 22 per body
 * station, NaN for a station no patch of the level holds; `capacity` records
 * are kept on the device until read.  Destroy the stations before their level. */
tmk_status tmk_stations_create(tmk_level* lvl, int nfault, const double* x_fault, int nbody,
                               const double* x_body, const double* y_body, const double center[2],
                               int capacity, tmk_stations** out);
void       tmk_stations_destroy(tmk_stations* st);
/* One record at `time` (asynchronous on `stream`, graph-capturable). */
tmk_status tmk_stations_record(tmk_stations* st, double time, void* stream);
/* Values per record (1 + values of every station) and, per station, whether a
 * patch of the level holds it. */
tmk_status tmk_stations_layout(const tmk_stations* st, int* values_per_record, int* present);
/* Copy out (at most max_records) records made since the last read and start
 * over; *dropped = records lost to a full buffer or to max_records. */
tmk_status tmk_stations_read(tmk_stations* st, double* out, int max_records, int* nrec,
                             long long* dropped);
/* Record `st` at the end of every step of its level, at the level's new time,
 * after the finer levels' substeps, reflux and average-down when the level is
 * in a hierarchy (postTimeStep's order); st = NULL stops. */
tmk_status tmk_level_attach_stations(tmk_level* lvl, tmk_stations* st);

/* ---------------------------------------------------------------------------
 * Coarse-fine coupling (AMRLevelLinElast::levelSetup,
 * srcLinElast/AMRLevelLinElast.cpp:1960-2050).  A fine level is attached to the
 * next coarser level with the refinement ratio between them; the fine domain
 * must be the refined coarse domain, every fine patch aligned to the ratio, and
 * the fine level properly nested (each coarse cell an operator reads is a valid
 * cell of the coarse level), else TMK_ERR_BAD_DESC.  Attaching replaces an
 * earlier attachment of either level.  Both levels must use the same precision
 * and fault law.  The volume update of an attached level also stores the
 * fluxes of its coarse-fine faces for the flux registers.
 * ------------------------------------------------------------------------- */
tmk_status tmk_level_attach_coarser(tmk_level* fine, tmk_level* coarse, int ref_ratio);
tmk_status tmk_level_detach_coarser(tmk_level* fine);
/* Coarse-fine ghost fill of the fine level's current state from the coarse
 * level's state before (old) and after (new) its last step, at time
 * coefficient alpha: PiecewiseLinearFillPatch::fillInterp for U (radius
 * TMK_NGHOST) and D1PiecewiseLinearFillPatch::fillInterp for the fault rows
 * (srcLinElast/D1PiecewiseLinearFillPatch.cpp:276-324).  tmk_level_step_cf
 * performs it; this entry point exposes it alone. */
tmk_status tmk_level_fill_coarse_fine(tmk_level* fine, double alpha, void* stream);
/* LevelFluxRegister::reflux(U, -1/dx) of the coarse level with the fluxes its
 * finer level accumulated since the coarse level's last step
 * (srcLinElast/AMRLevelLinElast.cpp:505-506). */
tmk_status tmk_level_reflux(tmk_level* coarse, void* stream);
/* CoarseAverage (U) and D1CoarseAverage (fault rows) of the finer level onto
 * the coarse level (srcLinElast/AMRLevelLinElast.cpp:508-515,
 * srcLinElast/D1CoarseAverage.cpp:62-139). */
tmk_status tmk_level_average_down(tmk_level* coarse, void* stream);
/* Regrid prolongation: FineInterp (U) and D1FineInterp (fault rows) of the
 * coarse level onto every valid cell of the fine level
 * (srcLinElast/AMRLevelLinElast.cpp:927-931, srcLinElast/D1FineInterp.cpp:61-267). */
tmk_status tmk_level_interp_from_coarser(tmk_level* fine, void* stream);
/* Copy the valid cells (U and fault rows) where the patches of two levels of
 * the same domain overlap: the "copy from old state" of a regrid
 * (srcLinElast/AMRLevelLinElast.cpp:934-946). */
tmk_status tmk_level_copy_overlap(tmk_level* dst, const tmk_level* src, void* stream);
/* Number of coarse-fine faces in the flux register of an attached fine level. */
tmk_status tmk_level_register_size(const tmk_level* fine, int* entries);

/* ---------------------------------------------------------------------------
 * Subcycled AMR hierarchy (Chombo AMR::timeStep over AMRLevelLinElast::advance
 * and postTimeStep, srcLinElast/AMRLevelLinElast.cpp:420-515).  The caller owns
 * the levels; creating the hierarchy attaches level l+1 to level l with
 * ratios[l].  One tmk_amr_step advances level 0 by dt0 and level l by
 * dt0 / (ratios[0] ... ratios[l-1]), each finer level taking ratio substeps per
 * step of its coarser level, then refluxes and averages down.  No host sync.
 * ------------------------------------------------------------------------- */
tmk_status tmk_amr_create(int nlevels, tmk_level* const* levels, const int* ratios, double time,
                          tmk_amr** out);
void       tmk_amr_destroy(tmk_amr* amr);
tmk_status tmk_amr_step(tmk_amr* amr, double dt0, void* stream);
/* Hierarchy autotuner: for each level, finest first, times every candidate
 * tuning (as tmk_level_autotune, runs of 16 or 32 rows) over `ncoarse` whole
 * subcycled coarse steps after one untimed one, keeps the fastest, and puts
 * the hierarchy's state and clock back as they were.  per_level (optional,
 * one entry per level) receives the choices, *ms_per_coarse_step (optional)
 * the final time.  Synchronous on `stream`; TMK_ERR_BAD_DESC while a recorded
 * graph launches the hierarchy's kernels. */
tmk_status tmk_amr_autotune(tmk_amr* amr, double dt0, int ncoarse, void* stream, tmk_tuning* per_level,
                            double* ms_per_coarse_step);
tmk_status tmk_amr_time(const tmk_amr* amr, int level, double* time);
/* Cell-updates of one tmk_amr_step: sum over levels of valid cells x substeps. */
long long  tmk_amr_cell_updates(const tmk_amr* amr);
/* Kernel launches of one tmk_amr_step. */
int        tmk_amr_launches_per_step(const tmk_amr* amr);

/* ---------------------------------------------------------------------------
 * CUDA graphs of whole steps.  tmk_level_graph_create records `nsteps` (even)
 * steps of a level without a coarser level, starting at `time` by `dt`;
 * tmk_amr_graph_create records `ncoarse` (even) subcycled coarse steps of a
 * hierarchy by `dt0` from its current time.  Recording runs nothing.
 * tmk_graph_launch replays the steps on `stream` starting at `time` (the start
 * times of the recorded fault solves are shifted accordingly) and, for a
 * hierarchy, advances its clock.  The recorded steps keep the level layout,
 * attachments and dt of the recording: rebuild the graph after a regrid.
 * ------------------------------------------------------------------------- */
tmk_status tmk_level_graph_create(tmk_level* lvl, int nsteps, double time, double dt, tmk_graph** out);
tmk_status tmk_amr_graph_create(tmk_amr* amr, int ncoarse, double dt0, tmk_graph** out);
tmk_status tmk_graph_launch(tmk_graph* graph, double time, void* stream);
void       tmk_graph_destroy(tmk_graph* graph);

#ifdef __cplusplus
}
#endif
#endif /* TETEMOKO_GB300_H */
