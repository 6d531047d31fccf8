/*
 * swgb300 -- GB300-native backend for the finite-difference time-stepping hot
 * path of SeismicWaves.jl (acoustic constant-density C-PML, 2D and 3D, and the
 * isotropic elastic 2D (P-SV) C-PML path).
 *
 * Plain C ABI: no C++ types, no exceptions, no torch types.  Every entry point
 * returns an int status (SW_OK on success); the text of the last error of a
 * context is available from sw_ctx_last_error().
 *
 * Array conventions follow the reference's Julia structures: all grids are
 * column-major with axis 0 fastest (x), the last axis is depth, indices are
 * 1-based; traces are (nt, nrec) column-major with time fastest; positions are
 * (npos, ndim) column-major.  Unless a call takes an `on_device` flag set to
 * 1, every pointer is a host pointer and the call copies in and out.  With
 * on_device = 1 the bulk arrays (vp, srctf, traces, observed, invcov_diag, invcov,
 * grad, misfit) are device pointers; the small tables (grid indices, C-PML
 * coefficients, windows, positions) are always host memory.
 *
 * Where each entry point sits in the reference (SeismicWaves.jl v0.9.0, paths
 * relative to its source tree):
 *
 *   sw_ctx_create / sw_ctx_destroy
 *       the backend module a package extension returns from select_backend
 *       (ext/SeismicWaves_CUDABackendExt.jl:13-25, src/models/backend_selection.jl:2-40)
 *   sw_cpml_coefficients
 *       compute_CPML_coefficientsAxis! + the free-top override
 *       (src/models/cpmlcoeffs.jl:18-100, src/models/acoustic/acou_init_bc.jl:7-40)
 *   sw_wavesim_create / sw_wavesim_destroy
 *       build_wavesim -> AcousticCDCPMLWaveSimulation (src/apis/build.jl:18-40,
 *       src/models/acoustic/acou_models.jl:90-202): preallocated device fields
 *   sw_wavesim_set_vp, sw_wavesim_set_vp64
 *       set_wavesim_matprop! -> update_matprop! -> precompute_fact!
 *       (src/apis/utils.jl:3-8, src/models/acoustic/acou_models.jl:53-60)
 *   sw_acoustic_forward
 *       run_swforward! shot loop + swforward_1shot! time loop + forward_onestep_CPML!
 *       (src/apis/forward.jl:71-114, src/models/acoustic/acou_forward.jl:22-62,
 *       src/models/acoustic/backends/shared/acoustic2D_xPU.jl:78-126, acoustic3D_xPU.jl:96-160);
 *       all shots of the call advance together in one launch per time step
 *   sw_acoustic_gradient
 *       run_swgradient! + swgradient_1shot! (CD) with LinearCheckpointer, L2 misfit,
 *       prescale_residuals!, adjoint_onestep_CPML!, correlate_gradient!, muting and
 *       the 2/vp^3 rescaling (src/apis/gradient.jl:93-136,
 *       src/models/acoustic/acou_gradient.jl:4-95, src/utils/checkpointers.jl:1-107,
 *       src/inversion/misfits/L2Misfit.jl:24-77, acoustic2D_xPU.jl:64-76 and :128-169,
 *       correlate_gradient_xPU.jl:1-10, src/utils/mute_grad.jl:13-80)
 *   sw_acoustic_vd_create / sw_acoustic_vd_destroy
 *       build_wavesim -> AcousticVDStaggeredCPMLWaveSimulation (src/apis/build.jl:60-72,
 *       src/models/acoustic/acou_models.jl:311-454)
 *   sw_acoustic_vd_set_material, sw_acoustic_vd_set_material64
 *       update_matprop! -> precompute_fact! (acou_models.jl:283-300)
 *   sw_acoustic_vd_forward
 *       run_swforward! + swforward_1shot! (VD) + forward_onestep_CPML!
 *       (src/models/acoustic/acou_forward.jl:83-125,
 *       src/models/acoustic/backends/shared/acoustic2D_VD_xPU.jl:1-125)
 *   sw_acoustic_vd_gradient
 *       run_swgradient! + swgradient_1shot! (VD) with LinearCheckpointer, L2 misfit,
 *       prescale_residuals!, adjoint_onestep_CPML!, correlate_gradient_m0! /
 *       correlate_gradient_m1!, back_interp, muting and the vp / rho chain rule
 *       (src/models/acoustic/acou_gradient.jl:97-202, acoustic2D_VD_xPU.jl:64-192,
 *       src/models/acoustic/backends/shared/correlate_gradient_xPU.jl:12-21)
 *   sw_elastic_create / sw_elastic_destroy
 *       build_wavesim -> ElasticIsoCPMLWaveSimulation (src/models/elastic/ela_models.jl:177-420)
 *   sw_elastic_set_material
 *       update_matprop! -> precomp_elaprop! with the half-point interpolations
 *       (ela_models.jl:143-173, src/utils/interpolations.jl:1-47)
 *   sw_elastic_forward
 *       run_swforward! shot loop + swforward_1shot! (moment-tensor and external-force shots)
 *       + forward_onestep_CPML! (src/models/elastic/ela_forward.jl:4-159,
 *       src/models/elastic/backends/shared/elastic2D_iso_xPU.jl:1-357)
 *   sw_elastic_gradient
 *       run_swgradient! + swgradient_1shot! (elastic) with LinearCheckpointer, L2 misfit,
 *       adjoint_onestep_CPML!, correlate_gradients!, back-interpolation and muting
 *       (src/models/elastic/ela_gradient.jl:4-362, elastic2D_iso_xPU.jl:359-448,
 *       src/models/elastic/backends/shared/correlate_gradient_xPU.jl:1-83,
 *       src/inversion/misfits/L2Misfit.jl:44-95)
 */
#ifndef SWGB300_H
#define SWGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SW_OK = 0,
  SW_ERR_ARG = 1,         /* invalid argument (the reference's @assert / error) */
  SW_ERR_OOM = 2,         /* device allocation failed */
  SW_ERR_CUDA = 3,        /* CUDA runtime error */
  SW_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  SW_ERR_STATE = 5,       /* call made in the wrong state (e.g. gradient on a forward-only wavesim) */
  SW_ERR_UNSUPPORTED = 6, /* input the backend deliberately rejects (see sw_ctx_last_error) */
  SW_ERR_CAPACITY = 7     /* problem larger than the fixed scratch of sw_acoustic2d_forward_noalloc */
};

typedef struct sw_ctx sw_ctx;
typedef struct sw_wavesim sw_wavesim;
typedef struct sw_elastic sw_elastic;
typedef struct sw_acoustic_vd sw_acoustic_vd;

/* Library version (major*10000 + minor*100 + patch). */
int sw_version(void);

/* One context per device; `stream` is a cudaStream_t to launch on, or NULL
 * for a stream owned by the context.  A context is used by one host thread. */
int sw_ctx_create(int device, void* stream, sw_ctx** out);
int sw_ctx_destroy(sw_ctx* ctx);
const char* sw_ctx_last_error(const sw_ctx* ctx);
/* The stream the context launches on (cudaStream_t). */
void* sw_ctx_stream(const sw_ctx* ctx);

/* InputParametersAcoustic{T,N} + CPMLBoundaryConditionParameters{T}. */
typedef struct {
  int32_t ndim;      /* 2 or 3 */
  int32_t n[3];      /* grid points per axis (axis 0 fastest; last axis = depth) */
  double h[3];       /* grid spacing per axis [m] */
  double dt;         /* time step [s] */
  int32_t halo;      /* C-PML thickness in grid points (>= 0) */
  double rcoef;      /* target reflection coefficient */
  int32_t freetop;   /* 1: free surface at index 1 of the last axis */
} sw_acoustic_params;

/* C-PML coefficients of one axis, as compute_CPML_coefficientsAxis! returns
 * them: a and b have 2*(halo+1) entries, a_h and b_h 2*halo entries.
 * freetop_axis = 1 applies the free-surface override of the first half. */
int sw_cpml_coefficients(double vel_max, double dt, int32_t halo, double rcoef, double h, double f0,
                         int32_t freetop_axis, float* a, float* a_h, float* b, float* b_h);
/* The same coefficients in FP64 (sw_acoustic_shot.cpml64 of the compensated forward). */
int sw_cpml_coefficients64(double vel_max, double dt, int32_t halo, double rcoef, double h, double f0,
                           int32_t freetop_axis, double* a, double* a_h, double* b, double* b_h);

/* One shot (ScalarShot) as possrcrec_scaletf hands it to the backend:
 * nearest-grid-point indices and the scaled source time functions. */
typedef struct {
  int32_t nt;               /* time steps of this shot (may differ between shots) */
  int32_t nsrc;
  const int32_t* src_idx;   /* (nsrc, ndim), 1-based grid indices */
  const float* srctf;       /* (nt, nsrc), already scaled by dt^2 vp(src)^2 / prod(h) */
  int32_t nrec;
  const int32_t* rec_idx;   /* (nrec, ndim), 1-based grid indices */
  float* traces;            /* (nt, nrec) output: pressure after injection, every step */
  const float* cpml;        /* ndim blocks [a, a_h, b, b_h] of this shot's C-PML coefficients */
  /* used by sw_acoustic_gradient only */
  const float* observed;    /* (nt, nrec) observed data of the L2 misfit */
  const float* invcov_diag; /* NULL: identity inverse covariance; else its diagonal (nt) */
  int32_t nwin;             /* number of time windows (0 = whole trace) */
  const int32_t* windows;   /* (2, nwin): 1-based inclusive [first, last] pairs (host memory) */
  const double* src_pos;    /* (nsrc, ndim) metres, muting only (host memory) */
  const double* rec_pos;    /* (nrec, ndim) metres, muting only (host memory) */
  const float* invcov;      /* gradient: NULL, or the full inverse covariance (nt, nt) column-major
                               (L2Misfit.invcov as a dense matrix); takes precedence over invcov_diag */
  int32_t misfit_kind;      /* gradient: 0 = L2Misfit, 1 = CCTSMisfit (src/inversion/misfits/CCTSMisfit.jl:17-61;
                               windows and inverse covariances are then unused, nt <= 13000) */
  double misfit_dt;         /* CCTSMisfit.dt (misfit_kind 1) */
  const double* cpml64;     /* NULL, or the cpml coefficients in FP64 (host memory): the compensated forward
                               (sw_wavesim_set_precision 1) evaluates the C-PML strips with them */
} sw_acoustic_shot;

/* GradParameters. */
typedef struct {
  int32_t check_freq;       /* checkpoint period K (>= 1, < nt of every shot) */
  int32_t mute_radius_src;  /* grid points; 0 = off */
  int32_t mute_radius_rec;
  int32_t compute_misfit;
  int32_t snapshot_bf16;    /* 0: FP32 snapshots; 1: the recompute buffer (the second time differences
                               kept between checkpoints) in BF16; 2: also the checkpoints' (p, d) in
                               per-snapshot-scaled BF16; 3 (3D only): the recompute buffer in FP16 with
                               a power-of-two scale per row and 128-point x tile (8x BF16's precision
                               in the same 2 bytes, plus one byte per 128 points).  Acoustic path. */
} sw_grad_params;

/* build_wavesim.  `gradient` = 1 allows sw_acoustic_gradient.  Device memory
 * for the shots is allocated at the first call that needs it and reused. */
int sw_wavesim_create(sw_ctx* ctx, const sw_acoustic_params* params, int32_t gradient,
                      const sw_grad_params* gparams, sw_wavesim** out);
int sw_wavesim_destroy(sw_wavesim* ws);

/* set_wavesim_matprop!: vp has prod(n) entries (column-major). */
int sw_wavesim_set_vp(sw_wavesim* ws, const float* vp, int32_t on_device);

/* set_wavesim_matprop! with a Float64 model (the reference's arrays): fact =
 * vp^2 dt^2 is formed from the FP64 values, so the compensated forward of
 * sw_wavesim_set_precision keeps its full precision; the stencils that take
 * vp itself use its FP32 rounding.  The FP64 model stays on the device until
 * sw_wavesim_set_vp replaces it. */
int sw_wavesim_set_vp64(sw_wavesim* ws, const double* vp, int32_t on_device);

/* run_swforward!: all shots advance together (shots that do not fit in device
 * memory at once run in consecutive groups). */
int sw_acoustic_forward(sw_wavesim* ws, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device);

/* run_swgradient! with the L2 misfit: grad (prod(n) entries, float64) is the
 * sum over shots of each shot's muted, 2/vp^3-rescaled gradient; misfit
 * (may be NULL) receives the sum of the shots' misfits.  Traces are written
 * to each shot's `traces`. */
int sw_acoustic_gradient(sw_wavesim* ws, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device,
                         double* grad, double* misfit);

/* sw_acoustic_forward with snapshots (RunParameters.snapevery): after every
 * time step it with it % snapevery == 0 the pressure field p[it] of each shot
 * is copied (unpadded, column-major, prod(n) floats) into snapshots[k] +
 * (it/snapevery - 1) * prod(n); snapshots[k] (host or device memory) holds
 * floor(nt_k / snapevery) fields.  Replaces LinearSnapshotter + savesnapshot!
 * in swforward_1shot! (src/utils/snapshotter.jl:1-41,
 * src/models/acoustic/acou_forward.jl:54-57).  snapevery < nt as the reference asserts. */
int sw_acoustic_forward_snapshots(sw_wavesim* ws, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device,
                                  int32_t snapevery, float* const* snapshots);

/* Stencil tuning knobs used by the autotuner: tz = height (in planes of the
 * marching axis) of a block's tile, 0 = built-in heuristic; variant selects
 * the 2D stencil implementation: 0, 2, 3 = register-pipelined loads with 4,
 * 8 or 16 warps per block, 1 = TMA bulk copies through shared memory with a
 * producer warp; + 4 keeps a second row of loads in flight in the forward
 * kernels of the 4-warp stencil; + 8 runs the grouped 2D adjoint (4+ shots)
 * with 5 resident blocks per SM instead of 4 (registers capped at 102; with + 256);
 * + 16*k additionally prefetches the rows k rows ahead into L2 (k = 1..15);
 * by default the 2D adjoint runs per shot with plain FP32 correlation sums
 * flushed into an FP64 total every 32 steps; + 256 selects instead the grouped
 * adjoint (4 shots per block, one Kahan-compensated FP32 sum per group; 4+
 * shots); + 512 stages the rows of the 4-warp stencil through a per-warp
 * shared-memory ring filled by cp.async (three rows in flight per warp
 * instead of one, no registers held by the copies).  + 1024 makes the 2D
 * forward kinds (forward, recompute) and the adjoint advance two time steps
 * per launch wherever nothing happens between the steps (temporal blocking,
 * the same rounding as two one-step launches); bits 11-13 pick the rows per
 * block of that kernel (0 = heuristic: 32, fewer for small batches; 1 = 8,
 * 2 = 16, 3 = 32, 4 = 64, 5 = 128, 6 = 4) and bits 14-15 its resident-block
 * bound (0 = 6 forward / 5 adjoint blocks per SM, 1 = 4 / 3, 2 = 7 / 4).
 * 3D: + 65536 runs the step as one launch instead of three (rows outside the
 * y / z strips, the z slabs, the y slabs); + 131072 runs the three launches
 * without the software pipeline.  2D, 4 warps per block: by default the
 * 4-point lane groups that meet an x strip are advanced by extra blocks at the
 * end of the stencil launch, one group per thread (the main blocks skip
 * them); + 262144 keeps them in the main blocks' per-point C-PML path.
 * Results do not depend on any of them beyond rounding. */
int sw_wavesim_set_tuning(sw_wavesim* ws, int32_t tz, int32_t variant);

/* Band height (rows per block along the marching axis) of the one-step
 * stencil per kind: the forward (and the forward of the gradient), the
 * recompute of the gradient's adjoint phase, and the adjoint; 0 = the tz of
 * sw_wavesim_set_tuning (or its heuristic).  Lets an autotuner pick each
 * kind's band from that kind's own timing; results do not change.  No
 * reference counterpart. */
int sw_wavesim_set_band_heights(sw_wavesim* ws, int32_t tz_forward, int32_t tz_recompute, int32_t tz_adjoint);

/* Arithmetic of the forward passes (sw_acoustic_forward and the forward of
 * sw_acoustic_gradient), 2D and 3D: 0 = FP32 state (default); 1 =
 * compensated: p and d held as unevaluated sums of two FP32 numbers, fact =
 * vp^2 dt^2 and 1/h^2 as FP32 pairs of their FP64 values, the second
 * differences, the increment and both state updates evaluated with
 * error-free transformations (about 48 significant bits; the C-PML memory
 * variables stay FP32).  Traces and misfits then agree with an FP64
 * simulation to ~1e-7 at several thousand steps, where FP32 state drifts to
 * ~1e-6; the forward takes about twice the bytes and several times the
 * arithmetic.  The gradient's recompute and adjoint stay FP32 (they start
 * from checkpoints rounded to FP32).  No reference counterpart: the
 * reference runs in the precision of its arrays (Float64 on the CPU). */
int sw_wavesim_set_precision(sw_wavesim* ws, int32_t mode);

/* Bounded waits of the TMA stencil (tuning variant 1): every mbarrier wait
 * gives up after wait_cycles SM clock cycles (default 4e9, about 2 s), sets
 * the context's error flag and leaves; the call then returns SW_ERR_TIMEOUT
 * and the context stays usable.  withhold_stage >= 0 is a test hook: the
 * producer warp of the launch's first block stops before issuing that stage
 * of its row pipeline, so the consumers' wait on it runs out (nothing is in
 * flight when they leave); -1 = off.  No reference counterpart. */
int sw_wavesim_set_wait_test(sw_wavesim* ws, int64_t wait_cycles, int32_t withhold_stage);

/* CUDA graphs (on by default): a batch's whole device-side time loop
 * (forward; for the gradient also misfit, adjoint and shot sum) is captured
 * into a graph on the second call with the same batch layout and replayed on
 * later calls.  No reference counterpart (the reference launches every kernel
 * from its time loop).  on = 0 launches directly. */
int sw_wavesim_use_graphs(sw_wavesim* ws, int32_t on);

/* Per-kernel timing collected with CUDA events on the context's stream while
 * enabled (0 = off).  kind: 0 = forward stencil, 1 = adjoint stencil (with the
 * correlation on the acoustic path), 2 = source/receiver kernels, 3 = other,
 * 4 = recompute stencil of the gradient, 5 = elastic gradient correlation;
 * bytes = algorithmic bytes. */
int sw_profile_enable(sw_ctx* ctx, int32_t on);
int sw_profile_read(sw_ctx* ctx, int32_t kind, double* total_ms, int64_t* launches, double* bytes);
/* Kernel launches inside the brackets that sw_profile_read counts as
 * `launches` (one bracket per step of a kind; the 3D step as three launches,
 * the variable-density adjoint pair and the elastic displacement pair launch
 * several kernels). */
int sw_profile_read_kernels(sw_ctx* ctx, int32_t kind, int64_t* kernels);

/* ---------------------------------------------------------------------------
 * Isotropic elastic 2D (P-SV), 4th-order staggered displacement-stress scheme
 * with C-PML.  Grids follow ElasticIsoCPMLWaveSimulation: sigma_xx, sigma_zz,
 * lambda, mu, rho on (nx, nz) nodes; ux on (nx-1, nz); uz on (nx, nz-1);
 * sigma_xz on (nx-1, nz-1).  Traces are (nt, 2, nrec) column-major (ux, uz).
 * ------------------------------------------------------------------------- */
typedef struct {
  int32_t n[2];       /* nx, nz */
  double h[2];        /* dx, dz */
  double dt;
  int32_t halo;
  double rcoef;
  int32_t freetop;    /* free surface at the top (mirror conditions, sigma_zz = 0 at j = 1) */
  int32_t interp_rho; /* rho at half points: 0 = arithmetic average (reference default), 1 = harmonic */
  int32_t interp_mu;  /* mu at (i+1/2, j+1/2): 0 = arithmetic (reference default), 1 = harmonic */
} sw_elastic_params;

/* Grid points of one table, grouped by item (a source or a receiver): item k
 * owns entries offsets[k] .. offsets[k+1]-1; entry e is grid point
 * (ij[2e], ij[2e+1]) (1-based, on the table's own grid) with weight coef[e].
 * This is the output of spread_positions (src/utils/utils.jl:168-214) or, with
 * sincinterp = false, one nearest point of weight 1 per item
 * (ela_models.jl:6-90). */
typedef struct {
  const int32_t* offsets; /* count+1 entries */
  const int32_t* ij;
  const float* coef;
} sw_point_table;

typedef struct {
  int32_t nt;
  int32_t kind;            /* 0 = MomentTensorShot, 1 = ExternalForceShot */
  int32_t nsrc;
  const float* srctf;      /* kind 0: (nt, nsrc); kind 1: (nt, 2, nsrc); divided by dx*dz as possrcrec_scaletf does */
  const float* momtens;    /* kind 0: (3, nsrc) = Mxx, Mzz, Mxz of each source; host memory */
  sw_point_table src[2];   /* kind 0: [sigma_xx/sigma_zz nodes, sigma_xz nodes]; kind 1: [ux nodes, uz nodes] */
  int32_t nrec;
  sw_point_table rec[2];   /* [ux nodes, uz nodes] */
  float* traces;           /* (nt, 2, nrec) output */
  const float* cpml;       /* C-PML coefficients, axis x then z, each [a, a_h, b, b_h] (init_bdc!,
                              src/models/elastic/ela_init_bc.jl:7-40) */
  const float* observed;   /* gradient: observed traces (nt, 2, nrec) */
  const float* invcov_diag;/* gradient: NULL (identity) or the diagonal of the inverse covariance (nt) */
  int32_t nwin;
  const int32_t* windows;  /* (2, nwin) 1-based inclusive time windows; host memory */
  const double* src_pos;   /* (nsrc, 2) metres, for muting; host memory */
  const double* rec_pos;   /* (nrec, 2) metres, for muting; host memory */
  const float* invcov;     /* gradient: NULL, or the full inverse covariance (nt, nt) column-major, applied to
                              each component; takes precedence over invcov_diag */
  int32_t misfit_kind;      /* gradient: 0 = L2Misfit, 1 = CCTSMisfit per component trace
                               (src/inversion/misfits/CCTSMisfit.jl:30-44, :63-80; windows and inverse
                               covariances are then unused, nt <= 13000) */
  double misfit_dt;         /* CCTSMisfit.dt (misfit_kind 1) */
} sw_elastic_shot;

/* One elastic simulation (a set of preallocated device fields).  gradient = 1
 * also prepares the adjoint fields and the checkpointing (gparams as for the
 * acoustic path; snapshot_bf16 must be 0). */
int sw_elastic_create(sw_ctx* ctx, const sw_elastic_params* params, int32_t gradient, const sw_grad_params* gparams,
                      sw_elastic** out);
int sw_elastic_destroy(sw_elastic* es);
/* lambda, mu, rho: host arrays of (nx, nz) floats (check_matprop's conditions apply). */
int sw_elastic_set_material(sw_elastic* es, const float* lambda, const float* mu, const float* rho);
/* Forward modelling of nshots shots in one batch; traces written per shot.
 * on_device = 1: srctf and traces are device pointers. */
int sw_elastic_forward(sw_elastic* es, int32_t nshots, const sw_elastic_shot* shots, int32_t on_device);
/* Gradient of the summed L2 misfit with respect to rho, lambda and mu, each
 * (nx, nz) FP64, summed over the shots; misfit (may be NULL) = sum of the shots'
 * misfits.  on_device = 1: srctf, traces, observed, invcov_diag and the
 * outputs are device pointers. */
int sw_elastic_gradient(sw_elastic* es, int32_t nshots, const sw_elastic_shot* shots, int32_t on_device,
                        double* grad_rho, double* grad_lambda, double* grad_mu, double* misfit);
/* sw_elastic_forward with snapshots (RunParameters.snapevery): after every
 * step it with it % snapevery == 0, each shot's ucur and sigma fields are
 * copied into snapshots[k] + (it/snapevery - 1) * B as one block of
 * B = (nx-1)nz + nx(nz-1) + 2 nx nz + (nx-1)(nz-1) floats: ux (nx-1, nz),
 * uz (nx, nz-1), sigma_xx, sigma_zz (nx, nz), sigma_xz (nx-1, nz-1), each
 * column-major.  Replaces savesnapshot! in swforward_1shot!
 * (src/models/elastic/ela_forward.jl:74-78, src/utils/snapshotter.jl:1-41). */
int sw_elastic_forward_snapshots(sw_elastic* es, int32_t nshots, const sw_elastic_shot* shots, int32_t on_device,
                                 int32_t snapevery, float* const* snapshots);

/* Rows per thread block of the elastic stencil kernels: 8, 16 or 32 (0 =
 * default 8); + 64 selects the one-point-per-thread kernels instead of the
 * four-points-per-thread ones.  The four-point displacement update runs as
 * two launches (ux, then uz; 72 registers each, 7 resident blocks per SM,
 * 5 % faster than one launch of both at 96); + 128 selects the single
 * launch.  A tuning knob of this backend; no reference counterpart. */
int sw_elastic_set_tuning(sw_elastic* es, int32_t tz);

/* ---------------------------------------------------------------------------
 * Variable-density acoustic 2D, 4th-order staggered pressure-velocity scheme
 * with C-PML (AcousticVDStaggeredCPMLWaveSimulation).  p, vp and rho live on
 * the (nx, nz) nodes, vx on (nx-1, nz), vz on (nx, nz-1).  Shots use
 * sw_acoustic_shot, with srctf already scaled by dt vp(src)^2 rho(src) /
 * (dx dz) as possrcrec_scaletf does for this simulation
 * (src/models/acoustic/acou_forward.jl:66-80).
 * ------------------------------------------------------------------------- */
/* params->ndim must be 2.  interp_rho: 1/rho at the half points, 0 =
 * arithmetic average (the reference's default), 1 = harmonic.  gradient = 1
 * prepares the adjoint fields and the checkpointing (gparams as for the
 * constant-density path; snapshot_bf16 must be 0). */
int sw_acoustic_vd_create(sw_ctx* ctx, const sw_acoustic_params* params, int32_t interp_rho, int32_t gradient,
                          const sw_grad_params* gparams, sw_acoustic_vd** out);
int sw_acoustic_vd_destroy(sw_acoustic_vd* vd);
/* vp, rho: host arrays of (nx, nz) floats (check_matprop's conditions apply). */
int sw_acoustic_vd_set_material(sw_acoustic_vd* vd, const float* vp, const float* rho);
/* Forward modelling of nshots shots in one batch; traces (pressure after
 * injection) written per shot.  on_device = 1: srctf and traces are device pointers. */
int sw_acoustic_vd_forward(sw_acoustic_vd* vd, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device);
/* sw_acoustic_vd_forward with snapshots: after every step it with
 * it % snapevery == 0, each shot's pcur and vcur are copied into
 * snapshots[k] + (it/snapevery - 1) * B as one block of B = nx nz + (nx-1) nz
 * + nx (nz-1) floats: p (nx, nz), vx (nx-1, nz), vz (nx, nz-1), each
 * column-major (savesnapshot! in acou_forward.jl:118-121). */
int sw_acoustic_vd_forward_snapshots(sw_acoustic_vd* vd, int32_t nshots, const sw_acoustic_shot* shots,
                                     int32_t on_device, int32_t snapevery, float* const* snapshots);
/* Gradient of the summed L2 misfit with respect to vp and rho, each (nx, nz)
 * FP64 summed over the shots, with the reference's sign convention; misfit
 * (may be NULL) = sum of the shots' misfits.  on_device = 1: srctf, traces,
 * observed, invcov_diag, invcov and the outputs are device pointers. */
int sw_acoustic_vd_gradient(sw_acoustic_vd* vd, int32_t nshots, const sw_acoustic_shot* shots, int32_t on_device,
                            double* grad_vp, double* grad_rho, double* misfit);
/* Rows per thread block of the VD stencil kernels: 8, 16 or 32 (0 = default
 * 8).  A tuning knob of this backend; results do not depend on it. */
int sw_acoustic_vd_set_tuning(sw_acoustic_vd* vd, int32_t tz);

/* Compensated forward of the variable-density path (mode 1; 0 = FP32, the
 * default): p, vx and vz as unevaluated sums of two FP32 numbers, fact_m0 /
 * fact_m1 and 1/dx, 1/dz as FP32 pairs of their FP64 values, the staggered
 * differences and both updates in double-FP32, the C-PML memory variables
 * and coefficients (sw_acoustic_shot.cpml64, or the FP32 ones widened) in
 * FP64.  The gradient's recompute and adjoint stay FP32.  No reference
 * counterpart (the reference runs in the precision of its arrays). */
int sw_acoustic_vd_set_precision(sw_acoustic_vd* vd, int32_t mode);

/* sw_acoustic_vd_set_material with Float64 arrays (host memory): the
 * material factors are formed from the FP64 values, so the compensated
 * forward keeps their full precision. */
int sw_acoustic_vd_set_material64(sw_acoustic_vd* vd, const double* vp, const double* rho);

/* 2D forward of one shot that allocates no device memory.  Has no
 * counterpart in the reference: it exists for callers that cannot let a
 * library call cudaMalloc -- code running inside another runtime's device
 * memory pool (CUDA.jl, PyTorch) that must account for every byte, fixed
 * device-memory budgets, and pipelines that cannot take the device-wide
 * synchronisation cudaMalloc/cudaFree may impose.  Its wavefields, memory
 * variables and shot tables live in a fixed 64 MiB device array inside the
 * library (every GPU that loads the library holds it until exit), enough for
 * grids up to about 3.5 million points; larger problems return
 * SW_ERR_CAPACITY.  vp (prod(n) floats), shot->srctf and shot->traces are
 * device pointers; the index tables and shot->cpml are host memory.  Work is
 * issued on `stream` (cudaStream_t, NULL = legacy default stream) and the call
 * returns after it finished.  Every call reuses the same array and clears
 * what must start at zero itself; calls whose GPU work overlaps race on it.
 * The first call on a device looks the array up (cudaGetSymbolAddress, with
 * that device current), so make it before any stream capture; the address is
 * cached per device ordinal for the device's primary context, so do not call
 * it after a cudaDeviceReset or under another context of that device.  Status
 * codes only (no context, no message). */
int sw_acoustic2d_forward_noalloc(const sw_acoustic_params* params, const float* vp, const sw_acoustic_shot* shot,
                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SWGB300_H */
