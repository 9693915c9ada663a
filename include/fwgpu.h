/*
 * fwgpu.h -- C ABI of the GB300 (sm_103a) monodomain-step library.
 *
 * The library advances Finitewave's explicit monodomain scheme on one GPU:
 * stimulus application, the finite-difference diffusion stencil, the per-node
 * ionic update and the activation-time / probe trackers, for the models and
 * stencils of the reference's cpuwave2D / cpuwave3D packages.
 *
 * Conventions
 *  - Every entry point returns an int status: FW_OK (0) or a negative FW_ERR_*
 *    code; fw_last_error() gives a message for the calling thread.  No C++
 *    exception, exit() or abort() crosses this interface.
 *  - All array arguments are caller-owned device pointers (plain pointers plus
 *    sizes).  The library allocates no device memory of its own.
 *  - Arrays are C-order over the grid shape (ni, nj) or (ni, nj, nk), exactly
 *    the reference's numpy layout.  A grid of N = ni*nj*nk nodes.  Per-node
 *    stencil weights are stored weight-major ("structure of arrays"):
 *    w[k*N + p] is weight k of node p, k in the reference's point order.
 *  - Every call takes a stream (a cudaStream_t passed as void*) and is
 *    asynchronous with respect to the host.  Results that depend on device
 *    data (tracker overflow, bad input) go to a device status word that the
 *    caller reads when it next synchronises.
 *  - Calls on different streams with disjoint buffers may run concurrently.
 */
#ifndef FWGPU_H
#define FWGPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define FW_API __attribute__((visibility("default")))
#else
#define FW_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------- status codes */
#define FW_OK 0
#define FW_ERR_ARG (-1)         /* invalid argument (pointer, size, enum)   */
#define FW_ERR_CUDA (-2)        /* a CUDA runtime call failed               */
#define FW_ERR_UNSUPPORTED (-3) /* valid but not implemented combination    */

/* bits of the device status word (int32, OR-ed by kernels) */
#define FW_DEV_LAT_OVERFLOW 1   /* a cell crossed more often than capacity  */
#define FW_DEV_PROBE_OVERFLOW 2 /* a probe sample index beyond capacity     */
#define FW_DEV_BATCH_FAULT 4    /* a batch tile descriptor out of range     */
#define FW_DEV_TIMEOUT 8        /* a bounded on-chip wait gave up           */
#define FW_DEV_TIP_OVERFLOW 16  /* more spiral tips than the tracker holds  */
#define FW_DEV_NONFINITE 32     /* a myocyte's potential became inf or NaN  */

/* fw_step_args.debug_flags (testing the error paths without a fault):
 * FW_DEBUG_FORCE_TIMEOUT makes the TMA kernels treat their first pipeline
 * wait as timed out after the awaited copy has in fact arrived, so the
 * timeout exit (status bit, waits for copies in flight, early return) runs
 * on a healthy GPU.  The results of such a call are not defined. */
#define FW_DEBUG_FORCE_TIMEOUT 1

/* ------------------------------------------------------------ enumerations */
enum fw_model {
    FW_MODEL_AP = 1,   /* Aliev-Panfilov       cpuwave2D/model/aliev_panfilov_2d.py  */
    FW_MODEL_MS = 2,   /* Mitchell-Schaeffer   cpuwave2D/model/mitchell_schaeffer_2d.py */
    FW_MODEL_FK = 3,   /* Fenton-Karma (MLR-I) cpuwave2D/model/fenton_karma_2d.py    */
    FW_MODEL_TP06 = 4, /* ten Tusscher-Panfilov 2006 cpuwave2D/model/tp06_2d.py      */
    FW_MODEL_CRN = 5,  /* Courtemanche 1998    cpuwave2D/model/courtemanche_2d.py    */
    FW_MODEL_BK = 6,   /* Barkley              cpuwave2D/model/barkley_2d.py         */
    FW_MODEL_BO = 7,   /* Bueno-Orovio         cpuwave2D/model/bueno_orovio_2d.py    */
    FW_MODEL_LR91 = 8  /* Luo-Rudy 1991        cpuwave2D/model/luo_rudy91_2d.py      */
};

enum fw_stencil {
    FW_STENCIL_ISO5 = 1,    /* IsotropicStencil2D   (i-1,j),(i,j-1),(i,j),(i,j+1),(i+1,j) */
    FW_STENCIL_ANISO9 = 2,  /* AsymmetricStencil2D  (i-1,j-1)...(i+1,j+1)                 */
    FW_STENCIL_ISO7 = 3,    /* IsotropicStencil3D   order of isotropic_stencil_3d.py:16-23  */
    FW_STENCIL_ANISO19 = 4, /* AsymmetricStencil3D  order of asymmetric_stencil_3d.py:25-44 */
    FW_STENCIL_SYM9 = 5,    /* SymmetricStencil2D weights (fw_build_weights only): the
                               9-point layout of ANISO9, stepped as ANISO9      */
    FW_STENCIL_ANISO19_XY = 6 /* ANISO19 weights whose planes 9, 10, 13..18 (the
                               couplings of k +- 1 with i +- 1 or j +- 1) are all
                               zero, as AsymmetricStencil3D builds them for fibers
                               with no z component: stepped reading the other 11
                               planes (the skipped terms are exact zeros, so the
                               sums are the ANISO19 ones); stored and built as
                               ANISO19 (19 planes)                              */
};

/* Arithmetic policy.  FW_F64: every array float64 (the reference's default
 * npfloat).  FW_F32: u, gates and weights float32; for TP06, Courtemanche
 * and Luo-Rudy 1991 the ion-concentration state variables are compensated
 * float32 pairs (see fw_state_is_pair). */
enum fw_precision { FW_F64 = 0, FW_F32 = 1 };

/* Execution form.  FW_FORM_PLAIN: one launch per time step (plus a stimulus
 * launch on steps where a stimulus fires), reference operation order.
 * FW_FORM_FUSED: 2D FP32 Aliev-Panfilov / Mitchell-Schaeffer / Fenton-Karma
 * only; several time steps per launch on shared-memory tiles (temporal
 * blocking), stimuli and trackers applied inside the launch. */
enum fw_form { FW_FORM_PLAIN = 0, FW_FORM_FUSED = 1 };

enum fw_stim_kind { FW_STIM_VOLTAGE = 0, FW_STIM_CURRENT = 1 };

#define FW_MAX_STATE 24
#define FW_MAX_PARAMS 64
#define FW_MAX_STIMS 16
#define FW_MAX_AT 4
#define FW_MAX_LAT 2
#define FW_MAX_PROBE 4
#define FW_MAX_PROBE_VARS 8
#define FW_MAX_TIP 1
#define FW_MAX_ECG 2
#define FW_MAX_ECG_LEADS 8
#define FW_MAX_FUSED_STATE 4

/* A set of global step indices n with first <= n <= last and
 * n % stride == 0.  Trackers are active on exactly those steps; the host
 * derives first/last from the tracker's start_time/end_time by replaying the
 * float64 time accumulation t += dt (core/tracker/tracker.py:70-83). */
typedef struct fw_window {
    int64_t first, last, stride;
} fw_window;

/* One stimulus.  Replaces StimVoltageCoord2D/3D, StimCurrentCoord2D/3D,
 * StimVoltageMatrix2D/3D, StimCurrentMatrix2D/3D, StimCurrentArea2D/3D
 * (cpuwave2D/stimulation/, cpuwave3D/stimulation/) as driven by
 * StimSequence.stimulate_next (core/stimulation/stim_sequence.py:65-77).
 * Applied on steps first..last (inclusive) to nodes p inside the half-open
 * box with mesh[p] == 1 and (mask == NULL || mask[p] != 0):
 *   voltage: u[p] = value
 *   current: u[p] += value (value = dt * curr_value), then
 *            u[p] = min(u[p], u_max) when has_umax. */
typedef struct fw_stim {
    int32_t kind;
    int32_t has_umax;
    int64_t first, last;
    double value;
    double u_max;
    int64_t lo[3], hi[3];
    const int8_t *mask;
} fw_stim;

/* ActivationTime2D/3DTracker (cpuwave2D/tracker/activation_time_2d_tracker.py:
 * 51-63): on active steps n, act_step[p] = n where act_step[p] < 0 and
 * u[p] > threshold (u read after stimuli, before diffusion).  act_step is
 * int32, initialised to -1 by the caller; the host maps n to its time. */
typedef struct fw_at_tracker {
    fw_window win;
    double threshold;
    int32_t *act_step;
} fw_at_tracker;

/* LocalActivationTime2D/3DTracker (local_activation_time_2d_tracker.py:58-89):
 * on active steps, cross = u >= threshold && !activated[p]: activated[p] = 1
 * and n is appended to the cell's crossing list; backcross = u < threshold &&
 * activated[p]: activated[p] = 0.  cross_steps is (capacity, N) int32,
 * cross_count is N int32; the host rebuilds the reference's layered output.
 * More than `capacity` crossings set FW_DEV_LAT_OVERFLOW. */
typedef struct fw_lat_tracker {
    fw_window win;
    double threshold;
    uint8_t *activated;
    int32_t *cross_steps;
    int32_t *cross_count;
    int32_t capacity;
} fw_lat_tracker;

/* ActionPotential*Tracker / MultiVariable*Tracker / Variable*Tracker
 * (action_potential_2d_tracker.py:46-53, multi_variable_2d_tracker.py:58-69):
 * on active steps, out[((s * n_vars) + v) * n_cells + c] = var_v[cells[c]]
 * with sample index s = sample_offset + (n - win.first) / win.stride
 * (win.first must be the first active step).  var id 0 is u (the value the
 * trackers see: after stimuli, before the step); id k >= 1 is state var k-1
 * (already advanced by the ionic update, as in the reference). */
typedef struct fw_probe_tracker {
    fw_window win;
    int32_t n_cells;
    int32_t n_vars;
    int32_t var_ids[FW_MAX_PROBE_VARS];
    const int64_t *cells;
    double *out;
    int64_t sample_offset;
    int64_t capacity; /* samples */
} fw_probe_tracker;

/* ECG2DTracker / ECG3DTracker (cpuwave2D/tracker/ecg_2d_tracker.py:61-79,
 * 114-153; cpuwave3D/tracker/ecg_3d_tracker.py:51-69, 99-140): on active
 * steps n, for every lead c
 *   out[s * n_leads + c] += sum over myocytes p = (i, j[, k]) with d > 0 of
 *                           (diffuse(u)[p] - u[p]) / (d * dr),
 *   d = (x_c - i)^2 + (y_c - j)^2 + (z_c - k)^2   (k = 0 in 2D),
 * u as the trackers see it (after stimuli, before the step) and diffuse(u)
 * the stencil sum with the model's weights; s = sample_offset +
 * (n - win.first) / win.stride.  `out` (capacity x n_leads float64) must
 * be zero where samples are added.  Plain form only. */
typedef struct fw_ecg_tracker {
    fw_window win;
    int32_t n_leads;
    int32_t reserved;
    double coords[FW_MAX_ECG_LEADS][3];
    double dr;
    double *out;
    int64_t sample_offset;
    int64_t capacity; /* samples */
} fw_ecg_tracker;

/* One spiral-wave tip: grid cell (k, i, j) of the crossing and its position
 * x = j + dy, y = i + dx inside the cell (the reference's [x, y]). */
typedef struct fw_tip {
    int32_t sample;   /* index of the tracked step (sample_offset + ...)  */
    int32_t k, i, j;  /* k = z index (0 in 2D)                            */
    double x, y;
} fw_tip;

/* SpiralWaveCore2DTracker / 3DTracker (cpuwave2D/tracker/
 * spiral_wave_core_2d_tracker.py:88-249, cpuwave3D/tracker/
 * spiral_wave_core_3d_tracker.py): on active steps, every cell (i, i+1) x
 * (j, j+1) of every z layer with 5 <= i < ni - 5, 5 <= j < nj - 5 whose
 * threshold isoline is crossed in both u_prev (the potential at the
 * tracker's previous active step) and u is refined to the intersection of
 * the two bilinear isolines; found tips are appended to `out` (order is not
 * kept: the host sorts by sample, k, i, j) and `count` is advanced; then
 * u_prev := u.  More than `capacity` tips set FW_DEV_TIP_OVERFLOW. */
typedef struct fw_tip_tracker {
    fw_window win;
    double threshold;
    void *u_prev;      /* (N) in the model precision, the last active u   */
    fw_tip *out;
    int32_t *count;    /* device, tips written so far                     */
    int64_t capacity;  /* tips                                            */
    int64_t sample_offset;
} fw_tip_tracker;

/* Everything one model instance needs to advance.  Replaces the body of
 * CardiacModel.run (core/model/cardiac_model.py:164-189) together with the
 * model's run_diffusion_kernel / run_ionic_kernel. */
typedef struct fw_step_args {
    int32_t model;      /* enum fw_model   */
    int32_t stencil;    /* enum fw_stencil */
    int32_t precision;  /* enum fw_precision */
    int32_t form;       /* enum fw_form    */
    int64_t ni, nj, nk; /* nk = 1 for 2D grids */
    const int8_t *mesh; /* tissue mesh codes 0/1/2 (stimuli test mesh == 1)  */
    const int8_t *myo;  /* 1 where mesh == 1 and special_boundaries == 0     */
    const void *weights;         /* (nw, N), float64 or float32 by precision */
    void *u[2];                  /* u[0]: u at n_begin, u[1]: the other buffer */
    void *state[FW_MAX_STATE];   /* the model's state variables after u      */
    double params[FW_MAX_PARAMS];
    double dt;
    int32_t n_stims;
    int32_t n_at;
    int32_t n_lat;
    int32_t n_probe;
    fw_stim stims[FW_MAX_STIMS];
    fw_at_tracker at[FW_MAX_AT];
    fw_lat_tracker lat[FW_MAX_LAT];
    fw_probe_tracker probe[FW_MAX_PROBE];
    int32_t *status;  /* device int32 status word (may be NULL)             */
    int32_t fused_k;  /* FW_FORM_FUSED time steps per launch: 2, 4 or 8
                         (0 = 4); 3 also for variant 3                      */
    int32_t fused_variant; /* FW_FORM_FUSED kernel: 0 = automatic (the TMA
                              pipeline when weights_packed is given and
                              nj % 16 == 0, else 1); 1 = cp.async staging,
                              64x32-node regions, two CTAs per SM; 2 = same,
                              64x64 regions; 3 = TMA pipeline (persistent
                              CTAs, double-buffered 64x32 regions, 4 x 1
                              nodes per thread); 4 = the TMA pipeline with
                              2 x 2 nodes per thread (even fused_k).
                              6 = variant 4 in two-wide float32
                              instructions (f32x2, even fused_k);
                              7 = 64-column strips marched down the rows
                              with the fused_k <= 4 time levels in flight
                              (no probe trackers).
                              Variants 1-4, 6 and 7 give bitwise the same
                              results; 5 = variant 3 with the
                              AsymmetricStencil2D weights formed on chip
                              from fibers_f32 (within float32 rounding of
                              the others)                                  */
    const void *weights_packed; /* FW_FORM_FUSED: off-centre float32 weights
                                   node-major, (N, 4) for ISO5 or (N, 8)
                                   for ANISO9, from fw_pack_weights; NULL
                                   when not available.  The TMA variants
                                   also read the centre plane of `weights`
                                   (16-byte aligned)                        */
    int32_t n_ecg;
    int32_t n_tip;
    fw_ecg_tracker ecg[FW_MAX_ECG];
    fw_tip_tracker tip[FW_MAX_TIP];
    int32_t debug_flags; /* 0 in normal use; FW_DEBUG_* bits for tests      */
    int32_t reserved2;
    int64_t pitch;       /* row pitch in nodes of u[0], u[1], the state
                            arrays, myo, weights, weights_packed and the
                            local activation trackers' `activated` flags
                            (their N is ni * pitch); 0 = nj.  Stimulus
                            masks and the other tracker arrays always have
                            rows of nj nodes.  fw_batch_plan only: fw_step
                            takes 0 or nj                                 */
    void *state_b[FW_MAX_FUSED_STATE]; /* FW_FORM_FUSED and batches: second
                            buffers of the state variables (same type and
                            size as state[], equal to them at non-myocytes).
                            A launch reads every region's state from one
                            buffer and writes its tiles' new state to the
                            other, so no region reads state a neighbouring
                            tile has already advanced.  The buffers change
                            roles with u[0] / u[1]: on return the current
                            state is in state[] after an even number of
                            steps and in state_b[] after an odd one      */
    const float *fibers_f32; /* fused_variant 5 only: the fibers of a 2D
                            AsymmetricStencil2D tissue as float32 (N, 2),
                            rows of nj nodes, 16-byte aligned.  The kernel
                            forms each region's nine weights on chip from
                            them and the myocyte flags (float32 flux sums)
                            instead of reading weights_packed and the
                            centre plane; NULL otherwise                  */
    double fly_D_al, fly_D_ac; /* fused_variant 5: the stencil's D_al, D_ac */
    double fly_cond;         /* fused_variant 5: the tissue's scalar
                                conductivity                              */
    double fly_scale;        /* fused_variant 5: D_model * dt / dr**2      */
    const void *weight_rows; /* FW_STENCIL_ANISO19_XY, plain form: the
                            distinct rows of the eleven weight planes it
                            reads (0-8, 11, 12), in the precision's type,
                            padded to 12 values per row (16-byte aligned),
                            with weight_row_index giving each node's row;
                            the step reads these instead of `weights`
                            (same values, same sums).  NULL otherwise      */
    const int32_t *weight_row_index; /* (N) row of each node, or NULL    */
} fw_step_args;

/* A planned batch of tissues (fw_batch_plan).  Host-side handle; the
 * device data lives in the caller's plan buffer. */
typedef struct fw_batch {
    void *plan;          /* device plan buffer given to fw_batch_plan        */
    int32_t n_tissues;
    int32_t n_tiles;     /* fused regions over all tissues                   */
    int32_t ksteps;      /* time steps per launch                            */
    int32_t grid;        /* persistent CTAs per launch                       */
    int32_t kernel;      /* 1 = cp.async staging, 2 = TMA pipeline, 3 = TMA
                            pipeline with 2 x 2 nodes per thread in two-wide
                            float32 instructions (every tissue planned with
                            fused_variant 6); 2 and 3 give the same bits   */
    int32_t reserved;
    int32_t group_end[6]; /* kernels 2, 3: end of each (model, stencil) group in
                             the tile list -- AP/ISO5, AP/ANISO9, MS/ISO5,
                             MS/ANISO9, FK/ISO5, FK/ANISO9 -- each advanced by
                             its own kernel launch                          */
} fw_batch;

/* Library version (major*10000 + minor*100 + patch). */
FW_API int fw_version(void);

/* sizeof of the ABI structs as compiled into the library, so a binding can
 * check its own layout: which = 0 fw_step_args, 1 fw_stim, 2 fw_at_tracker,
 * 3 fw_lat_tracker, 4 fw_probe_tracker, 5 fw_window, 6 fw_batch,
 * 7 fw_ecg_tracker, 8 fw_tip_tracker, 9 fw_tip.  0 for unknown. */
FW_API size_t fw_struct_size(int32_t which);

/* Number of kernels this library has launched in the process so far
 * (a monotonic statistics counter, for benchmarks and tests). */
FW_API int64_t fw_launch_count(void);

/* Message for the last non-OK status returned on the calling thread. */
FW_API const char *fw_last_error(void);

/* Number of state variables after u, and the parameter count, of a model;
 * the order is that of the reference class's state_vars (minus "u") and of
 * the parameter list documented in fw_models.cuh. */
FW_API int fw_model_info(int32_t model, int32_t *n_state, int32_t *n_params);

/* 1 when state variable `index` of `model` is stored as float64 under
 * `precision`: every variable under FW_F64, none under FW_F32. */
FW_API int fw_state_is_f64(int32_t model, int32_t precision, int32_t index);

/* 1 when state variable `index` of `model` is stored as a compensated
 * float32 pair under `precision`: the ion concentrations of TP06,
 * Courtemanche and Luo-Rudy 1991 under FW_F32, 8 bytes per node (float
 * hi, float lo: the value hi + lo, |lo| <= ulp(hi) / 2).  Other variables
 * are stored in the precision's type. */
FW_API int fw_state_is_pair(int32_t model, int32_t precision, int32_t index);

/* Stencil weights.  Replaces Stencil.compute_weights (core/stencil/stencil.py:
 * 14) as implemented by IsotropicStencil2D (isotropic_stencil_2d.py:41-69),
 * AsymmetricStencil2D (asymmetric_stencil_2d.py:46-84), IsotropicStencil3D
 * (isotropic_stencil_3d.py:45-74) and AsymmetricStencil3D
 * (asymmetric_stencil_3d.py:61-105).  Computed in float64 with the
 * reference's operation order (bitwise equal to it), then stored as float64
 * or rounded to float32 by `precision`.
 *   mesh       int8 codes (N)
 *   cond       float64 conductivity per node (N), or NULL for cond_scalar
 *   fibers     float64 (N, ndim) unit vectors; NULL for isotropic stencils
 *   dr2        dr**2 as the host language computes it
 *   w_out      (nw, N) float64 or float32 */
FW_API int fw_build_weights(int32_t stencil, int32_t precision, const int8_t *mesh,
                     const double *cond, double cond_scalar,
                     const double *fibers, double D_al, double D_ac,
                     double D_model, double dt, double dr2, int64_t ni,
                     int64_t nj, int64_t nk, void *w_out, void *stream);

/* One diffusion pass u_new[p] = sum_k w[k][p] * u[nbr_k(p)] over the flat
 * myocyte list idx.  Replaces the stencils' diffusion_kernel(u_new, u, w,
 * indexes) callables (isotropic_stencil_2d.py:97-132, asymmetric_stencil_2d.py
 * :164-201, isotropic_stencil_3d.py:78-109, asymmetric_stencil_3d.py:108-160),
 * which the ECG trackers also call (ecg_2d_tracker.py:61-79). */
FW_API int fw_diffuse(int32_t stencil, int32_t precision, void *u_new, const void *u,
               const void *w, const int64_t *idx, int64_t n_idx, int64_t ni,
               int64_t nj, int64_t nk, void *stream);

/* One ionic pass over idx: state updated in place and u_new[p] += dt * I(p).
 * Replaces the models' ionic_kernel_2d/3d (e.g. aliev_panfilov_2d.py:376-406)
 * as called by run_ionic_kernel.  state and params as in fw_step_args. */
FW_API int fw_ionic(int32_t model, int32_t precision, void *u_new, const void *u,
             void *const *state, const int64_t *idx, int64_t n_idx,
             double dt, const double *params, void *stream);

/* Repack float32 weight-major weights (nw, N) into the node-major layout of
 * the fused TMA kernel: out[p * nwo + q] = w[plane_q * N + p] over the
 * off-centre planes (nwo = 4 for ISO5, 8 for ANISO9; the centre weight is
 * implied because each stencil row sums to one).  2D stencils only. */
FW_API int fw_pack_weights(int32_t stencil, const float *w, int64_t n,
                           float *out, void *stream);

/* One ECG sample: the sum of fw_ecg_tracker for the potential u (N nodes)
 * with weights w (nw, N) over the nodes with myo[p] != 0, for n_leads
 * leads at coords (n_leads x 3 float64 in HOST memory, passed to the kernel
 * by value), added to out[0..n_leads-1] (float64, device).  Replaces compute_ecg after model.diffusion_kernel
 * (ecg_2d_tracker.py:61-79 with :114-153; ecg_3d_tracker.py:51-69 with
 * :99-140). */
FW_API int fw_ecg(int32_t stencil, int32_t precision, const void *u,
                  const void *w, const int8_t *myo, int64_t ni, int64_t nj,
                  int64_t nk, const double *coords, int32_t n_leads,
                  double dr, double *out, void *stream);

/* Advance n_steps time steps starting at global step n_begin (the model's
 * step counter).  On return the current u is a->u[n_steps & 1]. */
FW_API int fw_step(const fw_step_args *a, int64_t n_begin, int64_t n_steps,
            void *stream);

/* ---- batches of tissues (no single reference counterpart: the reference
 * runs one CardiacModel.run loop per tissue, core/model/cardiac_model.py:
 * 130-189; a batch advances many such runs together) -------------------- */

/* Device bytes of the plan for these tissues.  Each tissue is an
 * fw_step_args as for fw_step with: a 2D grid, FW_F32, model AP / MS / FK,
 * stencil ISO5 / ANISO9, at most one activation tracker and one local
 * activation tracker, no probe tracker, and u[0], u[1] equal at
 * non-myocytes.  Tissues may differ in size, model, stencil, parameters,
 * stimuli and trackers. */
FW_API int fw_batch_plan_size(const fw_step_args *const *tissues, int32_t n,
                              int64_t *plan_bytes);

/* Build the device plan (descriptor table and tile list) in `plan`
 * (16-byte aligned device memory of at least fw_batch_plan_size bytes) and
 * fill *out.  n_begin[i] is tissue i's global step at batch offset 0 (its
 * stimulus and tracker windows are in its own step numbering).  Copies the
 * plan synchronously on `stream`. */
FW_API int fw_batch_plan(const fw_step_args *const *tissues, int32_t n,
                         const int64_t *n_begin, void *plan,
                         int64_t plan_bytes, fw_batch *out, void *stream);

/* Device bytes of the scratch a batch run needs (tile counters).  The
 * scratch must be zero before its first use; every launch leaves it zero,
 * so it can be reused by later runs on the same stream. */
FW_API int fw_batch_scratch_size(int64_t *bytes);

/* Advance every tissue of the batch by n_steps time steps from batch offset
 * `offset` (tissue i at its step n_begin[i] + offset).  The current u of
 * each tissue is its u[offset & 1] on entry and u[(offset + n_steps) & 1] on
 * return, as after the same steps of fw_step.  Calls sharing one scratch
 * buffer must be ordered (the same stream). */
FW_API int fw_batch_run(const fw_batch *b, void *scratch, int64_t offset,
                        int64_t n_steps, void *stream);

/* fw_batch_run without a scratch argument; no counterpart in the reference
 * (the reference runs on the CPU and has no device scratch).  For callers
 * that cannot hand the library a scratch buffer: code that may not allocate
 * device memory itself -- for instance a binding that receives the tissues'
 * arrays and the plan buffer from another runtime and has no allocator of
 * its own for the device, or a program that fixes its device memory at
 * set-up.  The tile counters then live in a fixed array inside the library
 * (256 bytes per device).  A batch's scratch has a fixed size
 * (fw_batch_scratch_size), so the limit is checked when the library is
 * compiled; a NULL or empty plan and a negative offset or step count are
 * rejected with FW_ERR_ARG.  The call allocates nothing.  The first call on a device does
 * a one-time set-up (looks up the array's device address and zeroes it on
 * `stream`), so make that first call before any stream capture.  All calls
 * on one device share the array: calls whose launches may overlap (other
 * streams, other host threads) race and must be ordered by the caller.
 * Otherwise identical to fw_batch_run. */
FW_API int fw_batch_run_noalloc(const fw_batch *b, int64_t offset,
                                int64_t n_steps, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FWGPU_H */
