/*
 * fwi_psv.h -- C ABI of the GB300 (sm_103a) engine for the 2-D elastic P-SV
 * FWI hot path: staggered-grid stress/velocity time stepping with Holberg
 * coefficients and CPML, source injection, seismogram recording, the adjoint
 * pass and the lambda/mu/rho gradient.
 *
 * Replaces (reference = Mohammad-debug/CUDA_FWI, paths relative to its root):
 *   forward_kernel_PSV_GPU / forward_kernel_PSV   CUDA_week2/fd_kernel.cuh:12-43, 75-120
 *   adjoint_kernel_PSV_GPU / adjoint_kernel_PSV   CUDA_week2/fd_kernel.cuh:46-70, 123-173
 * and the setup those calls depend on:
 *   holbergcoeff                 CUDA_week2/holbergcoeff.cu:6
 *   FDCpml::cpml_pro             CUDA_week2/fd_cpml.cu:59
 *   FDMedium::average_parameters CUDA_week2/fd_medium.cu:128
 *   create_wavelet               CUDA_week2/fd_seismogram.cu:166
 *   FDGrid::total_grid           CUDA_week2/fd_grid.cu:52
 *   calculate_l2_adjoint_sources CUDA_week2/fd_wave_model.cu:972
 *
 * Conventions
 *   - Every call returns an int status (FWI_OK = 0 or a negative FWI_ERR_*);
 *     nothing here calls exit().  fwi_psv_strerror() names a status and
 *     fwi_psv_last_error() gives the detail message of the calling thread.
 *   - Host arrays are FP64, row-major, in the reference's layouts:
 *       wavefield, lam, mu, rho ........ [nzt][nxt]
 *       mu_zx, rho_zp, rho_xp ........... [nzt-1][nxt-1]
 *       CPML profiles a,b,K,a_half,.. .. [2*(npml+1)]
 *       CPML x-strip memory ............. [nzt][2*(npml+1)]
 *       CPML z-strip memory ............. [2*(npml+1)][nxt]
 *       signals, seismograms ............ [nseis][nt]
 *       FWI storage ..................... [nft][nfz][nfx]
 *       gradients ....................... [nfz][nfx]
 *     Grid indices (source/receiver x,z, FWI window) are padded-grid indices,
 *     as after FDSeismogram::grid_adjustment / FDFWI::parse_configuration.
 *   - The device computes in FP32.  An engine owns its device memory, is
 *     bound to one device and one CUDA stream, and is not thread-safe; use one
 *     engine per host thread.
 */
#ifndef FWI_PSV_H
#define FWI_PSV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FWI_PSV_ABI_VERSION 2

enum {
    FWI_OK = 0,
    FWI_ERR_INVALID = -1,     /* bad argument, size or index */
    FWI_ERR_UNSUPPORTED = -2, /* valid for the reference but outside this engine */
    FWI_ERR_NOMEM = -3,       /* device or host allocation failed / over budget */
    FWI_ERR_CUDA = -4,        /* CUDA runtime error (detail in fwi_psv_last_error) */
    FWI_ERR_STATE = -5,       /* call out of order (e.g. backward before forward) */
    FWI_ERR_DIVERGED = -6,    /* |syn-obs| > 1e10, where the reference exits */
    FWI_ERR_NOFORWARD = -7,   /* backward without a retained forward */
    FWI_ERR_NODEVICE = -8,    /* no CUDA device / driver */
    FWI_ERR_IO = -9           /* a file could not be written (the FWI resume file) */
};

/* ---- setup helpers (host) ---------------------------------------------- */

int fwi_psv_abi_version(void);
const char* fwi_psv_strerror(int status);
const char* fwi_psv_last_error(void);

/* holbergcoeff.cu:6-60: hc[0..6] for fdorder 2..12 and max_rel_err 0..4. */
int fwi_psv_holberg(int fdorder, int max_rel_err, double hc[7]);

/* fd_cpml.cu:59-192: six profiles of length 2*(npml+1). */
int fwi_psv_cpml_profile(int npml, double dh, double fpml, double npower, double k_max_pml,
                         double rcoef, double damp_v_pml, double dt, double* a, double* b,
                         double* K, double* a_half, double* b_half, double* K_half);

/* fd_grid.cu:52-71 */
int fwi_psv_total_grid(int nx, int nz, int fdorder, int npml, int fsurf, int* fpad, int* ppad,
                       int* nxt, int* nzt);

/* fd_seismogram.cu:166-185 (shape 1 = Ricker). */
int fwi_psv_wavelet(double* signal, int nt, double dt, double amp, double fc, double ts,
                    int shape);

/* fd_medium.cu:128-159 on the host (FP64); outputs [nzt-1][nxt-1]. */
int fwi_psv_average_parameters(int nzt, int nxt, const double* mu, const double* rho,
                               double* mu_zx, double* rho_zp, double* rho_xp);

/* ---- device memory ------------------------------------------------------ */

/* No counterpart in the reference (which calls cudaMalloc directly and exits
 * when it fails, forward_kernel_PSV_GPU.cu:19-27).  Once set, every device
 * allocation of the library's engines, multi-model engines and FWI loop goes
 * through alloc(bytes, ctx) and is returned through release(ptr, ctx): an
 * application's pool allocator, for example.  alloc returns device memory of
 * the current device aligned to 256 bytes, or NULL; a NULL (or a misaligned
 * pointer, handed back at once) makes the call that needed the memory return
 * FWI_ERR_NOMEM, and the engine stays usable.  A buffer is released through
 * the allocator that made it, even after a later change (so release and ctx
 * must stay valid while an engine made under them lives), and only after the
 * device has been synchronised (as cudaFree does).  alloc = release = NULL
 * restores cudaMalloc / cudaFree.  Set it between calls, not while
 * another thread runs one.  (The caller's d_* buffers of the
 * reference-signature calls are the caller's, as in the reference.) */
typedef void* (*fwi_psv_alloc_fn)(size_t bytes, void* ctx);
typedef void (*fwi_psv_free_fn)(void* ptr, void* ctx);
int fwi_psv_set_device_allocator(fwi_psv_alloc_fn alloc, fwi_psv_free_fn release, void* ctx);

/* ---- engine ------------------------------------------------------------ */

typedef struct fwi_psv_engine fwi_psv_engine;

/* Geometry and scheme: the leading scalar arguments of forward_kernel_PSV
 * (fd_kernel.cuh:12-17) plus the CPML profiles (FDCpml::a..K_half). */
typedef struct fwi_psv_desc {
    int nt, nzt, nxt, fpad, ppad, npml, fsurf, fdorder;
    double dt, dx, dz;
    double hc[7];
    const double *a, *b, *K, *a_half, *b_half, *K_half;
} fwi_psv_desc;

/* Gradient strategies (what the adjoint reads the forward wavefield from). */
enum {
    FWI_STORE_FULL = 0,     /* every sampled step kept in HBM (the reference's FDFWI storage) */
    FWI_STORE_BINOMIAL = 1, /* binomial checkpointing with forward recompute */
    FWI_STORE_RANDOM = 2    /* random-boundary wavefield reconstruction (no CPML on the source side) */
};
/* FWI_STORE_RANDOM keeps one state per shot.  The recording forward keeps
 * the CPML (seismograms, misfit and residual as with the other strategies);
 * a second forward runs without CPML in a seeded random-velocity frame filling
 * the padding (velocities scaled by 1 - 0.5 (depth into the padding / ppad) u,
 * u uniform in [0, 1) per block of 16 x 16 cells); the backward rebuilds that
 * second wavefield by undoing its steps in reverse (FP32 round-off makes it
 * drift slightly) and correlates it with the adjoint wavefield, which keeps
 * the CPML.  Cost per shot
 * gradient: 4 nt time steps (the frame forward and the reverse sweep count as
 * recompute_steps).  Needs the TMA mapping (the default), no free surface (its
 * surface row is assigned, not incremented, so it cannot be undone) and
 * FWI_GRAD_REFERENCE (FWI_GRAD_EXACT always checkpoints). */

/* Gradient formula.
 * FWI_GRAD_EXACT has no reference counterpart: it is dJ/d(lam, mu, rho) of
 * J = sum 0.5 dt (syn-obs)^2 for the raw (unaveraged) models, sampled at the
 * FWI window's grid points (fwi_dt does not apply: every time step enters).
 * It always runs the checkpointed schedule, one time step per unit (snapshots
 * and budget as for FWI_STORE_BINOMIAL, whatever the strategy), needs mu > 0
 * on every interior cell, and its backward returns FWI_ERR_UNSUPPORTED
 * otherwise. */
enum {
    FWI_GRAD_REFERENCE = 0, /* the reference's correlation kernel (adjoint_kernel_PSV_GPU.cu:830-863) */
    FWI_GRAD_EXACT = 1      /* discrete adjoint of the FP32 scheme (matches finite differences) */
};

/* Create an engine on CUDA device `device`.  The descriptor is copied. */
int fwi_psv_create(const fwi_psv_desc* desc, int device, fwi_psv_engine** out);
int fwi_psv_destroy(fwi_psv_engine* e);

/* All work of the engine is queued on this stream (a cudaStream_t; NULL = the
 * engine's own non-blocking stream). */
int fwi_psv_set_stream(fwi_psv_engine* e, void* cuda_stream);

/* Materials, reference layouts (fd_medium.cuh: lam, mu [nzt][nxt]; mu_zx,
 * rho_zp, rho_xp [nzt-1][nxt-1]), as passed to forward_kernel_PSV. */
int fwi_psv_set_model(fwi_psv_engine* e, const double* lam, const double* mu,
                      const double* mu_zx, const double* rho_zp, const double* rho_xp);

/* lam, mu, rho [nzt][nxt]; the staggered averages are formed on the device
 * (FDMedium::average_parameters as a kernel). */
int fwi_psv_set_model_lmr(fwi_psv_engine* e, const double* lam, const double* mu,
                          const double* rho);

/* Sources: FDSeismogram source arrays (x, z padded; comp 2 = vz, the only
 * component the reference implements; shot = shot_to_fire) and their signals
 * [nsrc][nt]. */
int fwi_psv_set_sources(fwi_psv_engine* e, int nsrc, const int* x, const int* z,
                        const int* comp, const int* shot, const double* signal);

/* Receivers: the receiver FDSeismogram arrays (shot = receiver_to_record_shot). */
int fwi_psv_set_receivers(fwi_psv_engine* e, int nrec, const int* x, const int* z,
                          const int* comp, const int* shot);

/* FWI sub-sampling and window ([full_waveform_inversion] after padding,
 * fd_fwi.cu:28-51).  Defaults: 1,1,1 and the whole padded grid. */
int fwi_psv_set_fwi(fwi_psv_engine* e, int fwi_dt, int fwi_dx, int fwi_dz, int x1, int x2,
                    int z1, int z2);

/* strategy = FWI_STORE_*; snapshots = checkpoint slots per shot for
 * FWI_STORE_BINOMIAL (0 = as many as budget_bytes allows); budget_bytes = cap
 * on the engine's device memory (0 = 90% of free memory at the call). */
int fwi_psv_set_strategy(fwi_psv_engine* e, int strategy, int snapshots, size_t budget_bytes);

/* Gradient formula (FWI_GRAD_*). */
int fwi_psv_set_gradient_mode(fwi_psv_engine* e, int mode);

/* Forward pass for `nshots` shots (ids in `shots`) run together on the device.
 *   obs      [nrec][nt] observed data, or NULL (no misfit; backward then needs
 *            a residual from elsewhere).
 *   rec_out  [nrec][nt] synthetic seismograms (rows of receivers recorded by
 *            a shot of this batch are written, others untouched), or NULL.
 *   misfit   [nshots] per-shot J = sum 0.5 dt (syn-obs)^2, or NULL.
 *   flags    FWI_FWD_KEEP: retain what backward needs (storage or checkpoints);
 *            FWI_FWD_RESIDENT_OBS: reuse the observed data already on the device
 *            from the previous forward of the same batch (obs is ignored).
 */
enum { FWI_FWD_KEEP = 1, FWI_FWD_RESIDENT_OBS = 2 };
int fwi_psv_forward(fwi_psv_engine* e, int nshots, const int* shots, const double* obs,
                    double* rec_out, double* misfit, int flags);

/* Backward for the batch of the last forward(keep=1): adjoint pass driven by
 * the residual at the receivers, gradient accumulation.  Gradients are
 * [nfz][nfx]; with sum_shots != 0 one summed triple is written, otherwise
 * nshots consecutive triples ([nshots][nfz][nfx] each).  Any output may be NULL. */
int fwi_psv_backward(fwi_psv_engine* e, double* grad_lam, double* grad_mu, double* grad_rho,
                     int sum_shots);

/* Shot gradients of `nshots` shots summed into grad_* ([nfz][nfx] each; any
 * may be NULL), with misfit[nshots] (or NULL).  The shots run in sub-batches
 * (FWI_FWD_* flags apply; the batch size is set by fwi_psv_set_exec or chosen
 * so a sub-batch's working set stays in L2): per sub-batch a forward sweep
 * with checkpoints or storage, the residual against obs ([nrec][nt]), the
 * backward, and a device-side sum.  The gradients stay on the device until
 * the end; one host transfer of the sum. */
int fwi_psv_gradient(fwi_psv_engine* e, int nshots, const int* shots, const double* obs,
                     double* misfit, double* grad_lam, double* grad_mu, double* grad_rho,
                     int flags);

/* Energy sums of the last forward (Ws) and backward (Wr) for shot slot `slot`
 * of the batch, [nzt][nxt] (the reference's We arrays). */
int fwi_psv_energy(fwi_psv_engine* e, int slot, double* Ws, double* Wr);

/* Final wavefield (vx, vz, sxx, szx, szz [nzt][nxt]) of batch slot `slot` after
 * the last forward (which=0) or backward (which=1). */
int fwi_psv_wavefield(fwi_psv_engine* e, int which, int slot, double* vx, double* vz,
                      double* sxx, double* szx, double* szz);

/* Counters of the last forward/backward/gradient call: kernel launches, time
 * steps of the recording forward sweep, of recomputation and of the adjoint
 * (per shot for fwi_psv_gradient), and device bytes held. */
typedef struct fwi_psv_stats {
    int64_t launches, forward_steps, recompute_steps, adjoint_steps;
    int64_t device_bytes, snapshots;
    double last_forward_ms, last_backward_ms;  /* device time of the compute (CUDA events) */
    int64_t h2d_bytes, d2h_bytes;              /* host<->device bytes of the last call */
    int64_t batch;                             /* shots per launch of the last gradient call */
} fwi_psv_stats;
int fwi_psv_get_stats(fwi_psv_engine* e, fwi_psv_stats* out);

/* The binomial checkpoint schedule behind FWI_STORE_BINOMIAL (Griewank &
 * Walther's revolve bound) for reversing `nsteps` super-steps (fwi_dt time
 * steps each) with `slots` checkpoint slots.  actions is [cap][3] of
 * (kind, a, b): 0 = advance state a -> b, 1 = save state b into slot a,
 * 2 = restore slot a (-1 = the zero initial state) holding state b,
 * 3 = adjoint of super-step a.  *count = actions written (FWI_ERR_INVALID if
 * cap is too small, with *count = actions needed); *forward_steps = advance cost. */
int fwi_psv_checkpoint_plan(int nsteps, int slots, int* actions, int cap, int* count,
                            long long* forward_steps);

/* Device time of one launch of each hot kernel on the current batch, averaged
 * over `reps` launches timed with CUDA events on the engine's stream, in the
 * form the checkpointed gradient runs most: ms[0] forward stress, ms[1]
 * forward velocity (no energy sum: the recompute sweeps), ms[2] adjoint stress
 * (+ux/uz and the gradient), ms[3] adjoint velocity (+energy).  Source and
 * receiver events are not included.  Needs a prior forward; it overwrites the
 * wavefield state (the retained forward is dropped). */
int fwi_psv_time_kernels(fwi_psv_engine* e, int reps, double ms[4]);

/* Execution options: use_graphs != 0 captures the time loop in CUDA graphs
 * (default 1); block_x selects the thread mapping of the stencil passes:
 * 0 the default (256), 256 TMA-staged 128x16 tiles in persistent CTAs, 64
 * vectorised cells (float4 per thread), 32 scalar cells, 128 (or tile_z > 0,
 * rows per tile) the register z-march; batch = shots per launch of
 * fwi_psv_gradient (0 = automatic).  Every mapping computes the same stencil;
 * rounding differs between mappings. */
int fwi_psv_set_exec(fwi_psv_engine* e, int use_graphs, int block_x, int tile_z, int batch);

/* Wavefield snapshots of the recording forward sweep (forward_kernel_PSV_GPU.cu
 * :1067-1080): field `which` (0 vx, 1 vz, 2 sxx, 3 szx, 4 szz; the reference
 * writes szz) of every batch slot after each time step it with
 * it % interval == 0.  interval 0 switches them off. */
int fwi_psv_set_snapshots(fwi_psv_engine* e, int interval, int which);
/* Snapshot k (time step k * interval) of batch slot `slot` of the last
 * forward, [nzt][nxt]. */
int fwi_psv_snapshot(fwi_psv_engine* e, int slot, int k, double* out);

/* Grid and FWI-window extents of an engine (after fwi_psv_set_fwi). */
typedef struct fwi_psv_layout {
    int nt, nzt, nxt, fpad, ppad, npml, fsurf, fdorder;
    int fwi_dt, fwi_dx, fwi_dz, x1, x2, z1, z2, nfz, nfx;
    int device;
} fwi_psv_layout;
int fwi_psv_get_layout(fwi_psv_engine* e, fwi_psv_layout* out);

/* ---- device-resident models, preconditioning, trial misfits --------------- */

/* lam, mu, rho [nzt][nxt] FP64 already in device memory (cudaMalloc'd by the
 * caller, current device = the engine's); the staggered averages
 * (FDMedium::average_parameters, fd_medium.cu:128-159) and the dt scaling run
 * as a kernel, giving the same materials as fwi_psv_set_model_lmr. */
int fwi_psv_set_model_device(fwi_psv_engine* e, const double* d_lam, const double* d_mu,
                             const double* d_rho);

/* Energy-weight preconditioning of each shot's gradient before the shot sum
 * (scale_gradients_with_energy_weights, fd_wave_model.cu:1004-1052):
 * g /= (sqrt(Ws Wr) + 0.005 max sqrt(Ws Wr)) C^2 with Ws, Wr the forward and
 * adjoint energy sums of that shot and C the medium averages
 * (FDMedium::medium_average, fd_medium.cu:253-277). on = 0 switches it off. */
int fwi_psv_set_precondition(fwi_psv_engine* e, int on, double c_lam, double c_mu, double c_rho);

/* Per-shot misfits of `nshots` shots from forward-only runs in sub-batches
 * (no storage, no checkpoints): the trial runs of the step-length search.
 * obs and flags as for fwi_psv_gradient. */
int fwi_psv_misfit(fwi_psv_engine* e, int nshots, const int* shots, const double* obs, double* misfit,
                   int flags);

/* ---- FWI optimiser ---------------------------------------------------------
 * The reference's inversion loop (FDWaveModel::fwi_simulate, fd_wave_model.cu
 * :736-955) on the device: medium averages, batched checkpointed gradients
 * with energy-weight preconditioning, the parabolic step-length search
 * (fwi_step_length_estimation.cu:16-223) with batched forward-only trials,
 * and the bounded, max-normalised material update (FDMedium::fwi_grad_update,
 * fd_medium.cu:161-240: rho in [1.5, 3000] with half the step, lam <= 48e9,
 * mu <= 27e9).  Gradients, models and updates stay on the device; the host
 * runs the search's control flow.  Differences from the reference, each
 * selectable: FWI_ORDER_SUMMED sums the shot gradients before one update per
 * iteration (the reference updates after every shot: FWI_ORDER_PER_SHOT);
 * FWI_TRIAL_SUM compares misfits summed over all shots in the search (the
 * reference keeps only the last shot's: FWI_TRIAL_LAST_SHOT).  The update
 * touches the FWI window's sample cells; a failed search stops the loop with
 * the model unchanged instead of exiting the process. */
enum { FWI_ORDER_SUMMED = 0, FWI_ORDER_PER_SHOT = 1 };
enum { FWI_TRIAL_SUM = 0, FWI_TRIAL_LAST_SHOT = 1 };
typedef struct fwi_psv_fwi_opts {
    int max_iter;          /* [FDM] max_iteration */
    double max_error;      /* [FDM] max_error: stop once the misfit falls below it */
    double step_length;    /* first step-length estimate (the reference starts at 0.01) */
    int order;             /* FWI_ORDER_* */
    int trial_misfit;      /* FWI_TRIAL_* */
    int precondition;      /* energy-weight preconditioning (the reference: 1) */
    const double *true_lam, *true_mu, *true_rho; /* optional [nzt][nxt]: model error per iteration */
    double restart_step;   /* no counterpart in the reference, which exits when a search finds no
                            * step that lowers the misfit: > 0 retries such a search once, on the
                            * same gradient, from this step-length estimate (e.g. the initial one,
                            * after the searches' starting steps have shrunk); 0 stops there, as
                            * the reference would (status 1) */
    const char* resume_file; /* no counterpart in the reference (whose per-iteration model CSVs,
                            * fd_wave_model.cu:919-952, have no loader): when not NULL, after each
                            * completed iteration the loop state -- iterations done, the next
                            * search's starting step, whether the loop stopped, the log so far and
                            * the model -- replaces this file (written beside it and renamed); a
                            * run that finds the file continues from it (the model arguments'
                            * values are then replaced by the file's) until max_iter iterations in
                            * all, giving the log and model of an uninterrupted run.  A file of
                            * another grid or option set is FWI_ERR_INVALID. */
} fwi_psv_fwi_opts;
typedef struct fwi_psv_fwi_iter {
    double misfit;         /* summed shot misfit at the model the gradient was taken at */
    double step_length;    /* step of the parabolic fit (0 when the search failed) */
    int trials;            /* trial forward sweeps (over all shots) of the search (and its retry) */
    int status;            /* 0; 1 no step reduced the misfit (model kept); 2 no bracketing third step */
    double model_error;    /* ||m - m_true|| / ||m_true|| over lam, mu, rho (each relative), or -1 */
    double seconds;        /* wall time of the iteration */
} fwi_psv_fwi_iter;
/* lam, mu, rho [nzt][nxt]: starting model in, final model out.  log holds
 * max_iter entries (max_iter * shots for FWI_ORDER_PER_SHOT); *done = entries
 * written.  obs [nrec][nt] as for fwi_psv_gradient. */
int fwi_psv_fwi_run(fwi_psv_engine* e, const fwi_psv_fwi_opts* opts, int nshots, const int* shots,
                    const double* obs, double* lam, double* mu, double* rho, fwi_psv_fwi_iter* log,
                    int* done);

/* Parabola through (sl[i], L2[i]), i = 0..2, and its vertex -x1/(2 x2)
 * (calc_opt_step + solvelin, fwi_step_length_estimation.cu:226-271 and
 * solvelin.cu:6-42, float multiplier and back-substitution accumulator kept). */
double fwi_psv_calc_opt_step(const double L2[3], const double sl[3]);

/* The step-length search's state machine (fwi_step_length_estimation.cu:46-223)
 * with a caller-supplied trial: trial(ctx, step, &misfit) evaluates the model
 * updated with `step` (rho with half of it).  L2_0 = misfit at step 0.  On
 * return *opt = optimum step (status 0 or 2) and *trials = trial calls;
 * status 1: no step reduced the misfit within 6 halvings (*opt = 0). */
typedef int (*fwi_psv_trial_fn)(void* ctx, double step, double* misfit);
int fwi_psv_step_search(double est, double L2_0, fwi_psv_trial_fn trial, void* ctx, double* opt,
                        int* trials, int* status);

/* ---- independent models in one launch ------------------------------------
 * Many models of uneven grid size, fdorder and nt (one shot each) advanced
 * together: every pass of a time step is one launch per fdorder over the
 * tiles of all models still running (models sorted by nt, tiles model-major),
 * one binomial reversal plan over the longest nt serves every model, and the
 * whole gradient is replayed as CUDA graphs.  Each model is the reference's
 * per-shot call (forward_kernel_PSV_GPU + adjoint_kernel_PSV_GPU with the
 * reference gradient, fwi intervals 1, window = the padded grid from the free
 * surface down).  The thread mapping and tile height of each fdorder group are
 * chosen by timing the candidates on the group's own tiles (autotune != 0;
 * at the engine's first forward or gradient, so both run the same mappings and
 * compute the same traces), cached in a JSON file ($FWI_PSV_TUNE_CACHE,
 * default ~/.cache/cuda_fwi_gb300/autotune.json) keyed by GPU and group shape. */
typedef struct fwi_psv_model {
    fwi_psv_desc grid;                 /* as for fwi_psv_create */
    const double *lam, *mu, *rho;      /* [nzt][nxt] */
    int nsrc;                          /* vz sources (padded indices) */
    const int *src_x, *src_z;
    const double* src_signal;          /* [nsrc][nt] */
    int nrec;                          /* vz receivers (padded indices) */
    const int *rec_x, *rec_z;
} fwi_psv_model;
typedef struct fwi_psv_multi fwi_psv_multi;
int fwi_psv_multi_create(int nmodels, const fwi_psv_model* models, int device, fwi_psv_multi** out);
int fwi_psv_multi_destroy(fwi_psv_multi* m);
/* use_graphs (default 1); snapshots = checkpoint slots of the common plan
 * (default 32; 0 = as many as 80% of free memory holds); autotune (default 1). */
int fwi_psv_multi_set_exec(fwi_psv_multi* m, int use_graphs, int snapshots, int autotune);
/* Forward modelling of every model (forward_simulate, fd_wave_model.cu:133-230):
 * rec_out[k] [nrec_k][nt_k] receives model k's vz traces (NULL entries skipped). */
int fwi_psv_multi_forward(fwi_psv_multi* m, double* const* rec_out);
/* obs[k] [nrec_k][nt_k]; misfit[k]; grad_*[k] [nzt_k][nxt_k] (any may be NULL). */
int fwi_psv_multi_gradient(fwi_psv_multi* m, const double* const* obs, double* misfit,
                           double* const* grad_lam, double* const* grad_mu, double* const* grad_rho);
/* Choice for order group g (after the first gradient when autotuning):
 * info = {half order, models, forward mapping, forward tile rows, adjoint mapping,
 * adjoint tile rows, read from the cache (1) or timed now (0)}; ms = {forward pair,
 * adjoint stress} per launch over the whole group, as timed when the choice was made
 * (the cache keeps them).  Mappings: 0 z-march (tile rows), 1 scalar cells, 2 vectorised cells,
 * 3 TMA-staged tiles (tensor maps per model in device memory). */
int fwi_psv_multi_tuning(fwi_psv_multi* m, int group, int info[7], double ms[2]);
int fwi_psv_multi_get_stats(fwi_psv_multi* m, fwi_psv_stats* out);

/* ---- failure detection ---------------------------------------------------- */

/* No counterpart in the reference (whose CUDA errors exit the process,
 * forward_kernel_PSV_GPU.cu:19-27).  Every wait of the engine's kernels on
 * their own asynchronous copies is bounded; when one runs out the kernel sets
 * an error word, drains its copies (bounded) and returns, the later launches of
 * the call return at once, and the call returns FWI_ERR_CUDA with the engine
 * still usable.  fwi_psv_set_wait_limit sets that bound (default 2 s; 1e-6 to
 * 60 s).  A device watchdog scans the recorded traces every 64 steps and the
 * gradients at the end of a backward for NaN / Inf; the call then returns
 * FWI_ERR_DIVERGED (as a residual above 1e10 does). */
int fwi_psv_set_wait_limit(fwi_psv_engine* e, double seconds);
/* Test hook: the next forward's first TMA-staged step (the fused step, or the
 * stress pass of the two-pass step) makes one CTA expect more bytes than its
 * copies deliver, so its wait runs out and the forward returns FWI_ERR_CUDA
 * (FWI_ERR_UNSUPPORTED on the other mappings and with the exact adjoint). */
int fwi_psv_debug_stall_next(fwi_psv_engine* e);

/* ---- allocation-free misfit ---------------------------------------------- */

/* No counterpart in the reference (whose misfit, calculate_l2_adjoint_sources,
 * runs on the host).  For callers that cannot allocate device memory from the
 * code that evaluates the misfit: applications whose HBM is reserved up front
 * by their own pool allocator, and time-critical loops where cudaMalloc/cudaFree
 * would synchronise the device and stall other streams.  Given device-resident
 * FP32 traces d_syn and d_obs ([nrows][nt]) it writes d_resid = syn - obs
 * ([nrows][nt], FP32, difference taken in FP64) and *misfit = sum 0.5 dt diff^2
 * (FP64, summed in trace order) on `stream` (a cudaStream_t, NULL = legacy
 * default stream), then waits for the stream.  It allocates nothing: its
 * scratch is a fixed device array of FWI_NOALLOC_MAX_ROWS traces that every GPU
 * loading the library holds until exit; more traces return FWI_ERR_INVALID.
 * The first call on a device looks up the array's address with that device
 * current and keeps it for the life of the process (do not call
 * cudaDeviceReset between calls).  Every call copies the misfit to the host and
 * waits for its stream, so it cannot be called while that stream is being
 * captured.  An error already pending on entry is returned as FWI_ERR_CUDA and
 * left pending.  All calls share the array: calls that overlap on the GPU race.
 * Returns FWI_ERR_DIVERGED when |diff| > 1e10, as the engine does. */
#define FWI_NOALLOC_MAX_ROWS 65536
int fwi_psv_misfit_noalloc(const float* d_syn, const float* d_obs, int nrows, int nt, double dt,
                           float* d_resid, double* misfit, void* stream);

/* ---- reference-shaped calls --------------------------------------------- */

/* forward_kernel_PSV (fd_kernel.cuh:12-43) with flat FP64 host arrays in the
 * reference layouts: resets the state, runs nt steps on the device and writes
 * back the final wavefield, We, the CPML memory, rec_signal rows of `ishot`
 * and, when fwinv, the FWI storage (fwi_vx .. fwi_szz, [nft][nfz][nfx]). */
int fwi_psv_forward_kernel(int ishot, int nt, int nzt, int nxt, int fpad, int ppad, double dt,
                           double dx, double dz, int snap_interval, int fsurf, const double* hc,
                           int fdorder, double* vx, double* vz, double* sxx, double* szx,
                           double* szz, double* We, const double* lam, const double* mu,
                           const double* mu_zx, const double* rho_zp, const double* rho_xp,
                           int npml, const double* a, const double* b, const double* K,
                           const double* a_half, const double* b_half, const double* K_half,
                           double* mem_vx_x, double* mem_vx_z, double* mem_vz_x,
                           double* mem_vz_z, double* mem_sxx_x, double* mem_szx_x,
                           double* mem_szz_z, double* mem_szx_z, int nsrc, const int* src_x,
                           const int* src_z, const int* src_comp, const double* src_signal,
                           const int* source_to_fire_shot, int nrec, const int* rec_x,
                           const int* rec_z, const int* rec_comp, double* rec_signal,
                           const int* receiver_to_record_shot, int fwinv, int fwi_dt,
                           int fwi_dx, int fwi_dz, int fwi_x1, int fwi_x2, int fwi_z1,
                           int fwi_z2, double* fwi_vx, double* fwi_vz, double* fwi_sxx,
                           double* fwi_szx, double* fwi_szz);

/* adjoint_kernel_PSV (fd_kernel.cuh:46-70): reverse-time pass injecting
 * src_signal (the residual) at the src positions, gradient from the FWI
 * storage written by fwi_psv_forward_kernel.  Writes grad_lam/mu/rho, the
 * final adjoint wavefield, We and the CPML memory. */
int fwi_psv_adjoint_kernel(int ishot, int nt, int nzt, int nxt, int fpad, int ppad, double dt,
                           double dx, double dz, int snap_interval, int fsurf, const double* hc,
                           int fdorder, double* vx, double* vz, double* sxx, double* szx,
                           double* szz, double* We, const double* lam, const double* mu,
                           const double* mu_zx, const double* rho_zp, const double* rho_xp,
                           int npml, const double* a, const double* b, const double* K,
                           const double* a_half, const double* b_half, const double* K_half,
                           double* mem_vx_x, double* mem_vx_z, double* mem_vz_x,
                           double* mem_vz_z, double* mem_sxx_x, double* mem_szx_x,
                           double* mem_szz_z, double* mem_szx_z, int nsrc, const int* src_x,
                           const int* src_z, const int* src_comp, const double* src_signal,
                           const int* source_to_fire_shot, int fwinv, int fwi_dt, int fwi_dx,
                           int fwi_dz, int fwi_x1, int fwi_x2, int fwi_z1, int fwi_z2,
                           const double* fwi_vx, const double* fwi_vz, const double* fwi_sxx,
                           const double* fwi_szx, const double* fwi_szz, double* grad_lam,
                           double* grad_mu, double* grad_rho);

#ifdef __cplusplus
}
#endif
#endif /* FWI_PSV_H */
